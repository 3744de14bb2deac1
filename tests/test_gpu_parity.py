"""GPU parity: the CUDA library against the CPU oracle on the same inputs.

Plain form: neighbour lists identical to the oracle's (bit-exact membership and
order), forces within 1e-9 relative (the target is 1e-5), trajectories and
energies within FP64 round-off growth.  Precision form: force RMSE relative to
the force scale below 1e-5.
"""
import numpy as np
import pytest

import pfmds_gb300 as pf
from pfmds_gb300 import configs
from oracle.pyoracle import Oracle

pytestmark = pytest.mark.gpu


def _lj(d, **kw):
    kw.setdefault("integrators", [("nvt", 0.5, 30, 10 ** 8, 10), ("nve", 0.5, 30, 10 ** 8, 10)])
    configs.lj_gas(str(d), n_a=250, n_b=250, box=30.0, **kw)
    return str(d)


def _cu(d, **kw):
    configs.cu_slab(str(d), nx=6, ny=6, nz=4, steps=60, log_period=10, **kw)
    return str(d)


def _gr(d, **kw):
    kw.setdefault("steps", 40)
    configs.gr_on_cu(str(d), **kw)
    return str(d)


SYSTEMS = {"lj": _lj, "cu": _cu, "gr_morsec": _gr,
           "gr_ljc": lambda d: _gr(d, coupling="ljc"),
           "gr_simplified": lambda d: _gr(d, simplified=True),
           # a cosine power other than 2 (pow instead of the product form)
           "gr_morsec_delta1.5": lambda d: _gr(d, morse=(0.1, 2.2, 1.7, 1.5)),
           "gr_ljc_delta1.5": lambda d: _gr(d, coupling="ljc", ljc=(0.0168, 2.2, 1.5))}


def _compare_lists(s, o):
    for i in range(o.n_interactions):
        for j in range(3):
            try:
                ol = o.nlist(i, j)
            except Exception:
                break
            gl = s.nlist(i, j)
            assert np.array_equal(gl["nnum"], ol["nnum"]), (i, j)
            for r in range(len(ol["nnum"])):
                n = ol["nnum"][r]
                assert np.array_equal(gl["nlist"][r, :n], ol["nlist"][r, :n]), (i, j, r)
            if j == 0:
                assert np.array_equal(gl["lessnnum"], ol["lessnnum"]), (i, j)


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_step0_lists_forces_energies(tmp_path, built, name):
    d = SYSTEMS[name](tmp_path)
    o = Oracle(d, out_period=1, threads=1)
    o.step()
    s = pf.Simulation(d, form="plain", out_period=1)
    s.advance(1)
    _compare_lists(s, o)
    po, vo, fo = o.state()
    p, v, f = s.state()
    scale = np.abs(fo).max()
    assert np.abs(f - fo).max() / scale < 1e-9
    eo, eg = o.energies(), s.energies()
    np.testing.assert_allclose(eg["inter"], eo["inter"], rtol=1e-10, atol=1e-10)
    assert eg["temperature"] == pytest.approx(eo["temperature"], rel=1e-12)


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_trajectory_plain(tmp_path, built, name):
    d = SYSTEMS[name](tmp_path)
    o = Oracle(d, out_period=10 ** 6, threads=1)
    o.run(25)
    s = pf.Simulation(d, form="plain", out_period=10 ** 6)
    s.advance(25)
    assert s.md_step == o.md_step
    _compare_lists(s, o)
    po, vo, fo = o.state()
    p, v, f = s.state()
    assert np.abs(p - po).max() < 1e-8
    assert np.abs(v - vo).max() < 1e-9
    assert np.abs(f - fo).max() / np.abs(fo).max() < 1e-7
    eo, eg = o.energies(), s.energies()
    np.testing.assert_allclose(eg["inter"], eo["inter"], rtol=1e-8, atol=1e-8)
    assert eg["conserved"] == pytest.approx(eo["conserved"], rel=1e-9, abs=1e-9)


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_precision_form_forces(tmp_path, built, name):
    d = SYSTEMS[name](tmp_path)
    o = Oracle(d, out_period=1, threads=1)
    o.step()
    s = pf.Simulation(d, form="precision", out_period=1)
    s.advance(1)
    po, vo, fo = o.state()
    p, v, f = s.state()
    rmse = np.sqrt(((f - fo) ** 2).mean())
    scale = np.sqrt((fo ** 2).mean())
    assert rmse / scale < 1e-5, rmse / scale
    eo, eg = o.energies(), s.energies()
    np.testing.assert_allclose(eg["inter"], eo["inter"], rtol=1e-5, atol=1e-5)


def test_graphs_match_direct_launches(tmp_path, built):
    d = _cu(tmp_path)
    a = pf.Simulation(d, form="plain", out_period=10 ** 6, use_graphs=True)
    b = pf.Simulation(d, form="plain", out_period=10 ** 6, use_graphs=False)
    for _ in range(4):
        a.advance(10)
        b.advance(10)
    pa, va, fa = a.state()
    pb, vb, fb = b.state()
    assert np.array_equal(pa, pb) and np.array_equal(va, vb) and np.array_equal(fa, fb)


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_precision_lists_match_oracle(tmp_path, built, name):
    """Precision-form rows are in cell-scan order and tested on fixed-point
    separations: as sets they equal the reference's rows (the inputs put no pair
    within the fixed-point resolution of a cut-off)."""
    d = SYSTEMS[name](tmp_path)
    o = Oracle(d, out_period=1, threads=1)
    o.step()
    s = pf.Simulation(d, form="precision", out_period=1)
    s.advance(1)
    for i in range(o.n_interactions):
        for j in range(3):
            try:
                ol = o.nlist(i, j)
            except Exception:
                break
            gl = s.nlist(i, j)
            assert np.array_equal(gl["nnum"], ol["nnum"]), (i, j)
            for r in range(len(ol["nnum"])):
                n = ol["nnum"][r]
                assert np.array_equal(np.sort(gl["nlist"][r, :n]), np.sort(ol["nlist"][r, :n])), (i, j, r)
            if j == 0:
                assert np.array_equal(gl["lessnnum"], ol["lessnnum"]), (i, j)


@pytest.mark.parametrize("name", ["cu", "gr_morsec"])
def test_precision_runs_repeat_bitwise(tmp_path, built, name):
    d = SYSTEMS[name](tmp_path)
    runs = []
    for graphs in (True, False):
        s = pf.Simulation(d, form="precision", out_period=10 ** 6, use_graphs=graphs)
        s.advance(30)
        runs.append(s.state() + (s.energies()["conserved"],))
        s.close()
    for a, b in zip(runs[0][:3], runs[1][:3]):
        assert np.array_equal(a, b)
    assert runs[0][3] == runs[1][3]
