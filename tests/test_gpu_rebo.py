"""rebosc on the GPU: analytic forces against the oracle's numerical ones (the
reference's central differences, dx = 1e-6 A, whose own error is ~1e-7 eV/A),
energies against the oracle, trajectories, energy conservation, the precision
form, and rebosc as the carbon interaction that gives morsec its graphene
neighbours."""
import numpy as np
import pytest

import pfmds_gb300 as pf
from pfmds_gb300 import configs
from oracle.pyoracle import Oracle

pytestmark = pytest.mark.gpu


def _sheet(d, **kw):
    configs.graphene_rebo(str(d), nx=8, ny=5, seed=3, **kw)
    return str(d)


def test_step0_forces_and_energy(tmp_path, built):
    d = _sheet(tmp_path)
    o = Oracle(d, out_period=1, threads=1)
    o.step()
    s = pf.Simulation(d, form="plain", out_period=1)
    s.advance(1)
    _, _, fo = o.state()
    _, _, f = s.state()
    assert np.abs(f - fo).max() < 2e-6, np.abs(f - fo).max()
    assert np.abs(f.sum(0)).max() < 1e-9  # analytic: Newton's third law to round-off
    eo, eg = o.energies(), s.energies()
    np.testing.assert_allclose(eg["inter"], eo["inter"], rtol=1e-12)


def test_trajectory_follows_the_oracle(tmp_path, built):
    d = _sheet(tmp_path)
    o = Oracle(d, out_period=10 ** 6, threads=1)
    o.run(30)
    s = pf.Simulation(d, form="plain", out_period=10 ** 6)
    s.advance(30)
    po, vo, _ = o.state()
    p, v, _ = s.state()
    assert np.abs(p - po).max() < 1e-7
    assert np.abs(v - vo).max() < 1e-8
    assert s.energies()["conserved"] == pytest.approx(o.energies()["conserved"], rel=1e-8)


def test_nve_conserves_energy_and_repeats(tmp_path, built):
    # a gently displaced sheet stays near 300 K; the 0.15 A default heats to ~2,800 K,
    # where dt = 0.5 fs itself drifts by ~2e-3 eV/atom/ps
    d = _sheet(tmp_path, steps=2000, log_period=100, corrugation=0.03)
    runs = []
    for _ in range(2):
        s = pf.Simulation(d, form="plain", out_period=10 ** 6)
        s.advance(1)
        e0 = s.energies()["conserved"]
        s.advance(2000)
        runs.append((s.energies()["conserved"], s.state()))
        n = s.natoms
    assert abs(runs[0][0] - e0) / n < 5e-5  # eV per atom over 1 ps at dt 0.5 fs
    for x, y in zip(runs[0][1], runs[1][1]):
        assert np.array_equal(x, y)


def test_precision_form_uses_the_same_fp64_kernels(tmp_path, built):
    d = _sheet(tmp_path)
    a = pf.Simulation(d, form="plain", out_period=1)
    b = pf.Simulation(d, form="precision", out_period=1)
    a.advance(1)
    b.advance(1)
    fa, fb = a.state()[2], b.state()[2]
    assert np.abs(fa - fb).max() / np.abs(fa).max() < 1e-12
    assert b.energies()["inter"][0] == pytest.approx(a.energies()["inter"][0], rel=1e-13)


def test_rebosc_gives_morsec_its_graphene_neighbours(tmp_path, built):
    configs.gr_on_cu(str(tmp_path), carbon="rebosc", steps=20)
    d = str(tmp_path)
    o = Oracle(d, out_period=1, threads=1)
    o.step()
    s = pf.Simulation(d, form="plain", out_period=1)
    s.advance(1)
    _, _, fo = o.state()
    _, _, f = s.state()
    assert np.abs(f - fo).max() < 2e-6
    np.testing.assert_allclose(s.energies()["inter"], o.energies()["inter"], rtol=1e-10, atol=1e-10)
