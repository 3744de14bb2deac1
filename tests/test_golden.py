"""Golden fixtures (tests/golden/<case>/, made by make_golden.py from the CPU
oracle): the oracle still reproduces them, and the CUDA plain form matches them
-- lists bit for bit, forces within 1e-9 of the force scale, the 20-step state and
the log file the run writes."""
import os
import shutil

import numpy as np
import pytest

import pfmds_gb300 as pf
from oracle.pyoracle import Oracle

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
CASES = sorted(d for d in os.listdir(GOLDEN) if os.path.isdir(os.path.join(GOLDEN, d)))
STEPS = 20


def _copy(case, tmp_path):
    d = tmp_path / case
    shutil.copytree(os.path.join(GOLDEN, case), d, ignore=shutil.ignore_patterns("oracle.npz", "md_run.log"))
    return d


def _lists(sim, g):
    keys = sorted({k.rsplit("_", 1)[0] for k in g.files if k.startswith("nl_")})
    for key in keys:
        _, i, j = key.split("_")
        nl = sim.nlist(int(i), int(j))
        assert np.array_equal(nl["nnum"], g[key + "_nnum"]), key
        ent = np.concatenate([nl["nlist"][r, :n] for r, n in enumerate(nl["nnum"])] or [np.zeros(0, np.int32)])
        assert np.array_equal(ent, g[key + "_entries"]), key
        if j == "0":
            assert np.array_equal(nl["lessnnum"], g[key + "_less"]), key


def _log_rows(path):
    """(integrator name, step, values) of every log record; the closing record
    (md_simulation.f90:245-272) has no name."""
    rows = []
    for ln in open(path):
        f = ln.split()
        if not f:
            continue
        if f[0][0].isalpha():
            rows.append((f[0], int(f[1]), np.array([float(x) for x in f[2:]])))
        else:
            rows.append(("", int(f[0]), np.array([float(x) for x in f[1:]])))
    return rows


def test_cases_present():
    assert set(CASES) == {"cu_slab", "gr_ljc_simplified", "gr_morsec", "lj_gas"}


@pytest.mark.parametrize("case", CASES)
def test_oracle_reproduces_golden(tmp_path, built, case):
    g = np.load(os.path.join(GOLDEN, case, "oracle.npz"))
    d = _copy(case, tmp_path)
    o = Oracle(str(d), out_period=10 ** 6, threads=1)
    o.step()
    _lists(o, g)
    p, v, f = o.state()
    np.testing.assert_allclose(f, g["f0"], rtol=0, atol=1e-12 * np.abs(g["f0"]).max())
    o.run(STEPS)
    p, v, f = o.state()
    np.testing.assert_allclose(p, g["pos"], rtol=0, atol=1e-10)
    np.testing.assert_allclose(v, g["vel"], rtol=0, atol=1e-12)
    assert o.md_step == int(g["md_step"])


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_plain_form_matches_golden(tmp_path, built, case, monkeypatch):
    g = np.load(os.path.join(GOLDEN, case, "oracle.npz"))
    d = _copy(case, tmp_path)
    monkeypatch.chdir(d)  # outputs land beside the inputs, as when the fixtures were made
    s = pf.Simulation("", form="plain", out_period=10 ** 6, write_files=True, prefix="")
    s.advance(1)
    _lists(s, g)
    _, _, f = s.state()
    assert np.abs(f - g["f0"]).max() <= 1e-9 * np.abs(g["f0"]).max()
    np.testing.assert_allclose(s.energies()["inter"], g["e0_inter"], rtol=1e-10, atol=1e-10)
    s.advance(STEPS)
    s.finish()
    p, v, f = s.state()
    assert s.md_step == int(g["md_step"])
    assert np.abs(p - g["pos"]).max() < 1e-8
    assert np.abs(v - g["vel"]).max() < 1e-9
    e = s.energies()
    np.testing.assert_allclose(e["inter"], g["e_inter"], rtol=1e-8, atol=1e-8)
    assert e["conserved"] == pytest.approx(float(g["e_cons"]), rel=1e-9, abs=1e-9)
    s.close()
    mine, ref = _log_rows(d / "md_run.log"), _log_rows(os.path.join(GOLDEN, case, "md_run.log"))
    assert [(a, b) for a, b, _ in mine] == [(a, b) for a, b, _ in ref]
    for (_, step, x), (_, _, y) in zip(mine, ref):
        np.testing.assert_allclose(x, y, rtol=0, atol=2e-6, err_msg=f"log row at step {step}")
