"""GPU parity against the oracle on the benchmark configurations and on the
step-loop paths the other parity systems leave out.

* The 4,000-atom binary LJ gas through its integrator schedule: 1,000 nvt
  steps, 1,000 nve steps, then nvms until |PE - PE_prev| <= ms_de
  (md_simulation.f90:121-147).  md() compares the potential energies of
  consecutive steps once nvms computes them every step; the first comparison
  (step 2001 against step 2000, 1.9e-4 eV on this gas) is the smallest until
  far into the descent (the per-step change rises to 0.06 eV and is still
  7e-5 eV after the stage's 100,000 steps, so the specified ms_de = 1e-8 ends
  the stage by its length).  With ms_de = 1e-2 both must leave at step 2002.
  Lists are compared at every rebuild, forces and positions after every list
  period.
* The 65,536-atom Cu slab: lists bit-exact and forces within 1e-9 at step 0
  and after three rebuilds.
* A slab with a z-only layer (integrate_verlet_z_*, molecular_static_1D), atoms
  joining the xyz-moving group through change_particle_group_N, and
  invert_z_velocities (md_general.f90:82-95,382-396; md_integrators.f90:33,79,125),
  in both forms; and the same group growth driven through pfmd_set_group_n.
"""
import os

import numpy as np
import pytest

import pfmds_gb300 as pf
from pfmds_gb300 import configs
from oracle.pyoracle import Oracle

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


def _lists_equal(s, o):
    """Every list of every interaction: row lengths, entries in order, lessnnum."""
    for i in range(o.n_interactions):
        for j in range(3):
            try:
                ol = o.nlist(i, j)
            except Exception:
                break
            gl = s.nlist(i, j)
            assert np.array_equal(gl["nnum"], ol["nnum"]), (i, j)
            m = ol["nlist"].shape[1]
            mask = np.arange(m)[None, :] < ol["nnum"][:, None]
            assert np.array_equal(np.where(mask, gl["nlist"][:, :m], -1), np.where(mask, ol["nlist"], -1)), (i, j)
            if j == 0:
                assert np.array_equal(gl["lessnnum"], ol["lessnnum"]), (i, j)


def _max_dev(s, o):
    po, vo, fo = o.state()
    p, v, f = s.state()
    return (float(np.abs(p - po).max()), float(np.abs(v - vo).max()),
            float(np.abs(f - fo).max() / np.abs(fo).max()))


def test_lj_gas_4000_full_schedule(tmp_path, built):
    d = str(tmp_path)
    configs.lj_gas(d, log_period=100, ms_de=1e-2)
    o = Oracle(d, out_period=10 ** 9, threads=THREADS)
    s = pf.Simulation(d, form="plain", out_period=10 ** 9)
    o.step()
    s.advance(1)
    _lists_equal(s, o)
    dp, dv, df = _max_dev(s, o)
    assert df < 1e-9
    worst = [0.0, 0.0, 0.0]
    stage_energy = {}
    while True:
        fo = o.run(10)
        fg = s.advance(10)
        assert fo == fg and s.md_step == o.md_step, (s.md_step, o.md_step)
        if fo:
            break
        _lists_equal(s, o)
        dev = _max_dev(s, o)
        worst = [max(a, b) for a, b in zip(worst, dev)]
        # FP64 round-off differences (CUDA's cos and exp against glibc's) grow
        # along the trajectory; after 2,000+ steps they stay far below these
        assert dev[0] < 1e-7 and dev[1] < 1e-8 and dev[2] < 1e-6, (s.md_step, dev)
        if s.md_step in (1001, 2001):
            eo, eg = o.energies(), s.energies()
            assert eg["conserved"] == pytest.approx(eo["conserved"], rel=1e-9, abs=1e-9)
            stage_energy[s.md_step] = eg["conserved"]
    # md() leaves the nvms stage at the same step in both (the steps number of
    # md_simulation.f90:247 is md_step - 1): the second nvms step
    assert s.md_step == o.md_step == 2002
    eo, eg = o.energies(), s.energies()
    assert eg["pe"] == pytest.approx(eo["pe"], rel=1e-9, abs=1e-9)
    print("config-1 schedule: nvms exit at step", s.md_step, "max deviations (pos A, vel A/fs, force rel):", worst)


def test_lj_gas_4000_specified_schedule_into_nvms(tmp_path, built):
    """The schedule as specified (ms_de = 1e-8) through both switches and the
    first 300 nvms steps: energies at every log step, lists at every rebuild.
    Further into the descent the two paths part: nvms zeroes an atom's
    velocity when F.v <= 0 (md_integrators.f90:99-123), a discontinuous choice
    that round-off differences between the two machines' cos and exp flip, and
    the descents then follow different but equivalent paths."""
    d = str(tmp_path)
    configs.lj_gas(d, log_period=100)
    o = Oracle(d, out_period=10 ** 9, threads=THREADS)
    s = pf.Simulation(d, form="plain", out_period=10 ** 9)
    o.step()
    s.advance(1)
    worst = {"md": [0.0, 0.0, 0.0], "nvms": [0.0, 0.0, 0.0]}
    while s.md_step < 2301:
        assert not o.run(10) and not s.advance(10)
        _lists_equal(s, o)
        dev = _max_dev(s, o)
        stage = "md" if s.md_step <= 2001 else "nvms"
        worst[stage] = [max(a, b) for a, b in zip(worst[stage], dev)]
        if stage == "md":
            assert dev[0] < 1e-7 and dev[2] < 1e-6, (s.md_step, dev)
        else:  # 300 descent steps: deviations grow but stay small
            assert dev[0] < 1e-5 and dev[2] < 1e-4, (s.md_step, dev)
        if (s.md_step - 1) % 100 == 0:
            eo, eg = o.energies(), s.energies()
            for k in ("pe", "ke", "conserved"):
                assert eg[k] == pytest.approx(eo[k], rel=1e-8, abs=1e-7), (s.md_step, k)
    print("config-1 into nvms: max deviations (pos A, vel A/fs, force rel):", worst)


def test_cu_slab_65536_lists_and_forces(tmp_path, built):
    d = str(tmp_path)
    configs.cu_slab(d, steps=100, log_period=10)
    o = Oracle(d, out_period=10 ** 9, threads=THREADS)
    s = pf.Simulation(d, form="plain", out_period=10 ** 9)
    o.step()
    s.advance(1)
    assert s.natoms == 65536
    _lists_equal(s, o)
    assert _max_dev(s, o)[2] < 1e-9
    np.testing.assert_allclose(s.energies()["inter"], o.energies()["inter"], rtol=1e-11)
    for _ in range(3):  # through the rebuilds at steps 10, 20 and 30
        o.run(10)
        s.advance(10)
        _lists_equal(s, o)
        dp, dv, df = _max_dev(s, o)
        assert df < 1e-9 and dp < 1e-9 and dv < 1e-10, (s.md_step, dp, dv, df)
    eo, eg = o.energies(), s.energies()
    assert eg["conserved"] == pytest.approx(eo["conserved"], rel=1e-11)


def test_z_layer_group_growth_and_inversion_plain(tmp_path, built):
    d = str(tmp_path)
    configs.cu_deposit(d)
    o = Oracle(d, out_period=10 ** 9, threads=THREADS)
    s = pf.Simulation(d, form="plain", out_period=10 ** 9)
    p0 = s.state()[0]
    o.step()
    s.advance(1)
    _lists_equal(s, o)
    assert _max_dev(s, o)[2] < 1e-9
    for _ in range(12):
        o.run(5)
        s.advance(5)
        _lists_equal(s, o)
        dp, dv, df = _max_dev(s, o)
        assert dp < 1e-9 and dv < 1e-10 and df < 1e-8, (s.md_step, dp, dv, df)
        eo, eg = o.energies(), s.energies()
        assert eg["conserved"] == pytest.approx(eo["conserved"], rel=1e-10, abs=1e-10)
        assert eg["temperature"] == pytest.approx(eo["temperature"], rel=1e-10)
    p, v, _ = s.state()
    types = [ln.split()[-1] for ln in open(os.path.join(d, "cu_dep.xyz")).read().split("\n")[2:] if ln.strip()]
    zl = np.array([t == "CU_z" for t in types])
    dep = np.array([t == "CU_dep" for t in types])
    assert np.array_equal(p[zl, :2], p0[zl, :2]) and np.abs(p[zl, 2] - p0[zl, 2]).max() > 1e-4
    assert np.abs(p[dep] - p0[dep]).max() > 1e-2  # the joined atoms moved


def test_z_layer_group_growth_and_inversion_precision(tmp_path, built):
    d = str(tmp_path)
    configs.cu_deposit(d)
    o = Oracle(d, out_period=10 ** 9, threads=THREADS)
    s = pf.Simulation(d, form="precision", out_period=10 ** 9)
    o.step()
    s.advance(1)
    po, vo, fo = o.state()
    p, v, f = s.state()
    assert np.sqrt(((f - fo) ** 2).mean()) / np.sqrt((fo ** 2).mean()) < 1e-5
    o.run(60)
    s.advance(60)
    po, vo, fo = o.state()
    p, v, f = s.state()
    assert s.md_step == o.md_step
    assert np.abs(p - po).max() < 1e-4
    assert np.sqrt(((f - fo) ** 2).mean()) / np.sqrt((fo ** 2).mean()) < 1e-3
    assert s.energies()["conserved"] == pytest.approx(o.energies()["conserved"], rel=1e-6)


def test_set_group_n_matches_settings_schedule(tmp_path, built):
    """pfmd_set_group_n between steps reproduces change_particle_group_N's
    schedule: group 4 starts with group 2's size and gains one atom at step 3
    and every 5 steps after it (ts1 = 3, ts2 = 30, frec = 5)."""
    da, db = str(tmp_path / "a"), str(tmp_path / "b")
    configs.cu_deposit(da)
    configs.cu_deposit(db, change=None)
    o = Oracle(da, out_period=10 ** 9, threads=THREADS)
    s = pf.Simulation(db, form="plain", out_period=10 ** 9)
    types = [ln.split()[-1] for ln in open(os.path.join(db, "cu_dep.xyz")).read().split("\n")[2:] if ln.strip()]
    n2 = sum(t == "CU" for t in types)
    s.set_group_n(4, n2)
    for step in range(61):
        if step >= 3 and step < 30 and (step - 3) % 5 == 0:
            s.set_group_n(4, n2 + 1 + (step - 3) // 5)
        o.step()
        s.advance(1)
    _lists_equal(s, o)
    dp, dv, df = _max_dev(s, o)
    assert dp < 1e-9 and dv < 1e-10 and df < 1e-8, (dp, dv, df)
