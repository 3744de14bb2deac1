"""Batched form: replicas of a settings list stepped together by one persistent
kernel, checked replica by replica against the single-system library on the same
settings files."""
import numpy as np
import pytest

import pfmds_gb300 as pf
from pfmds_gb300 import configs

pytestmark = pytest.mark.gpu


def _batch(d, n_rep=6, steps=200, seed=11, **kw):
    return configs.batch_systems(str(d), n_rep=n_rep, n_min=500, n_max=2500, steps=steps, log_period=10,
                                 seed=seed, **kw)


def test_step0_forces_and_energies_match_single_system(tmp_path, built):
    ln, reps = _batch(tmp_path)
    assert {r["kind"] for r in reps} == {"lj", "rjl"}
    b = pf.Batch(str(tmp_path), ln)
    assert b.info()[0] == len(reps)
    b.run(1)
    ep, ek = b.energies()
    for r, rep in enumerate(reps):
        s = pf.Simulation(str(tmp_path), settings=rep["settings"], form="plain", out_period=10 ** 9)
        s.advance(1)
        p_ref, v_ref, f_ref = s.state()
        e = s.energies()
        p, v, f = b.state(r)
        assert np.array_equal(p, p_ref)
        assert np.abs(v - v_ref).max() < 1e-15  # zero_momentum: the same sums in another order
        rmse = np.sqrt(((f - f_ref) ** 2).mean()) / np.sqrt((f_ref ** 2).mean())
        assert rmse < 1e-5, (rep, rmse)
        assert ep[r] == pytest.approx(e["pe"], rel=2e-6, abs=1e-6 * rep["n"]), rep
        assert ek[r] == pytest.approx(e["ke"], rel=1e-12), rep
        s.close()


def test_trajectory_follows_single_system_precision_form(tmp_path, built):
    ln, reps = _batch(tmp_path, n_rep=4, seed=5)
    b = pf.Batch(str(tmp_path), ln)
    b.run(31)  # three list rebuilds; the energies of step 30, the launch's last
    ep, ek = b.energies()
    b.run(4)
    for r, rep in enumerate(reps):
        s = pf.Simulation(str(tmp_path), settings=rep["settings"], form="precision", out_period=10 ** 9)
        s.advance(31)  # steps 0..30: the energies of step 30
        e = s.energies()
        assert ep[r] == pytest.approx(e["pe"], rel=1e-5, abs=1e-5 * rep["n"]), rep
        assert ek[r] == pytest.approx(e["ke"], rel=1e-5), rep
        s.advance(4)
        p_ref, v_ref, _ = s.state()
        p, v, _ = b.state(r)
        d = np.abs(p - p_ref)
        box = np.abs(p_ref).max()
        assert np.minimum(d, box - d).max() < 1e-6, rep
        assert np.abs(v - v_ref).max() < 1e-6, rep
        s.close()


def test_energy_history_conserves(tmp_path, built):
    ln, reps = _batch(tmp_path, n_rep=6, steps=300, seed=3)
    b = pf.Batch(str(tmp_path), ln)
    b.run(150)
    b.run(150)  # the same run length: the captured graph replays
    assert b.graphs() >= 1
    h, per = b.history()
    assert per == 10 and h.shape == (30, len(reps), 2)
    tot = h[:, :, 0] + h[:, :, 1]
    n = np.array([r["n"] for r in reps])
    drift = np.abs(tot[-1] - tot[0]) / n
    assert (drift < 2e-4).all(), drift  # eV/atom over 150-300 fs


def test_autotuner_restores_state(tmp_path, built):
    ln, reps = _batch(tmp_path, n_rep=4, seed=9)
    b = pf.Batch(str(tmp_path), ln)
    b.run(20)
    before = [b.state(r) for r in range(len(reps))]
    tpa = b.tune(steps=10)
    assert all(t in (1, 2, 4, 8) for t in tpa)
    after = [b.state(r) for r in range(len(reps))]
    for x, y in zip(before, after):
        for u, w in zip(x, y):
            assert np.array_equal(u, w)
    assert b.info()[2] == 20
    b.run(10)
    # the tuned batch keeps following the reference physics: compare with a batch
    # run straight through with the same tile choices
    c = pf.Batch(str(tmp_path), ln)
    c.set_tpa(tpa)
    c.run(30)
    for r in range(len(reps)):
        pb, vb, _ = b.state(r)
        pc, vc, _ = c.state(r)
        assert np.abs(pb - pc).max() < 1e-6 and np.abs(vb - vc).max() < 1e-6


def test_list_overflow_names_the_replica(tmp_path, built):
    ln, reps = _batch(tmp_path, n_rep=3, seed=2)
    k = next(i for i, r in enumerate(reps) if r["kind"] == "rjl")
    sf = tmp_path / reps[k]["settings"]
    sf.write_text(sf.read_text().replace("\t96\t", "\t20\t"))
    b = pf.Batch(str(tmp_path), ln)
    with pytest.raises(pf.PfmdError) as ei:
        b.run(1)
    assert ei.value.code == pf.PFMD_E_NLIST_OVERFLOW
    assert reps[k]["settings"] in str(ei.value)


def test_unsupported_replica_is_rejected(tmp_path, built):
    ln, reps = _batch(tmp_path, n_rep=2, seed=4)
    sf = tmp_path / reps[0]["settings"]
    sf.write_text(sf.read_text().replace(" nve ", " nvms "))
    assert not pf.batch_accepts(str(tmp_path), reps[0]["settings"])[0]
    with pytest.raises(pf.PfmdError) as ei:
        pf.Batch(str(tmp_path), ln)
    assert ei.value.code == pf.PFMD_E_PARAM and "nve or nvt" in str(ei.value)


def _fields(line):
    return [float(x) for x in line.split()[1:]]


def _xyz_rows(path):
    lines = open(path).read().splitlines()
    n = int(lines[0])
    rows = [ln.split() for ln in lines[2:2 + n]]
    return np.array([[float(x) for x in r[:-1]] for r in rows]), [r[-1] for r in rows]


@pytest.mark.parametrize("out_period", [1, 10 ** 6])
def test_list_run_writes_what_single_runs_write(tmp_path, built, out_period):
    """run_md_simulation -ilist ... -batch against the same list run entry by entry
    (precision form): the same files, steps and times; energies and positions
    within the FP32-pair tolerance after 65 steps."""
    ln, reps = _batch(tmp_path, n_rep=4, steps=65, seed=4)
    assert {r["kind"] for r in reps} == {"lj", "rjl"}
    for r in reps:  # snapshots every 30 steps, trajectory frames every 20
        sf = tmp_path / r["settings"]
        txt = sf.read_text().replace("period_traj:\t\t\t\t100000000", "period_traj:\t\t\t\t20")
        sf.write_text(txt.replace("100000000", "30"))
    ob, os_ = tmp_path / "batch", tmp_path / "single"
    ob.mkdir()
    os_.mkdir()
    common = ["-ipath", f"{tmp_path}/", "-ilist", ln, "-op", str(out_period)]
    assert pf.run_md_simulation(common + ["-opath", f"{ob}/", "-batch"]) == 0
    assert pf.run_md_simulation(common + ["-opath", f"{os_}/", "-form", "precision"]) == 0
    names = sorted(p.name for p in os_.iterdir())
    assert names == sorted(p.name for p in ob.iterdir())
    for r in reps:
        pre = r["name"] + "_"
        assert {pre + "md_run.log", pre + "final_" + r["name"] + ".xyz", pre + "snapshot_000030.xyz",
                pre + "snapshot_000060.xyz"} <= set(names)
        lb = (ob / (pre + "md_run.log")).read_text().splitlines()
        ls = (os_ / (pre + "md_run.log")).read_text().splitlines()
        assert len(lb) == len(ls) == 8  # steps 0..60 by 10, then the closing record
        for x, y in zip(lb, ls):
            if x is not lb[-1]:
                assert x.split()[0] == y.split()[0] == "nve"
            fx, fy = _fields(x), _fields(y)
            assert len(fx) == len(fy)
            assert fx[:2] == fy[:2]  # step, time
            assert np.allclose(fx[2:], fy[2:], rtol=2e-5, atol=1e-5 * r["n"]), (r, x, y)
        for f in (pre + "final_" + r["name"] + ".xyz", pre + "snapshot_000060.xyz"):
            pb, tb = _xyz_rows(ob / f)
            ps, ts = _xyz_rows(os_ / f)
            assert tb == ts
            assert np.abs(pb - ps).max() < 1e-3, (r, f)  # printed to 4 decimals
        for f in [n for n in names if n.startswith(pre + "traj_")]:
            assert (ob / f).read_text().count("time_step") == (os_ / f).read_text().count("time_step") == 4
    ab = (ob / "all_out.txt").read_text().split("\n")
    as_ = (os_ / "all_out.txt").read_text().split("\n")
    ab, as_ = [x for x in ab if x.strip()], [x for x in as_ if x.strip()]
    assert len(ab) == len(as_) == len(reps)
    for x, y, r in zip(ab, as_, reps):
        fx, fy = _fields(x), _fields(y)
        assert fx[:2] == fy[:2] and fx[0] == 65
        assert np.allclose(fx[2:], fy[2:], rtol=2e-5, atol=1e-5 * r["n"]), (r, x, y)


def test_list_run_needs_equal_lengths(tmp_path, built):
    ln, reps = _batch(tmp_path, n_rep=2, steps=40, seed=4)
    sf = tmp_path / reps[1]["settings"]
    sf.write_text(sf.read_text().replace("md_step_limit:\t\t\t\t40", "md_step_limit:\t\t\t\t30"))
    b = pf.Batch(str(tmp_path), ln)
    with pytest.raises(pf.PfmdError) as ei:
        b.run_list(str(tmp_path) + "/")
    assert ei.value.code == pf.PFMD_E_PARAM and reps[1]["settings"] in str(ei.value)
