"""Batched form against the oracle (run_md_simulation_mpi.f90:68-88 runs each
entry of a settings list through md(); the oracle runs them one by one in FP64).

* Replicas of both kinds (binary LJ gas, Cu rjl slab) under nve and under nvt
  with one Nose-Hoover chain each, stepped together by the persistent kernel,
  against the oracle's run of each settings file: positions, velocities, the
  energies and the chain's energy after 60 steps.
* run_md_simulation -ilist -batch on a mixed list -- those four entries plus
  two graphene/Cu entries (tb, rjl, morsec; nvt and nve) that the batched kernel
  does not take and that run as concurrent md() calls -- against the oracle's
  -ilist run: every log record, the closing records in all_out and the final
  .xyz files, field by field; and against the same list run with -streams 1
  (one entry at a time), byte for byte.
The precision form's FP32 pair terms set the tolerances."""
import os
import re

import numpy as np
import pytest

import pfmds_gb300 as pf
from pfmds_gb300 import configs
from oracle.pyoracle import Oracle, run_md_simulation as oracle_cli

pytestmark = pytest.mark.gpu
STEPS = 60


def _entries(d):
    configs.lj_gas(d, n_a=300, n_b=300, box=30.0, seed=1, log_period=10, xyz_name="gas_nve.xyz",
                   settings_name="s_gas_nve.txt", integrators=[("nve", 0.5, STEPS, 30, 10)])
    configs.lj_gas(d, n_a=250, n_b=350, box=30.0, seed=2, temperature=150.0, log_period=10, xyz_name="gas_nvt.xyz",
                   settings_name="s_gas_nvt.txt", integrators=[("nvt", 0.5, STEPS, 30, 10)])
    configs.cu_slab(d, nx=5, ny=5, nz=4, seed=3, steps=STEPS, log_period=10, xyz_name="slab_nve.xyz",
                    settings_name="s_slab_nve.txt", integrator="nve")
    configs.cu_slab(d, nx=5, ny=6, nz=4, seed=4, temperature=500.0, steps=STEPS, log_period=10,
                    xyz_name="slab_nvt.xyz", settings_name="s_slab_nvt.txt", integrator="nvt")
    return ["s_gas_nve.txt", "s_gas_nvt.txt", "s_slab_nve.txt", "s_slab_nvt.txt"]


def _write_list(d, names, fname="list.txt"):
    with open(os.path.join(d, fname), "w") as f:
        f.write(f"{len(names)}\n")
        for k, n in enumerate(names):
            f.write(f"{n}\tp{k + 1}_\n")
    return fname


def test_replicas_match_oracle(tmp_path, built):
    d = str(tmp_path)
    names = _entries(d)
    for n in names:
        assert pf.batch_accepts(d, n)[0], n
    b = pf.Batch(d, _write_list(d, names))
    b.run(STEPS + 1)
    h5, per = b.history5()
    for r, n in enumerate(names):
        o = Oracle(d, settings=n, out_period=10 ** 9, threads=os.cpu_count() or 1)
        o.run(STEPS + 1)
        po, vo, _ = o.state()
        p, v, _ = b.state(r)
        xyz = n[2:].replace(".txt", ".xyz")  # s_gas_nve.txt -> gas_nve.xyz
        box = np.array([float(x) for x in re.search(r'Lattice="([^"]*)"', open(os.path.join(d, xyz)).read())
                        .group(1).split()])[[0, 4, 8]]
        dp = np.abs(p - po)
        dp = np.minimum(dp, box - dp)
        assert dp.max() < 1e-4, (n, dp.max())
        assert np.abs(v - vo).max() < 1e-5, (n, np.abs(v - vo).max())
        eo = o.energies()
        row = h5[STEPS // per, r]
        assert row[:3].sum() == pytest.approx(eo["pe"], rel=2e-6, abs=1e-5), n
        assert row[3] == pytest.approx(eo["ke"], rel=2e-5), n
        assert row[4] == pytest.approx(eo["nhc"], rel=1e-4, abs=1e-6), n
        if "nvt" in n:
            assert abs(eo["nhc"]) > 0.0
    b.close()


def _floats(line):
    return [float(x) for x in line.split()[1:]]


def _compare_text(a, b, what, rtol=2e-5, atol=2e-5):
    la, lb = a.rstrip("\n").split("\n"), b.rstrip("\n").split("\n")
    assert len(la) == len(lb), what
    for x, y in zip(la, lb):
        tx, ty = x.split(), y.split()
        assert len(tx) == len(ty), (what, x, y)
        for u, w in zip(tx, ty):
            try:
                fu, fw = float(u), float(w)
            except ValueError:
                assert u == w, (what, x, y)
                continue
            assert abs(fu - fw) <= atol + rtol * abs(fw), (what, x, y)


def test_mixed_list_cli_matches_oracle(tmp_path, built, monkeypatch):
    d = str(tmp_path / "in")
    os.makedirs(d)
    names = _entries(d)
    configs.gr_on_cu(d, n_gx=6, n_gy=4, n_cx=6, n_cy=3, layers=3, steps=STEPS, log_period=10, integrator="nvt",
                     xyz_name="gr.xyz", settings_name="s_gr.txt")
    configs.gr_on_cu(d, n_gx=8, n_gy=4, n_cx=7, n_cy=3, layers=3, seed=9, steps=STEPS, log_period=10,
                     integrator="nve", xyz_name="gr2.xyz", settings_name="s_gr2.txt")
    names.insert(2, "s_gr.txt")
    names.append("s_gr2.txt")
    assert not pf.batch_accepts(d, "s_gr.txt")[0] and not pf.batch_accepts(d, "s_gr2.txt")[0]
    lst = _write_list(d, names)
    outs = {}
    for who in ("gpu", "gpu_one_stream", "oracle"):
        o = str(tmp_path / who)
        os.makedirs(o)
        monkeypatch.chdir(o)  # the same output prefixes in every all_out file
        args = ["-ipath", d + "/", "-ilist", lst, "-ofile", "all_out.txt"]
        if who == "oracle":
            rc = oracle_cli(args)
        else:
            rc = pf.run_md_simulation(args + ["-batch", "-form", "precision"] +
                                      (["-streams", "1"] if who == "gpu_one_stream" else []))
        assert rc == 0, who
        outs[who] = o
    for f in sorted(os.listdir(outs["gpu_one_stream"])):
        if f.endswith((".txt", ".log", ".xyz")):
            assert open(os.path.join(outs["gpu"], f)).read() == \
                open(os.path.join(outs["gpu_one_stream"], f)).read(), f
    _compare_text(open(os.path.join(outs["gpu"], "all_out.txt")).read(),
                  open(os.path.join(outs["oracle"], "all_out.txt")).read(), "all_out")
    for k, n in enumerate(names):
        pre = f"p{k + 1}_"
        _compare_text(open(os.path.join(outs["gpu"], pre + "md_run.log")).read(),
                      open(os.path.join(outs["oracle"], pre + "md_run.log")).read(), n + " log")
        xyz = [f for f in os.listdir(outs["oracle"]) if f.startswith(pre + "final_")]
        assert xyz, n
        for f in xyz:
            _compare_text(open(os.path.join(outs["gpu"], f)).read(), open(os.path.join(outs["oracle"], f)).read(),
                          f, rtol=1e-5, atol=2e-4)
