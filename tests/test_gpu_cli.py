"""run_md_simulation, the drop-in executable, against the oracle's build of the
same program on the same inputs: standard output (timings excepted), the log,
snapshot, trajectory and final .xyz files, in single-file mode and in list mode
(-ilist, with the all_out file)."""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

import pfmds_gb300 as pf
from pfmds_gb300 import configs

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_EXE = os.path.join(ROOT, "oracle", "_build", "oracle_md")
TIMING = re.compile(r"TIME|time \(s\)|OPENMP THREADS|PERFOMANCE|:\s+[0-9.]+ S\s")
NUM = re.compile(r"^[-+]?(\d+\.?\d*|\.\d+)([eEdD][-+]?\d+)?$")


def _case(d):
    configs.lj_gas(str(d), n_a=60, n_b=60, box=18.0, min_sep=2.8,
                   integrators=[("nvt", 0.5, 20, 10, 5), ("nve", 0.5, 20, 10, 5)])


def _run(exe, cwd, args):
    r = subprocess.run([exe] + args, cwd=cwd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return r.stdout


def _same_text(a, b, what, atol=1e-9, rtol=1e-7):
    la, lb = a.splitlines(), b.splitlines()
    assert len(la) == len(lb), what
    for x, y in zip(la, lb):
        if TIMING.search(x) or TIMING.search(y):
            mask = lambda t: " ".join(re.sub(r"[0-9.]+", "#", t).split())
            assert mask(x) == mask(y), (what, x, y)
            continue
        tx, ty = x.split(), y.split()
        assert len(tx) == len(ty), (what, x, y)
        for u, v in zip(tx, ty):
            if NUM.match(u) and NUM.match(v) and any(c.isdigit() for c in u):
                fu, fv = float(u.replace("D", "E")), float(v.replace("D", "E"))
                assert abs(fu - fv) <= atol + rtol * abs(fv), (what, x, y)
            else:
                assert u == v, (what, x, y)


def _outputs(d):
    return sorted(f for f in os.listdir(d) if f.endswith((".log", ".xyz", ".txt")) and not f.startswith(
        ("md_run_settings", "second_settings", "AB.xyz", "parameters_", "list")))


def test_single_file_mode(tmp_path, built):
    a, b = tmp_path / "gpu", tmp_path / "cpu"
    _case(a)
    shutil.copytree(a, b)
    args = ["-i", "md_run_settings.txt", "-op", "10", "-omp_n", "4"]
    out_a = _run(pf.EXE_PATH, a, args)
    out_b = _run(ORACLE_EXE, b, args)
    _same_text(out_a, out_b, "stdout")
    files = _outputs(b)
    assert files == _outputs(a) and "md_run.log" in files and any(f.startswith("snapshot_") for f in files)
    for f in files:
        # positions in 16 decimals, energies in 6
        _same_text(open(a / f).read(), open(b / f).read(), f, atol=2e-6 if f.endswith(".log") else 1e-8, rtol=0)


def test_list_mode_with_all_out(tmp_path, built):
    a, b = tmp_path / "gpu", tmp_path / "cpu"
    _case(a)
    s = open(a / "md_run_settings.txt").read()
    s2 = s.replace("nve     0.50000    20", "nve     0.50000    10")
    assert s2 != s
    open(a / "second_settings.txt", "w").write(s2)
    open(a / "list.txt", "w").write("2\nmd_run_settings.txt first_\nsecond_settings.txt second_\n")
    shutil.copytree(a, b)
    args = ["-ilist", "list.txt", "-ofile", "all_out.txt", "-op", "5"]
    out_a = _run(pf.EXE_PATH, a, args)
    out_b = _run(ORACLE_EXE, b, args)
    _same_text(out_a, out_b, "stdout")
    files = _outputs(b)
    assert files == _outputs(a) and "all_out.txt" in files
    assert any(f.startswith("first_") for f in files) and any(f.startswith("second_") for f in files)
    for f in files:
        _same_text(open(a / f).read(), open(b / f).read(), f, atol=2e-6 if f.endswith((".log", ".txt")) else 1e-8,
                   rtol=0)


def test_precision_switches(tmp_path, built):
    """-fuse 0 and -async_io 0 change how the precision form runs, not what it
    writes: the same files, bit for bit (timings aside).  -skin 0 rebuilds every
    list at every update step: the same files within FP32 summation-order noise."""
    base = tmp_path / "base"
    configs.cu_slab(str(base), nx=4, ny=4, nz=4, steps=60, log_period=10, temperature=300.0)
    runs = {}
    for name, extra in (("default", []), ("plain_sched", ["-fuse", "0", "-async_io", "0"]),
                        ("noskin", ["-skin", "0"])):
        d = tmp_path / name
        shutil.copytree(base, d)
        out = _run(pf.EXE_PATH, d, ["-i", "md_run_settings.txt", "-op", "20", "-form", "precision"] + extra)
        runs[name] = (d, out)
    d0, out0 = runs["default"]
    files = _outputs(d0)
    assert "md_run.log" in files
    # the list-load lines report the largest row of lists of different ages
    # when one run keeps lists the other rebuilds
    load = re.compile(r"^\s*\w+\s+\d+\s+\d+\s*/\s*\d+\s*$")
    for name, exact in (("plain_sched", True), ("noskin", False)):
        d, out = runs[name]
        assert _outputs(d) == files
        tol = dict(atol=0.0, rtol=0.0) if exact else dict(atol=1e-6, rtol=1e-6)
        if exact:
            _same_text(out, out0, name + " stdout", **tol)
        else:
            keep = lambda t: "\n".join(x for x in t.splitlines() if not load.match(x))
            _same_text(keep(out), keep(out0), name + " stdout", **tol)
        for f in files:
            _same_text(open(d / f).read(), open(d0 / f).read(), name + " " + f, **tol)


def test_log_lines_written_at_segment_end_match(tmp_path, built):
    # log steps inside a device segment record their values on the device and
    # the lines are written when the segment ends; here no other event ends a
    # segment before the nvms exit, so the log of nvt, nve and the nvms stage up
    # to its exit comes from those records
    a, b = tmp_path / "gpu", tmp_path / "cpu"
    configs.lj_gas(str(a), n_a=60, n_b=60, box=18.0, min_sep=2.8, ms_de=1e-2,
                   integrators=[("nvt", 0.5, 30, 10 ** 8, 5), ("nve", 0.5, 30, 10 ** 8, 5),
                                ("nvms", 0.5, 200, 10 ** 8, 5)])
    shutil.copytree(a, b)
    args = ["-i", "md_run_settings.txt", "-op", "1000000", "-omp_n", "4"]
    out_a = _run(pf.EXE_PATH, a, args)
    out_b = _run(ORACLE_EXE, b, args)
    _same_text(out_a, out_b, "stdout")
    la, lb = open(a / "md_run.log").read(), open(b / "md_run.log").read()
    assert la.count("\n") > 12  # log lines of all three stages
    _same_text(la, lb, "md_run.log", atol=2e-6, rtol=0)
