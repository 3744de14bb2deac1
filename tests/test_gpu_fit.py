"""The moire fitting runner (run_gr_moire_fitting.f90 with fit_gr_moire.f90):
the library's runner, whose independent md() runs go to the GPU concurrently,
against a literal restatement of the reference's driver running every md() on
the CPU oracle (tests/helpers/moire_fit_ref.py).  Same evaluations in the same
order, the same parameters, and energies, heights and errors within print
precision."""
import os
import shutil

import numpy as np
import pytest

import pfmds_gb300 as pf
from pfmds_gb300 import configs
from tests.helpers import moire_fit_ref as ref

pytestmark = pytest.mark.gpu

MIN = (0.05, 2.0, 1.5, 1.0)  # morsec file order: d r a delt
MAX = (0.2, 2.6, 1.9, 3.0)


def _inputs(d):
    d.mkdir()
    n_c = []
    for i, (seed, h) in enumerate(((3, 3.1), (4, 3.4))):
        name = f"sys{i + 1}"
        configs.gr_on_cu(str(d), n_gx=7, n_gy=5, n_cx=6, n_cy=3, layers=3, seed=seed, height=h,
                         temperature=5.0, integrator="nvms", steps=24, log_period=8, xyz_name=name + ".xyz",
                         settings_name=name + "_settings.txt")
        os.rename(d / (name + ".xyz"), d / (name + "_start.xyz"))
        n_c.append(sum(1 for ln in (d / (name + "_start.xyz")).read_text().splitlines()[2:]
                       if ln.split()[-1] == "C"))
    (d / "morsec_min.txt").write_text(" ".join(map(str, MIN)) + "\n7.0 8.0\n")
    (d / "morsec_max.txt").write_text(" ".join(map(str, MAX)) + "\n")
    return n_c


def _fpfn(path, ip, out, n_c):
    lines = [f"{'input_path:':16s}{ip}", f"{'out_path:':16s}{out}", "interaction_name: morsec",
             "output_prefix: fit_"]
    for i in range(2):
        lines += [f"settings_filename_{i + 1}: sys{i + 1}_settings.txt", f"start_xyz_{i + 1}: sys{i + 1}_start.xyz",
                  f"c_num_{i + 1}: {n_c[i]}", f"zero_energy_level_{i + 1}: {-1000.0 * (i + 1)}",
                  f"final_file_{i + 1}: final_{i + 1}.txt"]
    lines += ["min_param_file: morsec_min.txt", "max_param_file: morsec_max.txt", "z: 1.0", "be0: -0.05",
              "grd0_1: 0.05", "grd0_2: 0.08"]
    path.write_text("\n".join(lines) + "\n")


def _fields(line):
    return [float(v) for v in line.split()]


def test_fit_matches_the_oracle_restatement(tmp_path, built):
    src = tmp_path / "src"
    n_c = _inputs(src)
    arms = {}
    for arm in ("gpu", "cpu"):
        ip, out = tmp_path / arm / "in", tmp_path / arm / "out"
        shutil.copytree(src, ip)
        out.mkdir(parents=True)
        arms[arm] = (f"{ip}/", f"{out}/")
    # GPU arm: the library's runner
    _fpfn(tmp_path / "fit_gpu.txt", *arms["gpu"], n_c)
    assert pf.run_gr_moire_fitting(["-fpfn", str(tmp_path / "fit_gpu.txt"), "-delta_error_gold", "0.02",
                                    "-delta_error_fit", "1e9", "-op", "1000"]) == 0
    gpu = (tmp_path / "gpu" / "out" / "fit_fit_out.txt").read_text().splitlines()
    # CPU arm: the restated driver on the oracle
    ip, out = arms["cpu"]
    setup = dict(input_path=ip, out_path=out, interaction="morsec", prefix="fit_",
                 settings=["sys1_settings.txt", "sys2_settings.txt"], start_xyz=["sys1_start.xyz", "sys2_start.xyz"],
                 xyz_file=["sys1.xyz", "sys2.xyz"], c_num=n_c, zero_level=[-1000.0, -2000.0],
                 final_file=["final_1.txt", "final_2.txt"], param_file="parameters_coupling.txt", rcut=(7.0, 8.0),
                 init_min=[MIN[1], MIN[3], MIN[0], MIN[2]], init_max=[MAX[1], MAX[3], MAX[0], MAX[2]],
                 z=1.0, be0=-0.05, grd0=[0.05, 0.08])
    f = ref.Fit(setup, out_period=1000)
    f.run(0.02, 1e9)
    cpu = f.lines
    assert len(gpu) == len(cpu) >= 13  # the 12 opening evaluations and at least one golden step
    for g, c in zip(gpu, cpu):
        fg, fc = _fields(g), _fields(c)
        assert fg[:5] == fc[:5], (g, c)  # evaluation number and parameters
        assert np.allclose(fg[5:], fc[5:], rtol=1e-7, atol=5e-6), (g, c)  # printed to 6 decimals
    # every evaluation left its numbered parameter file and both final files
    for k in range(1, len(gpu) + 1):
        assert (tmp_path / "gpu" / "in" / f"{k:06d}parameters_coupling.txt").exists()
        for i in (1, 2):
            assert (tmp_path / "gpu" / "out" / f"fit_{k:06d}_final_sys{i}.xyz").exists()
            rec = (tmp_path / "gpu" / "out" / f"fit_{k:06d}_final_{i}.txt").read_text().splitlines()[0]
            assert len(rec) > 81 and len(rec.split()) >= 3
    # the start structures are where they were
    assert (tmp_path / "gpu" / "in" / "sys1_start.xyz").exists() and not (tmp_path / "gpu" / "in" / "sys1.xyz").exists()
