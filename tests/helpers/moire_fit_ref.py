"""Restatement of PFMDS's moire fitting run on the CPU oracle -- test
infrastructure only.

It follows runners/run_gr_moire_fitting.f90:47-101 (the golden-section driver)
and fit_gr_moire.f90:16-111 (calc_error) literally, including the file renames
that stage each evaluation's structure and parameter file, and runs every md()
with the oracle (oracle/pyoracle.py).  gr_on_cu_analysis
(graphene_on_surface_analysis.f90:8-29) and position_analysis
(md_general.f90:400-421) are restated with numpy.  The library's fitting runner
is checked against what this produces.
"""
import math
import os

import numpy as np

from oracle import pyoracle


def read_particles(path):
    """(z, types) of an .xyz file (md_read_write.f90:42-61)."""
    with open(path) as f:
        n = int(f.readline().split()[0])
        f.readline()
        z, types = [], []
        for _ in range(n):
            t = f.readline().split()
            z.append(float(t[2].replace("d", "e").replace("D", "e")))
            types.append(t[7])
    return np.array(z), types


def position_analysis(z, types, names, minimum, maximum=1000.0):
    idx = [i for nm in names for i, t in enumerate(types) if t == nm]
    av, k, mi, ma = 0.0, 0, maximum, minimum
    for i in idx:
        v = z[i]
        if minimum < v < maximum:
            av += v
            k += 1
            ma = max(ma, v)
            mi = min(mi, v)
    return np.array([av / k if k else math.nan, mi, ma])


def gr_on_cu_analysis(path, zmin):
    z, types = read_particles(path)
    return (position_analysis(z, types, ["C", "C_a", "C_b"], zmin),
            position_analysis(z, types, ["CU", "CU_fixed", "#"], zmin))


class Fit:
    """setup: dict with input_path, out_path, interaction ('morsec' or 'ljc'),
    prefix, settings, start_xyz, xyz_file, c_num, zero_level, final_file (pairs),
    param_file, rcut, init_min, init_max (4 each), z, be0, grd0 (pair)."""

    def __init__(self, setup, out_period=1):
        self.s = setup
        self.sim_num = 0
        self.out_period = out_period
        self.lines = []

    def op(self, sim):
        return self.s["out_path"] + self.s["prefix"] + f"{sim:06d}_"

    def calc_error(self, params, from_init):
        s, ip = self.s, self.s["input_path"]
        self.sim_num += 1
        sim = self.sim_num
        p = params
        if s["interaction"] == "ljc":
            first = [p[2], p[0], p[1]]
        else:
            first = [p[2], p[0], p[3], p[1]]
        with open(ip + s["param_file"], "w") as f:
            f.write(" ".join(repr(float(v)) for v in first) + "\n")
            f.write(f"{s['rcut'][0]!r} {s['rcut'][1]!r}\nF\n")
        line = f"{sim:6d}" + "".join(f"{v:21.6f}" for v in first)
        prevop = self.op(sim - 1)
        error = 0.0
        for i in range(2):
            xyz = s["xyz_file"][i]
            if from_init:
                os.rename(ip + s["start_xyz"][i], ip + xyz)
            else:
                os.rename(prevop + "final_" + xyz, ip + xyz)
            op = self.op(sim)
            o = pyoracle.Oracle(ip, s["settings"][i], prefix=op, out_period=self.out_period, write_files=True)
            o.run(10 ** 12)
            o.finish()
            e = o.energies()
            del o
            be = float(f"{e['pe'] + e['ke']:20.9f}")  # the total energy as md() prints it
            arr1, arr2 = gr_on_cu_analysis(op + "final_" + xyz, s["z"])
            if from_init:
                os.rename(ip + xyz, ip + s["start_xyz"][i])
            else:
                os.rename(ip + xyz, prevop + "final_" + xyz)
            bd = arr1[0] - arr2[0]
            grd = arr1[2] - arr1[1]
            be = (be - s["zero_level"][i]) / s["c_num"][i]
            line += f"{be:21.6f}{bd:21.6f}{grd:21.6f}"
            if i == 0:
                t1, t2 = (be / s["be0"] - 1.0) ** 2, (grd / s["grd0"][0] - 1.0) ** 2
                error = t1 + t2
                line += f"{t1:21.6f}{t2:21.6f}"
            else:
                t3 = (grd / s["grd0"][1] - 1.0) ** 2
                error = error + t3
                line += f"{t3:21.6f}"
        line += f"{error:21.6f}"
        self.lines.append(line)
        os.rename(ip + s["param_file"], ip + f"{sim:06d}" + s["param_file"])
        return error

    def run(self, delta_error_gold, delta_error_fit):
        gold = (math.sqrt(5.0) - 1.0) / (math.sqrt(5.0) + 1.0)
        imin, imax = list(self.s["init_min"]), list(self.s["init_max"])
        mn, mx = list(imin), list(imax)
        params = [(a + b) / 2 for a, b in zip(imin, imax)]
        err = [0.0] * 4
        error, prev = 0.0, 0.0
        trace = []
        while abs(prev - error) > delta_error_fit or self.sim_num == 0:
            for k in range(3):
                prev = error
                if self.sim_num == 0:
                    prev = 1000000.0
                mn[k], mx[k] = imin[k], imax[k]
                params[k] = mn[k]
                err[0] = self.calc_error(params, True)
                params[k] = mx[k]
                err[3] = self.calc_error(params, True)
                params[k] = mn[k] + (mx[k] - mn[k]) * gold
                err[1] = self.calc_error(params, True)
                params[k] = mx[k] - (mx[k] - mn[k]) * gold
                err[2] = self.calc_error(params, True)
                de = max(err) - min(err)
                gold_i = 0
                while de > delta_error_gold and gold_i <= 20:
                    gold_i += 1
                    if err[1] < err[2]:
                        err[3] = err[2]
                        err[2] = err[1]
                        mx[k] = mx[k] - (mx[k] - mn[k]) * gold
                        params[k] = mn[k] + (mx[k] - mn[k]) * gold
                        err[1] = self.calc_error(params, False)
                    else:
                        err[0] = err[1]
                        err[1] = err[2]
                        mn[k] = mn[k] + (mx[k] - mn[k]) * gold
                        params[k] = mx[k] - (mx[k] - mn[k]) * gold
                        err[2] = self.calc_error(params, False)
                    de = max(err) - min(err)
                loc = int(np.argmin(err))
                error = err[loc]
                params[k] = [mn[k], mn[k] + (mx[k] - mn[k]) * gold, mx[k] - (mx[k] - mn[k]) * gold, mx[k]][loc]
                trace.append(list(params))
        return trace
