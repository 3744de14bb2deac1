"""Checks the files and output-unit text of one md() run against records built
by tests/helpers/fortran_records.py from the run's own numbers.

The run is stepped one MD step at a time; at every log, output, snapshot and
trajectory step the values that md() writes are read back through the
runner's API (energies, state, list lengths) and formatted here, independently
of the library's formatter."""
import os
import re

import numpy as np

from . import fortran_records as fr


def read_xyz_input(path):
    with open(path) as f:
        lines = f.read().split("\n")
    n = int(lines[0])
    box = [float(x) for x in re.search(r'Lattice="([^"]*)"', lines[1]).group(1).split()][0::4]
    rows = [ln.split() for ln in lines[2:2 + n]]
    mass = np.array([float(r[6]) for r in rows])
    types = [r[7] for r in rows]
    return n, box, mass, types


def parse_settings(text):
    """Group type lists, the integrators table and the group numbers the
    records need, read from the fixed-order settings text."""
    rec = [r.split() for r in text.split("\n")]
    k = 0

    def nxt():
        nonlocal k
        k += 1
        return rec[k - 1]

    S = {}
    S["step_limit"] = int(nxt()[1])
    S["log"] = nxt()[1]
    S["xyz"] = nxt()[1]
    nxt()
    nxt()
    ntypes = int(nxt()[1])
    ngroups = int(nxt()[1])
    S["groups"] = [[t for t in nxt()[1:1 + ntypes] if t != "#"] for _ in range(ngroups)]
    for key in ("all_moving", "xyz_moving", "z_moving", "all_atoms", "traj_group", "period_traj", "nchange"):
        S[key] = int(nxt()[1])
    for _ in range(2 * S["nchange"]):
        nxt()
    nxt()
    ninteg = int(nxt()[1])
    nxt()
    S["integrators"] = [(t[0], float(t[1]), int(t[2]), int(t[3]), int(t[4])) for t in (nxt() for _ in range(ninteg))]
    nxt()
    S["nhc_num"] = int(nxt()[1])
    for _ in range(S["nhc_num"]):
        nxt()
    nxt()
    ninter = int(nxt()[1])
    nl_n = {"lj": 2, "lj1g": 1, "ljc": 3, "morsec": 3, "tb": 1, "rebosc": 1, "rjl": 1}
    S["inters"] = []
    for _ in range(ninter):
        t = nxt()
        lists = [int(nxt()[2]) for _ in range(nl_n[t[0]])]
        S["inters"].append((t[0], lists))
    return S


def group_index(types, names):
    """create_particle_group's order: by type in the listed order, then by atom."""
    return [i for nm in names for i, t in enumerate(types) if t == nm]


class Expect:
    """Collects the expected records while a run is stepped."""

    def __init__(self, d, settings="md_run_settings.txt"):
        self.d = d
        with open(os.path.join(d, settings)) as f:
            self.text = f.read()
        self.S = parse_settings(self.text)
        self.n, self.box, self.mass, self.types = read_xyz_input(os.path.join(d, self.S["xyz"]))
        self.log, self.blocks, self.snaps, self.traj = [], [], {}, []

    def integrator_at(self, step):
        """Name and table row of the integrator md() uses at `step`
        (md_simulation.f90:121-136 with every stage length positive)."""
        acc = 0
        for row in self.S["integrators"]:
            if step <= acc + row[2]:
                return row
            acc += row[2]
        return self.S["integrators"][-1]

    def sample(self, run, step, out_period):
        """Records of `step` (already taken by `run`)."""
        name, _, _, snap, logp = self.integrator_at(step)
        S = self.S
        p = v = f = None
        if step % logp == 0 or step % out_period == 0:
            e = run.energies()
            total = e["pe"] + e["ke"]
            nhc = [e["nhc"]] if S["nhc_num"] == 1 else []
            if step % logp == 0:
                self.log.append(fr.log_line(name, step, run.sim_time, e["conserved"], e["nhc"], total, e["pe"],
                                            e["ke"], e["temperature"], e["inter"], nhc))
            if step % out_period == 0:
                p, v, f = run.state()
                ia = group_index(self.types, S["groups"][S["all_atoms"] - 1])
                m = self.mass[ia]
                mc = (m[:, None] * p[ia]).sum(0) / m.sum()
                loads = []
                for i, (nm, lists) in enumerate(S["inters"]):
                    for j, nmax in enumerate(lists):
                        loads.append((nm, j + 1, int(run.nlist(i, j)["nnum"].max(initial=0)), nmax))
                self.blocks.append((step, dict(step=step, integrator=name, conserved=e["conserved"], mc=mc,
                                               maxvel=float(np.sqrt((v ** 2).sum(1)).max()), loads=loads)))
        if step % snap == 0 and step != 0:
            if p is None:
                p, v, f = run.state()
            ia = group_index(self.types, S["groups"][S["all_atoms"] - 1])
            self.snaps[step] = fr.snapshot_file(len(ia), self.box, p[ia], v[ia], self.mass[ia],
                                                [self.types[i] for i in ia])
        if step % S["period_traj"] == 0:
            if p is None:
                p, v, f = run.state()
            it = group_index(self.types, S["groups"][S["traj_group"] - 1])
            if it:
                self.traj.append(fr.trajectory_frame(len(it), step, self.box, p[it], v[it], self.mass[it],
                                                     [self.types[i] for i in it]))

    # ---- comparisons -----------------------------------------------------

    def check_log(self, path):
        with open(path) as f:
            lines = f.read().split("\n")
        assert lines[:len(self.log)] == self.log

    def check_files(self, out_dir, prefix=""):
        for step, text in self.snaps.items():
            with open(os.path.join(out_dir, f"{prefix}snapshot_{step:06d}.xyz")) as f:
                assert f.read() == text, f"snapshot at step {step}"
        if self.traj:
            with open(os.path.join(out_dir, f"{prefix}traj_{self.S['traj_group']:02d}.xyz")) as f:
                assert f.read() == "".join(self.traj)

    def check_out(self, text, settings_name="md_run_settings.txt"):
        """The settings echo and every output block in the output-unit text."""
        lines = text.split("\n")
        ngroups = len(self.S["groups"])
        sizes = [len(group_index(self.types, g)) for g in self.S["groups"]]
        echo = fr.settings_echo(self.text, self.n, self.box, sizes[:ngroups], settings_name)
        i0 = lines.index(echo[0])
        assert lines[i0:i0 + len(echo)] == echo
        for step, b in self.blocks:
            k = lines.index("step = " + fr.I(step, 12) + " integrator = " + fr.A(b["integrator"], 6))
            assert lines[k - 1].startswith("exe time (s) = ") and len(lines[k - 1]) == len("exe time (s) = ") + 10
            assert lines[k + 1] == "conserved energy (eV) = " + fr.ES(b["conserved"], 21, 9)
            # the sums of forces and momenta are round-off: only their format is fixed
            assert re.fullmatch(r"forces sum \(eV/A\) = [ \d.E+-]{16}", lines[k + 2]), lines[k + 2]
            assert re.fullmatch(r"c\.o\.m\. velocity \(A/fs\) = [ \d.E+-]{16}", lines[k + 3]), lines[k + 3]
            assert lines[k + 4] == "c.o.m. position (A) = " + "".join(fr.F(x, 12, 6) for x in b["mc"])
            assert lines[k + 5] == "maximum velocity (A/fs) = " + fr.F(b["maxvel"], 12, 6)
            loads = fr.nlists_load_lines(b["loads"])
            assert lines[k + 6:k + 6 + len(loads)] == loads
