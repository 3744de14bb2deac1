"""Generates the golden fixtures under tests/golden/<case>/ with the CPU oracle.

Each case directory holds the reference-format inputs (settings, .xyz, parameter
files) and oracle.npz with: the neighbour lists after step 0 (ragged: nnum,
lessnnum and the concatenated valid entries of every list), the forces and
energies after step 0, and positions, velocities, forces and energies after
STEPS steps; md_run.log holds the log file of that run.  The oracle runs on one
thread so every reduction has a fixed order.

    python tests/golden/make_golden.py
"""
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

STEPS = 20


def cases():
    from pfmds_gb300 import configs
    return {
        "lj_gas": lambda d: configs.lj_gas(d, n_a=150, n_b=150, box=24.0,
                                           integrators=[("nvt", 0.5, 10, 10 ** 8, 5), ("nve", 0.5, 10, 10 ** 8, 5)]),
        "cu_slab": lambda d: configs.cu_slab(d, nx=4, ny=4, nz=3, steps=STEPS, log_period=5),
        "gr_morsec": lambda d: configs.gr_on_cu(d, n_gx=6, n_gy=4, n_cx=6, n_cy=3, layers=3, steps=STEPS,
                                                log_period=5),
        "gr_ljc_simplified": lambda d: configs.gr_on_cu(d, n_gx=6, n_gy=4, n_cx=6, n_cy=3, layers=3,
                                                        coupling="ljc", simplified=True, steps=STEPS,
                                                        log_period=5, integrator="nve"),
    }


def collect(o):
    """Lists, forces and energies of an oracle run at its current point."""
    out = {}
    for i in range(o.n_interactions):
        for j in range(3):
            try:
                nl = o.nlist(i, j)
            except Exception:
                break
            key = f"nl_{i}_{j}"
            out[key + "_nnum"] = nl["nnum"]
            out[key + "_less"] = nl["lessnnum"]
            out[key + "_entries"] = np.concatenate([nl["nlist"][r, :n] for r, n in enumerate(nl["nnum"])]
                                                   or [np.zeros(0, np.int32)]).astype(np.int32)
    return out


def make(case, builder):
    from oracle.pyoracle import Oracle
    d = os.path.join(HERE, case)
    if os.path.isdir(d):
        shutil.rmtree(d)
    os.makedirs(d)
    builder(d)
    cwd = os.getcwd()
    os.chdir(d)  # output files land beside the inputs, with an empty prefix
    try:
        o = Oracle("", out_period=10 ** 6, threads=1, write_files=True, prefix="")
        o.step()
        data = collect(o)
        p, v, f = o.state()
        e = o.energies()
        data.update(f0=f, e0_inter=e["inter"], e0_ke=e["ke"])
        o.run(STEPS)
        o.finish()
        p, v, f = o.state()
        e = o.energies()
        data.update(pos=p, vel=v, frc=f, e_inter=e["inter"], e_pe=e["pe"], e_ke=e["ke"], e_cons=e["conserved"],
                    md_step=o.md_step, sim_time=o.sim_time)
        del o
    finally:
        os.chdir(cwd)
    np.savez_compressed(os.path.join(d, "oracle.npz"), **data)
    # keep only the inputs and the log of the run
    for fn in os.listdir(d):
        if fn.startswith(("final_", "traj_", "snapshot_")):
            os.remove(os.path.join(d, fn))


if __name__ == "__main__":
    for name, b in cases().items():
        make(name, b)
        print(name, sorted(os.listdir(os.path.join(HERE, name))))
