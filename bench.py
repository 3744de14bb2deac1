"""Benchmark: atom-steps/s of PFMDS's MD hot path on one GB300.

Workload (the configuration the metric is quoted on): Cu fcc (001) slab of
32x32x16 cubic cells = 65,536 atoms under rjl (A 0.0855 eV, xi 1.224 eV,
p 10.96, q 2.278, r0 2.556 A, switch 4.5-5.0 A), list r_cut 5.5 A rebuilt every
10 steps, bottom two (001) layers fixed, random 0.05 A displacements, 300 K,
NVE with dt 1 fs.  Synthetic seeded input in PFMDS's own file formats.

One benchmark step = 10 MD steps (one list-rebuild period, ending with an energy
evaluation), run on the device from inputs already in HBM; L2 is flushed between
timed steps.  `value` is the precision form (FP32 forces with compensated sums,
FP64 integration and energies); the plain FP64 form is reported beside it with
the precision form's force RMSE against it.  `e2e` runs the same steps through the
C ABI with host buffers: set positions and velocities, advance, read positions,
velocities, forces and energies back.

--impl reference times the CPU oracle (the FP64 restatement of the reference's
Fortran/OpenMP algorithm, O(N^2) list search included) on all host cores.
Several GPUs: independent replicas, one per rank ("replicas only").
"""
import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import threading
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "atom-steps/s on 1 GB300: plain vs chosen form at stated force RMSE and NVE drift"
WORKLOAD = ("Cu fcc (001) slab 32x32x16 cells = 65,536 atoms, rjl (cut-off 5.0 A, list 5.5 A, update period 10 steps), "
            "bottom 2 layers fixed, 300 K, NVE dt 1 fs")
MD_PER_STEP = 10
DT_FS = 1.0


def bench_config():
    """The workload as both arms name it (the same dict in both JSON lines)."""
    return {"workload": WORKLOAD, "atoms": 65536, "md_steps_per_step": MD_PER_STEP,
            "l2": "flushed (256 MiB write) between timed GPU steps"}


def make_workload(d, seed=2024):
    from pfmds_gb300 import configs
    return configs.cu_slab(d, nx=32, ny=32, nz=16, seed=seed, temperature=300.0, dt=DT_FS, steps=10 ** 8,
                           log_period=MD_PER_STEP, integrator="nve")


def peaks():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            j = json.load(f)
        return float(j["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """SM clocks and clock-event (throttle) reasons sampled during the timed region.

    Reads NVML directly (libnvidia-ml, read-only queries) every ~1 ms from a
    thread, so that even a timed region of a few milliseconds gets samples; falls
    back to `nvidia-smi -lms 200` when NVML cannot be loaded."""
    # clock-event reason bits (nvml.h): SW power cap, HW slowdown, SW thermal, HW thermal
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown"}

    def __init__(self, index=0, period_s=0.001):
        self.index, self.period = index, period_s
        self.sm, self.mask, self.max_mhz = [], 0, None
        self.proc, self.lines, self.thread = None, [], None
        self.stop = threading.Event()
        self.source = None

    def _nvml(self):
        import ctypes as C
        lib = C.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        h = C.c_void_p()
        if lib.nvmlDeviceGetHandleByIndex_v2(C.c_uint(self.index), C.byref(h)) != 0:
            raise OSError("no NVML handle")
        mx = C.c_uint()
        if lib.nvmlDeviceGetMaxClockInfo(h, 1, C.byref(mx)) == 0:  # NVML_CLOCK_SM
            self.max_mhz = float(mx.value)
        reasons = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            lib.nvmlDeviceGetCurrentClocksThrottleReasons
        return lib, h, reasons

    def _poll_nvml(self, lib, h, reasons):
        import ctypes as C
        mhz, mask = C.c_uint(), C.c_ulonglong()
        while not self.stop.is_set():
            if lib.nvmlDeviceGetClockInfo(h, 1, C.byref(mhz)) == 0:
                self.sm.append(float(mhz.value))
            if reasons(h, C.byref(mask)) == 0:
                self.mask |= mask.value
            time.sleep(self.period)

    def __enter__(self):
        try:
            lib, h, reasons = self._nvml()
            self.thread = threading.Thread(target=self._poll_nvml, args=(lib, h, reasons), daemon=True)
            self.source = "nvml"
            self.thread.start()
            return self
        except (OSError, AttributeError):
            pass
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.index), "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=lambda: self.lines.extend(ln.strip() for ln in self.proc.stdout),
                                           daemon=True)
            self.source = "nvidia-smi"
            self.thread.start()
        except (OSError, ValueError):
            self.proc = None
        return self

    def __exit__(self, *a):
        self.stop.set()
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)

    def summary(self):
        sm, reasons = list(self.sm), set()
        for bit, name in self.REASONS.items():
            if self.mask & bit:
                reasons.add(name)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                self.max_mhz = float(f[1])
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": self.max_mhz, "reasons": sorted(reasons),
                "samples": len(sm), "source": self.source}


def nve_drift(sim, md_steps, chunk=100):
    """Slope of the conserved energy over `md_steps` NVE steps (least-squares line
    through one sample every `chunk` steps), in eV/atom/ns, and the RMS of the
    samples about that line (eV/atom)."""
    import numpy as np
    n = sim.natoms
    t, e = [0.0], [sim.energies()["conserved"]]
    for k in range(md_steps // chunk):
        sim.advance(chunk)
        t.append((k + 1) * chunk * DT_FS)
        e.append(sim.energies()["conserved"])
    t, e = np.asarray(t), np.asarray(e) / n
    slope, icpt = np.polyfit(t, e, 1)
    rms = float(np.sqrt(np.mean((e - (slope * t + icpt)) ** 2)))
    return float(slope * 1e6), rms


def form_rate(sim, md_steps, reps):
    """atom-steps/s of `reps` timed segments of `md_steps` MD steps (device time,
    L2 flushed before each) after one untimed segment."""
    sim.advance(md_steps)
    ms = 0.0
    for _ in range(reps):
        sim.flush_l2()
        ms += sim.advance_timed(md_steps)
    return sim.natoms * md_steps * reps / (ms / 1e3), ms / (md_steps * reps)


def other_configs(root, device):
    """The workload's sibling configurations, measured beside the headline: the
    binary LJ gas (4,000 atoms, nvt) in both forms with the CPU oracle, and the
    graphene/Cu(111) moire (tb + rjl + morsec, 500 K nvt) in both forms with the
    precision form's force error."""
    import numpy as np
    import pfmds_gb300 as pf
    from pfmds_gb300 import configs
    out = {}
    d1 = os.path.join(root, "lj_gas")
    configs.lj_gas(d1, log_period=10)
    r = {}
    for form in ("plain", "precision"):
        s = pf.Simulation(d1, form=form, out_period=10 ** 9, device=device)
        r[form] = form_rate(s, 10, 10)
        s.close()
    rate_cpu, t_cpu = cpu_oracle_rate(d1, os.cpu_count() or 1, 20)
    out["lj_gas_4000"] = {
        "workload": "binary LJ gas 2,000 A + 2,000 B in a 60 A cube (lj1g A-A, lj1g B-B, lj A-B, R2 7.5 A, "
                    "list 8.5 A every 10 steps), nvt 100 K, dt 0.5 fs",
        "plain": {"value": r["plain"][0], "ms_per_md_step": r["plain"][1]},
        "precision": {"value": r["precision"][0], "ms_per_md_step": r["precision"][1]},
        "cpu_oracle": {"value": rate_cpu, "cores": os.cpu_count() or 1, "sample": f"20 MD steps ({t_cpu:.2f} s)"},
        "unit": "atom-steps/s"}
    d3 = os.path.join(root, "moire")
    configs.gr_on_cu(d3, rotation=(49, 3, 2), layers=6, fixed_layers=1, temperature=500.0, integrator="nvt",
                     dt=0.5, steps=10 ** 8, log_period=10, coupling="morsec")
    r, f = {}, {}
    for form in ("plain", "precision"):
        s = pf.Simulation(d3, form=form, out_period=10 ** 9, device=device)
        s.advance(1)
        f[form] = s.state()[2]
        r[form] = form_rate(s, 10, 5 if form == "plain" else 10)
        n3 = s.natoms
        s.close()
    rmse = float(np.sqrt(((f["precision"] - f["plain"]) ** 2).mean()))
    frms = float(np.sqrt((f["plain"] ** 2).mean()))
    n_c = sum(1 for ln in open(os.path.join(d3, "gr_cu.xyz")).read().splitlines()[2:] if ln.split()[-1] == "C")
    out["graphene_cu_moire"] = {
        "workload": f"graphene (tb, {n_c} C) rotated 2.945 deg on Cu(111) (rjl, 6 layers), morsec coupling "
                    f"(D 0.1 eV, r0 2.2 A, alpha 1.7 1/A, cut-off 8 A), 500 K nvt, dt 0.5 fs; {n3} atoms",
        "plain": {"value": r["plain"][0], "ms_per_md_step": r["plain"][1]},
        "precision": {"value": r["precision"][0], "ms_per_md_step": r["precision"][1],
                      "force_rmse_rel": rmse / frms},
        "unit": "atom-steps/s"}
    return out


def batched_config(root, device, steps, n_rep=512, window=5000):
    """The batched form on its configuration: n_rep replicas (LJ gases and Cu rjl
    slabs of 500-20,000 atoms at 100-1,200 K, nve) stepped together by one persistent
    kernel, after the autotuner picked threads per row per size bucket.  Beside it:
    the same replicas run one at a time through the single-system library (plain
    and precision forms, on a sample of 8), the force error against the plain form
    at the final positions, and each replica's NVE drift from its energy history:
    over the timed run, which starts cold, and over a further `window` steps
    after it, with the plain FP64 form from the same states beside it."""
    import numpy as np
    import pfmds_gb300 as pf
    from pfmds_gb300 import configs
    d = os.path.join(root, "batch")
    t0 = time.perf_counter()
    ln, reps = configs.batch_systems(d, n_rep=n_rep, steps=steps + window, log_period=100,
                                     workers=os.cpu_count() or 1)
    t_gen = time.perf_counter() - t0
    b = pf.Batch(d, ln, device=device)
    R, n_all, _ = b.info()
    b.run(10)
    tpa = b.tune(10)
    ms = b.run(steps - 10)
    rate = n_all * (steps - 10) / (ms / 1e3)
    h, per = b.history()
    ns = np.array([r["n"] for r in reps], float)
    dts = np.array([0.5 if r["kind"] == "lj" else 1.0 for r in reps])
    tot = (h[:, :, 0] + h[:, :, 1]) / ns[None, :]
    rows = np.arange(h.shape[0], dtype=float) * per
    half = h.shape[0] // 2

    def slopes(e, t):  # eV/atom/ns over the whole run and over its second half
        return np.polyfit(t, e, 1)[0] * 1e6, np.polyfit(t[half:], e[half:], 1)[0] * 1e6

    dr = np.array([slopes(tot[:, r], rows * dts[r]) for r in range(R)])
    drift, drift2 = dr[:, 0], dr[:, 1]
    rng = np.random.default_rng(1)
    sample = sorted(rng.choice(R, size=min(8, R), replace=False).tolist())
    rel, t_one = [], {"plain": [0.0, 0.0], "precision": [0.0, 0.0]}
    for r in sample:
        p, v, f = b.state(r)
        s = pf.Simulation(d, settings=reps[r]["settings"], form="plain", out_period=10 ** 9, device=device)
        s.set_state(p, v)
        s.compute()
        fp = s.state()[2]
        rel.append(float(np.sqrt(((f - fp) ** 2).mean()) / np.sqrt((fp ** 2).mean())))
        s.close()
        for form in ("plain", "precision"):
            s = pf.Simulation(d, settings=reps[r]["settings"], form=form, out_period=10 ** 9, device=device)
            s.advance(10)
            t_one[form][0] += s.natoms * 20
            t_one[form][1] += s.advance_timed(20) / 1e3
            s.close()
    one = {k: v[0] / v[1] for k, v in t_one.items()}
    graphs = b.graphs()
    # the drift window: every replica equilibrated by the timed run, `window`
    # more steps; the plain FP64 form runs the same window from the same state on
    # one replica of each kind
    wpick = [next((k for k in sample if reps[k]["kind"] == kind), None) for kind in ("lj", "rjl")]
    w0 = {r: b.state(r)[:2] for r in wpick if r is not None}
    hw0 = h.shape[0]
    if window > 0:
        b.run(window)
    hw, _ = b.history()
    b.close()
    totw = (hw[hw0 - 1:, :, 0] + hw[hw0 - 1:, :, 1]) / ns[None, :]
    rows_w = np.arange(totw.shape[0], dtype=float) * per
    dw = np.array([np.polyfit(rows_w * dts[r], totw[:, r], 1)[0] * 1e6 for r in range(R)]) if window > 0 else None
    win_plain = []
    for r, (p0, v0) in w0.items():
        if window <= 0:
            break
        s = pf.Simulation(d, settings=reps[r]["settings"], form="plain", out_period=10 ** 9, device=device)
        s.set_state(p0, v0)
        e = []
        for k in range(totw.shape[0]):
            s.advance(1 if k == 0 else per)
            en = s.energies()
            e.append((en["pe"] + en["ke"]) / reps[r]["n"])
        s.close()
        win_plain.append({"replica": r, "kind": reps[r]["kind"], "atoms": reps[r]["n"],
                          "plain_fp64": float(np.polyfit(rows_w * dts[r], np.array(e), 1)[0] * 1e6),
                          "batched": float(dw[r])})
    # the plain FP64 form on two of the sampled replicas (one of each kind), same
    # start, same steps, energies every 100 steps: its drift is the integrator's
    plain_drift = []
    for kind in ("lj", "rjl"):
        r = next((k for k in sample if reps[k]["kind"] == kind), None)
        if r is None:
            continue
        s = pf.Simulation(d, settings=reps[r]["settings"], form="plain", out_period=10 ** 9, device=device)
        e = []
        for k in range(h.shape[0]):
            s.advance(1 if k == 0 else per)
            en = s.energies()
            e.append((en["pe"] + en["ke"]) / reps[r]["n"])
        s.close()
        pd = slopes(np.array(e), rows * dts[r])
        plain_drift.append({"replica": r, "kind": kind, "atoms": reps[r]["n"],
                            "temperature": reps[r]["temperature"], "plain_fp64": pd[0],
                            "plain_fp64_second_half": pd[1], "batched": drift[r], "batched_second_half": drift2[r]})
    return {
        "workload": f"{R} replicas (LJ gas or Cu rjl slab, 500-20,000 atoms, 100-1,200 K, nve), {n_all} atoms, "
                    f"{steps} steps, one persistent cooperative kernel per 100 steps"
                    + (", the run replayed as a captured CUDA graph" if graphs > 0 else ", launched directly"),
        "value": rate, "unit": "atom-steps/s", "ms_per_md_step": ms / (steps - 10),
        "tpa_per_bucket": dict(zip(["lj<2k", "lj<8k", "lj>=8k", "rjl<2k", "rjl<8k", "rjl>=8k"], tpa)),
        "one_at_a_time_sample": {"replicas": len(sample), "plain": one["plain"], "precision": one["precision"]},
        "speedup_vs_plain": rate / one["plain"], "speedup_vs_precision_one_at_a_time": rate / one["precision"],
        "force_rmse_rel_vs_plain": {"max": max(rel), "median": float(np.median(rel))},
        "nve_drift_eV_per_atom_per_ns": {"median_abs": float(np.median(np.abs(drift))),
                                         "max_abs": float(np.abs(drift).max()),
                                         "second_half_median_abs": float(np.median(np.abs(drift2))),
                                         "fraction_below_1e-5": float((np.abs(drift) < 1e-5).mean()),
                                         "window_fs": "steps x dt (0.5 fs LJ, 1 fs Cu), energies every 100 steps",
                                         "against_plain_fp64": plain_drift},
        "nve_drift_equilibrated": None if dw is None else {
            "window_steps": window, "after": f"the timed {steps}-step run",
            "median_abs": float(np.median(np.abs(dw))), "max_abs": float(np.abs(dw).max()),
            "fraction_below_1e-5": float((np.abs(dw) < 1e-5).mean()),
            "unit": "eV/atom/ns", "against_plain_fp64": win_plain},
        "input_generation_s": t_gen}


def gr_cu_list_config(root, device, n_entries=16, steps=2000, streams=16):
    """A settings list of graphene/Cu systems (tb, rjl, morsec; 600-3,360 atoms,
    nvt), the kind of entry the persistent batched kernel does not take, through
    run_md_simulation -ilist -batch: one entry at a time (-streams 1) and
    `streams` entries at a time, each an independent md() on its own host thread,
    stream and graphs.  Wall-clock time of the whole list run, set-up, file
    reading and writing included; the two runs' all_out records and log files
    must be identical."""
    import pfmds_gb300 as pf
    from pfmds_gb300 import configs
    d = os.path.join(root, "grlist")
    os.makedirs(d, exist_ok=True)
    sizes = [(10, 6, 9, 5), (16, 10, 14, 8), (20, 12, 18, 10), (24, 14, 21, 12)]
    names, atoms = [], 0
    for k in range(n_entries):
        gx, gy, cx, cy = sizes[k % len(sizes)]
        xyz, sname = f"gr{k}.xyz", f"s_gr{k}.txt"
        configs.gr_on_cu(d, n_gx=gx, n_gy=gy, n_cx=cx, n_cy=cy, seed=100 + k, steps=steps, log_period=1000,
                         integrator="nvt", xyz_name=xyz, settings_name=sname)
        with open(os.path.join(d, xyz)) as f:
            atoms += int(f.readline())
        names.append(sname)
    with open(os.path.join(d, "list.txt"), "w") as f:
        f.write(f"{len(names)}\n")
        for k, n in enumerate(names):
            f.write(f"{n} p{k + 1}_\n")
    out = {}
    for s in (1, streams):
        # output folders of one name length: all_out pads each entry's prefix
        o = os.path.join(d, "out_one" if s == 1 else "out_all") + "/"
        os.makedirs(o, exist_ok=True)
        args = ["-ipath", d + "/", "-ilist", "list.txt", "-opath", o, "-ofile", "all_out.txt", "-batch",
                "-form", "precision", "-device", str(device), "-streams", str(s)]
        sys.stdout.flush()
        saved = os.dup(1)
        null = os.open(os.devnull, os.O_WRONLY)
        os.dup2(null, 1)  # the command line's own banner and per-entry blocks
        try:
            t0 = time.perf_counter()
            rc = pf.run_md_simulation(args)
            wall = time.perf_counter() - t0
        finally:
            os.dup2(saved, 1)
            os.close(saved)
            os.close(null)
        if rc != 0:
            raise RuntimeError(f"list run with -streams {s} returned {rc}")
        files = {}
        for fn in sorted(os.listdir(o)):
            if fn == "all_out.txt" or fn.endswith("md_run.log"):
                with open(os.path.join(o, fn)) as f:
                    files[fn] = f.read().replace(o, "<out>/")  # all_out's records name the output prefix
        out[s] = (wall, files)
    w1, f1 = out[1]
    wn, fn_ = out[streams]
    return {"workload": f"{n_entries} graphene/Cu entries (tb, rjl, morsec; 600-3,360 atoms, nvt), {atoms} atoms, "
                        f"{steps} steps each, run_md_simulation -ilist -batch, precision form",
            "unit": "atom-steps/s (wall clock of the whole list run)",
            "one_at_a_time": {"value": atoms * steps / w1, "wall_s": w1},
            "concurrent": {"streams": streams, "value": atoms * steps / wn, "wall_s": wn},
            "speedup": w1 / wn, "identical_outputs": f1 == fn_ and len(f1) == n_entries + 1}


def learned_config(root, device, frames=500, run_steps=20000):
    """The learned form: networks for the tb (C) and rjl (Cu) interactions trained
    online on plain-form runs of a graphene/Cu(111) system at 300, 700, 1,200 and
    600 K (per-atom energies and forces of the plain kernels; force weight 2, the
    learning rate halved at each temperature), then run on a large graphene/Cu
    system of the same cell proportions (so the same lattice stretch) with the
    classical kernels checking the forces every 100 steps (fallback above
    0.05 eV/A), beside the precision and plain forms of the same system."""
    import pfmds_gb300 as pf
    from pfmds_gb300 import configs
    model, train = None, []
    t0 = time.perf_counter()
    # the learning rate halves at each temperature; the last pass runs at the
    # large system's 600 K
    for T, lr in ((300.0, 2e-3), (700.0, 1e-3), (1200.0, 5e-4), (600.0, 2.5e-4)):
        dT = os.path.join(root, f"learn_T{int(T)}")
        # 6,400 atoms: a cell of the large system's proportions (the same lattice
        # stretch), 5.5x smaller in x and y
        configs.gr_on_cu(dT, n_gx=32, n_gy=20, n_cx=30, n_cy=16, layers=4, temperature=T, integrator="nve", dt=0.5,
                         steps=10 ** 7, log_period=10, tb_list=(32, 4.5))
        s = pf.Simulation(dT, form="plain", out_period=10 ** 9, device=device)
        out = os.path.join(root, f"learned_{int(T)}.bin")
        r, fr = s.learned_train(out, frames=frames, stride=5, iters=8, lr=lr, model_in=model, force_weight=2.0,
                                tensor_cores=True)
        train.append({"temperature": T, "atoms": s.natoms, "energy_rmse_eV": {"C_tb": r[0], "Cu_rjl": r[1]},
                      "force_rmse_eV_per_A": fr})
        model = out
        s.close()
    t_train = time.perf_counter() - t0
    # 5.5 x the training cell in x and y, 6 Cu layers: 77,440 C + 174,240 Cu = 251,680 atoms
    dbig = os.path.join(root, "learn_big")
    # Cu rows hold up to 96 entries: the check every 100 steps, not the list
    # capacity, judges the networks (a denser Cu shell than the 64 of the
    # classical runs is what a drifting network produces first)
    configs.gr_on_cu(dbig, n_gx=176, n_gy=110, n_cx=165, n_cy=88, layers=6, temperature=600.0, integrator="nvt",
                     dt=0.5, steps=10 ** 7, log_period=100, tb_list=(32, 4.5), cu_nmax=96)
    # force evaluations (all interactions, the step's dominant cost) on the large
    # system: classical precision, learned FP32, learned BF16 tensor cores, plain
    res = {}
    for form in ("precision", "learned", "learned_tensor_cores", "plain"):
        s = pf.Simulation(dbig, form="plain" if form == "plain" else "precision", out_period=10 ** 9, device=device)
        n = s.natoms
        if form.startswith("learned"):
            s.learned_use(model, check_period=0, tensor_cores=form.endswith("cores"))
        s.compute()
        ms, _ = s.time_kernel("forces", 10 if form == "plain" else 50)
        res[form] = {"value": n / (ms / 1e3), "ms_per_force_evaluation": ms}
        if form.startswith("learned"):
            res[form]["force_rmse_vs_classical_eV_per_A"] = s.learned_check()
        s.close()
    # one training gradient (energies and force matching) of both networks on the
    # large system: the FP32 CUDA-core kernel against the tcgen05 kernel
    s = pf.Simulation(dbig, form="plain", out_period=10 ** 9, device=device)
    grad_ms = {}
    for tc in (False, True):
        s.learned_gradient(model, tensor_cores=tc, n_networks=2)  # warm-up
        grad_ms["tensor_cores" if tc else "fp32"] = min(
            s.learned_gradient(model, tensor_cores=tc, n_networks=2, timed=True)[2] for _ in range(3))
    s.close()
    res["training_gradient_ms"] = grad_ms
    # MD steps of the classical precision form on the same system (device time)
    s = pf.Simulation(dbig, form="precision", out_period=10 ** 9, device=device)
    s.advance(11)
    ms_prec_step = s.advance_timed(200) / 200
    s.close()
    # the checked run: classical kernels check the networks every 100 steps; the
    # RMSE of every check is collected, and the run's device time per MD step
    s = pf.Simulation(dbig, form="precision", out_period=10 ** 9, device=device)
    s.learned_use(model, check_period=100, max_rmse=0.05, tensor_cores=True)
    checks, run_ms, done = [], 0.0, 0
    try:
        s.advance(1)
        while done < run_steps:
            run_ms += s.advance_timed(100)
            done += 100
            st = s.learned_status()
            checks.append(st["last_rmse"])
            if st["fallen_back"]:
                break
        res["checked_run"] = dict(s.learned_status(), steps=done, check_period=100, max_rmse=0.05,
                                  check_rmse_max=max(checks), check_rmse_median=float(sorted(checks)[len(checks) // 2]),
                                  ms_per_md_step=run_ms / max(done, 1), value=n / (run_ms / max(done, 1) / 1e3),
                                  precision_ms_per_md_step=ms_prec_step,
                                  speedup_vs_precision_md=ms_prec_step / (run_ms / max(done, 1)))
    except pf.PfmdError as e:
        res["checked_run"] = dict(s.learned_status(), steps=done, error=str(e))
    s.close()
    return {
        "workload": f"graphene (tb) on Cu(111) (rjl, 6 layers), morsec coupling, {n} atoms, 600 K nvt, dt 0.5 fs; "
                    f"networks trained on a {train[0]['atoms']}-atom system of the same cell proportions at "
                    f"300/700/1,200/600 K, {frames} frames each (8 Adam steps per frame, force weight 2)",
        "unit": "atom-steps/s", "training": train, "training_s": t_train,
        "metric_here": "atoms per second of force evaluation (all interactions)",
        "precision": res["precision"], "learned": res["learned"],
        "learned_tensor_cores": res["learned_tensor_cores"], "plain": res["plain"],
        "checked_run": res["checked_run"],
        "training_gradient_ms": res["training_gradient_ms"],
        "training_kernels": "tcgen05 (BF16 operands, FP32 accumulation); fp32 beside it",
        "learned_speedup_vs_plain": res["learned_tensor_cores"]["value"] / res["plain"]["value"],
        "learned_vs_precision": res["learned_tensor_cores"]["value"] / res["precision"]["value"],
        "check": "classical kernels recompute the forces every 100 steps; RMSE above 0.05 eV/A switches back"}


def pinned_arrays(n, k):
    """k float64 (n, 3) host arrays in page-locked memory (torch's pinned
    allocator) when a CUDA torch is present, else ordinary numpy arrays."""
    import numpy as np
    try:
        import torch
        if torch.cuda.is_available():
            return [torch.zeros((n, 3), dtype=torch.float64, pin_memory=True).numpy() for _ in range(k)], True
    except (ImportError, RuntimeError):
        pass
    return [np.zeros((n, 3)) for _ in range(k)], False


def cpu_oracle_rate(d, threads, md_steps):
    """Atom-steps/s of the CPU oracle on the workload (set-up excluded)."""
    from oracle.pyoracle import Oracle
    o = Oracle(d, out_period=10 ** 9, threads=threads)
    n = o.natoms
    t0 = time.perf_counter()
    o.run(md_steps)
    t = time.perf_counter() - t0
    return n * md_steps / t, t


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, None
    import torch
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    backend = "nccl" if torch.cuda.is_available() else "gloo"
    dist.init_process_group(backend)
    return dist.get_rank(), dist.get_world_size(), dist


def dist_max(dist, x):
    if dist is None:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_sum(dist, x):
    if dist is None:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def traffic_from_profiles(kernel, form):
    p = os.path.join(HERE, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        j = json.load(f)
    e = j.get(f"{form}:{kernel}")
    return None if e is None else float(e)


def mean_entries(sim, inter, lst):
    """Mean entries per row of one neighbour list (k of the byte model)."""
    nl = sim.nlist(inter, lst)
    return float(nl["nnum"].mean())


def fp64_pipe_from_profiles(kernel):
    """FP64-pipe utilisation (% of peak) of a plain-form kernel from the committed
    ncu summary figures, or None."""
    p = os.path.join(HERE, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        j = json.load(f)
    e = j.get(f"plain:{kernel}:fp64_pipe_pct")
    return None if e is None else {"pct_of_peak": float(e), "source": "ncu (profiles/)"}


def run_ours(args):
    import pfmds_gb300 as pf
    rank, world, dist = dist_init()
    if world > 1:
        os.environ.setdefault("LOCAL_RANK", str(rank))
    device = int(os.environ.get("LOCAL_RANK", "0")) if world > 1 else 0
    K, W, S = args.steps, args.warmup, MD_PER_STEP
    hbm_peak, peak_kind = peaks()
    with tempfile.TemporaryDirectory() as d:
        make_workload(d, seed=2024 + rank)
        sim = pf.Simulation(d, form="precision", out_period=10 ** 9, device=device)
        n = sim.natoms
        for _ in range(W):
            sim.advance_timed(S)
        e0 = sim.energies()["conserved"]
        builds0 = int(sim.nlist_builds()[0])
        barrier(dist)
        launches0 = sim.kernel_launches
        total_ms = 0.0
        vis = os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")
        nvml_index = int(vis[device]) if len(vis) > device and vis[device].strip().isdigit() else device
        with ClockSampler(nvml_index) as clk:
            for _ in range(K):
                sim.flush_l2()
                total_ms += sim.advance_timed(S)
        launches = sim.kernel_launches - launches0
        builds = int(sim.nlist_builds()[0]) - builds0 if builds0 >= 0 else -1
        e1 = sim.energies()["conserved"]
        if args.quick:
            if rank == 0:
                print(json.dumps({"metric": METRIC, "value": n * S * K / (total_ms / 1e3), "unit": "atom-steps/s",
                                  "ms_per_md_step": total_ms / K / S, "quick": True, "gpu_launches": launches}))
            sim.close()
            return
        total_ms = dist_max(dist, total_ms)
        atoms_all = dist_sum(dist, float(n))
        value = atoms_all * S * K / (total_ms / 1e3)
        drift = (e1 - e0) / n / (K * S * DT_FS * 1e-6)  # eV/atom/ns over the timed window

        # roofline of the dominant kernel: time shares per MD step
        # roofline of the dominant kernel by time per MD step, on the algorithmic
        # bytes per atom of the hot-path model: a list pass reads 4 B per entry, the
        # force pass also the own position (16 B fixed point) and writes the force
        # (12 B FP32), and velocity Verlet streams 128 B per atom (x, v, f, 1/m read;
        # x, v written); the rjl density pass is an extra list pass of 4k + 16 B
        k_mean = mean_entries(sim, 0, 0)
        model = {"rjl_force": 4 * k_mean + 16 + 12 + 128, "rjl_density": 4 * k_mean + 16}
        cands = {}
        per_list = builds / (K * S) if builds >= 0 else 1.0 / 10  # rebuilds per MD step in the timed region
        for name, per_md in (("rjl_force", 1.0), ("rjl_density", 1.0), ("lists", per_list)):
            # the fastest of three 50-launch loops: single loops scattered by up to
            # 18% between boxes while the step time did not move
            ms, b = min((sim.time_kernel(name, reps=50) for _ in range(3)), key=lambda t: t[0])
            cands[name] = (ms, b, ms * per_md)
        dom = max(("rjl_force", "rjl_density"), key=lambda k: cands[k][2])
        ms, b_impl, _ = cands[dom]
        b_alg = model[dom] * n
        achieved = b_alg / (ms * 1e-3) / 1e9
        traffic = traffic_from_profiles(dom, "precision")
        step_bytes = (model["rjl_force"] + model["rjl_density"]) * n  # 8k + 172 per atom-step
        step_ms = total_ms / (K * S)
        roofline = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": hbm_peak,
                    "peak_kind": peak_kind, "unit": "GB/s", "frac": round(achieved / hbm_peak, 4),
                    "traffic": traffic, "alg_bytes_per_launch": int(b_alg),
                    "alg_bytes_per_atom": round(model[dom], 1), "entries_per_row": round(k_mean, 2),
                    "ms_per_launch": ms,
                    "impl_bytes_per_launch": int(b_impl),
                    "impl_overhead": "the 8 B per list entry pair-term cache that the density pass writes and "
                                     "the force pass reads, the FP64 force record (32 B) and 1/Eb (4 B per row "
                                     "and per entry) are implementation traffic, not algorithmic bytes",
                    "step": {"alg_bytes_per_atom_step": round(model["rjl_force"] + model["rjl_density"], 1),
                             "ms_per_md_step": step_ms,
                             "achieved": round(step_bytes / (step_ms * 1e-3) / 1e9, 1),
                             "frac": round(step_bytes / (step_ms * 1e-3) / 1e9 / hbm_peak, 4)},
                    "kernel_ms_per_md_step": {k: round(v[2], 5) for k, v in cands.items()}}

        # end to end through the C ABI with host buffers (pinned when torch can pin)
        bufs, pinned = pinned_arrays(n, 5)
        p0, v0 = bufs[0], bufs[1]
        sim.state(out=(p0, v0, bufs[2]))
        t_e2e = 0.0
        for _ in range(max(1, K)):
            t0 = time.perf_counter()
            sim.set_state(p0, v0)
            sim.advance(S)
            sim.state(out=(bufs[2], bufs[3], bufs[4]))
            sim.energies()
            t_e2e += time.perf_counter() - t0
        t_e2e = dist_max(dist, t_e2e)
        e2e = {"value": atoms_all * S * max(1, K) / t_e2e, "unit": "atom-steps/s",
               "h2d_bytes_per_step": 2 * 24 * n, "d2h_bytes_per_step": 3 * 24 * n + 8 * 6,
               "api": "pfmd_set_state + pfmd_advance + pfmd_get_state + pfmd_energies",
               "host_buffers": "pinned" if pinned else "pageable"}

        # plain FP64 form beside it, and the precision form's force error against it
        plain = pf.Simulation(d, form="plain", out_period=10 ** 9, device=device)
        for _ in range(max(1, W // 2)):
            plain.advance(S)
        pms = 0.0
        Kp = max(2, K // 2)
        for _ in range(Kp):
            plain.flush_l2()
            pms += plain.advance_timed(S)
        pms = dist_max(dist, pms)
        plain_rate = atoms_all * S * Kp / (pms / 1e3)
        pk = {}
        for name in ("rjl_force", "rjl_density"):
            pk[name] = plain.time_kernel(name, reps=5)[0]
        pdom = max(pk, key=pk.get)
        # plain FP64 model: position 24 B, force 24 B instead of 16 and 12
        p_model = {"rjl_force": 4 * k_mean + 24 + 24 + 128, "rjl_density": 4 * k_mean + 24}
        p_ach = p_model[pdom] * n / (pk[pdom] * 1e-3) / 1e9
        plain_roof = {"bound": "fp64", "kernel": pdom, "ms_per_launch": pk[pdom],
                      "hbm_achieved": round(p_ach, 1), "hbm_frac": round(p_ach / hbm_peak, 4),
                      "fp64_pipe": fp64_pipe_from_profiles(pdom)}
        ref_p = pf.Simulation(d, form="plain", out_period=10 ** 9, device=device)
        pre_p = pf.Simulation(d, form="precision", out_period=10 ** 9, device=device)
        ref_p.advance(1)
        pre_p.advance(1)
        _, _, fp = ref_p.state()
        _, _, fq = pre_p.state()
        import numpy as np
        rmse = float(np.sqrt(((fq - fp) ** 2).mean()))
        frms = float(np.sqrt((fp ** 2).mean()))
        # NVE drift of both forms over the same window from the same equilibrated
        # state: the precision form runs args.equil_steps first, then each form
        # runs args.drift_steps from that state, with the conserved energy
        # (md_simulation.f90:205's column) sampled every 100 fs
        pre_p.advance(args.equil_steps)
        pe_, ve_, _ = pre_p.state()
        pre_p.close()
        drift_forms = {}
        for form in ("precision", "plain"):
            s_ = pf.Simulation(d, form=form, out_period=10 ** 9, device=device)
            s_.set_state(pe_, ve_)
            s_.advance(1)  # step 0: lists, forces and energies of the equilibrated state
            drift_forms[form] = nve_drift(s_, args.drift_steps)
            s_.close()
        d_pre, rms_pre = drift_forms["precision"]
        d_pla, rms_pla = drift_forms["plain"]
        plain_line = {"value": plain_rate, "ms_per_step": pms / Kp, "ms_per_md_step": pms / Kp / S, "dtype": "f64",
                      "roofline": plain_roof, "speedup_of_precision_form": value / plain_rate}

        extra = other_configs(d, device) if (rank == 0 and not args.no_extra) else None
        if extra is not None and args.batch_steps > 0:
            extra["batched_512"] = batched_config(d, device, args.batch_steps)
        if extra is not None:
            extra["gr_cu_list"] = gr_cu_list_config(d, device)
        if extra is not None and args.learned_steps > 0:
            extra["learned"] = learned_config(d, device, frames=args.learned_frames, run_steps=args.learned_steps)

        cpu = None
        if rank == 0 and not args.no_cpu_baseline:
            threads = os.cpu_count() or 1
            rate, t = cpu_oracle_rate(d, threads, args.cpu_md_steps)
            cpu = {"value": rate, "unit": "atom-steps/s", "cores": threads, "kind": "port",
                   "sample": f"{args.cpu_md_steps} MD steps of the same 65,536-atom workload "
                             f"({t:.1f} s, O(N^2) list search at step 0 as the reference), FP64 oracle, OpenMP"}
        clocks = clk.summary()
        for s in (sim, plain, ref_p):
            s.close()
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": "atom-steps/s", "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": total_ms / K, "ms_per_md_step": total_ms / K / S, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "dtype_detail": "precision form: FP32 pair forces with Kahan sums; FP64 positions, velocities, energies",
        "data": "synthetic",
        "config": bench_config(),
        "form": "precision", "parallelism": f"replicas x{world}", "atoms_per_replica": n,
        "list_rebuilds": {"timed": builds, "update_steps": K * S // 10,
                          "rule": "skin-triggered at the reference's update steps: rebuild when the "
                                  "displacement since the build plus over the last period exceeds "
                                  "half of 5.5 - 5.0 A; a rebuild filters a 6.5 A outer list, itself "
                                  "rebuilt by the cell kernels only when an atom moved 0.5 A since its "
                                  "build"},
        "kick_drift": "fused into the previous step's force kernel except after energy steps",
        "force_rmse": {"value": rmse, "rel": rmse / frms, "unit": "eV/A", "against": "plain FP64 form"},
        "nve_drift": {"value": d_pre, "unit": "eV/atom/ns", "window_fs": args.drift_steps * DT_FS,
                      "equilibration_fs": args.equil_steps * DT_FS,
                      "fit": "least-squares slope of the conserved energy, one sample per 100 fs, both forms "
                             "from the same state after the equilibration",
                      "rms_about_fit_eV_per_atom": rms_pre, "timed_window_value": drift,
                      "plain_fp64": {"value": d_pla, "window_fs": args.drift_steps * DT_FS,
                                     "rms_about_fit_eV_per_atom": rms_pla}},
        "plain": plain_line,
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": clocks,
        "other_configs": extra,
    }
    print(json.dumps(line), flush=True)


def run_case(name):
    """One small run of a single kernel family's workload (for ncu captures of
    that family): the bench slab, the binary LJ gas, the graphene/Cu moire, the
    slab's state transfers, a 64-replica batch or a learned-form force
    evaluation, in the plain or precision form."""
    import pfmds_gb300 as pf
    from pfmds_gb300 import configs
    d = tempfile.mkdtemp()
    form = "plain" if name.endswith("plain") else "precision"
    if name.startswith("slab"):
        configs.cu_slab(d, nx=32, ny=32, nz=16, steps=10 ** 6, log_period=10)
        pf.Simulation(d, form=form, out_period=10 ** 9).advance(23)
    elif name.startswith("gas"):
        configs.lj_gas(d, log_period=10)
        pf.Simulation(d, form=form, out_period=10 ** 9).advance(33)
    elif name.startswith("moire"):
        configs.gr_on_cu(d, rotation=(49, 3, 2), layers=6, fixed_layers=1, temperature=500.0, integrator="nvt",
                         dt=0.5, steps=10 ** 8, log_period=10, coupling="morsec")
        pf.Simulation(d, form=form, out_period=10 ** 9).advance(13)
    elif name == "state":
        # the end-to-end leg's transfers: set_state from and state() into
        # page-locked arrays, 10 of each after one step
        make_workload(d)
        s = pf.Simulation(d, form="precision", out_period=10 ** 9)
        s.advance(1)
        bufs, _ = pinned_arrays(s.natoms, 5)
        s.state(out=(bufs[0], bufs[1], bufs[2]))
        for _ in range(10):
            s.set_state(bufs[0], bufs[1])
            s.state(out=(bufs[2], bufs[3], bufs[4]))
    elif name == "batch":
        ln, _ = configs.batch_systems(d, n_rep=64, n_min=500, n_max=20000, steps=1000, log_period=100, seed=5)
        b = pf.Batch(d, ln)
        b.run(10)
        b.run(200)
    elif name == "learned":
        configs.gr_on_cu(d, n_gx=64, n_gy=64, n_cx=61, n_cy=61, layers=4, temperature=600.0, integrator="nve",
                         dt=0.5, steps=10 ** 7, log_period=100, tb_list=(32, 4.5))
        m = os.path.join(d, "m.bin")
        s = pf.Simulation(d, form="plain", out_period=10 ** 9)
        s.learned_train(m, frames=2, stride=0, iters=1, lr=1e-3)
        s.close()
        s = pf.Simulation(d, form="precision", out_period=10 ** 9)
        s.learned_use(m, check_period=0, tensor_cores=True)
        for _ in range(4):
            s.compute()
    else:
        raise SystemExit(f"unknown case {name}")
    print(json.dumps({"case": name, "done": True}), flush=True)


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    K, W, S = args.steps, args.warmup, MD_PER_STEP
    from oracle.pyoracle import Oracle
    with tempfile.TemporaryDirectory() as d:
        make_workload(d)
        o = Oracle(d, out_period=10 ** 9, threads=threads)
        n = o.natoms
        for _ in range(W):
            o.run(S)
        t0 = time.perf_counter()
        for _ in range(K):
            o.run(S)
        t = time.perf_counter() - t0
    value = n * S * K / t
    line = {"metric": METRIC, "impl": "reference", "value": value, "unit": "atom-steps/s", "n_gpus": 0,
            "steps": K, "warmup": W, "ms_per_step": t / K * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": bench_config(), "form": "reference FP64 algorithm (CPU oracle)",
            "cpu_baseline": {"value": value, "unit": "atom-steps/s", "cores": threads, "kind": "port",
                             "sample": f"{K} timed steps of {S} MD steps after {W} warm-up steps"},
            "e2e": {"value": value, "unit": "atom-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-md-steps", type=int, default=10)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip the LJ-gas, moire and batched configurations")
    ap.add_argument("--batch-steps", type=int, default=5000, help="MD steps of the batched configuration (0 skips)")
    ap.add_argument("--learned-steps", type=int, default=20000, help="MD steps of the learned form's run (0 skips)")
    ap.add_argument("--drift-steps", type=int, default=10000,
                    help="MD steps of the NVE drift measurement (both forms, after the equilibration)")
    ap.add_argument("--equil-steps", type=int, default=2000,
                    help="MD steps of precision-form equilibration before the drift window")
    ap.add_argument("--quick", action="store_true",
                    help="headline timing loop only (no plain form, e2e, roofline or CPU legs), for profiling")
    ap.add_argument("--learned-only", action="store_true",
                    help="the learned form's leg alone (prints its JSON), for profiling its kernels")
    ap.add_argument("--learned-frames", type=int, default=500, help="training frames per temperature")
    ap.add_argument("--case", default=None,
                    help="run one small workload for a kernel family and exit (ncu captures): slab_plain, "
                         "slab_prec, gas_plain, gas_prec, moire_plain, moire_prec, state, batch, learned")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        # the reference arm builds and loads only the CPU oracle: nothing of the
        # CUDA library is loaded into this process
        from oracle import build_oracle
        build_oracle.build()
        run_reference(args)
        return
    import __graft_entry__
    __graft_entry__.build()
    if args.case:
        run_case(args.case)
    elif args.learned_only:
        with tempfile.TemporaryDirectory() as d:
            print(json.dumps(learned_config(d, 0, frames=args.learned_frames, run_steps=args.learned_steps)),
                  flush=True)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
