"""Seeded synthetic systems written in PFMDS's own input formats.

PFMDS ships no example inputs (its examples live in a separate manual
repository), so the workloads are generated here: the extended .xyz file read by
read_box_size / read_particles (md_read_write.f90:22-61), the potential parameter
files of the read_*_parameters routines, and the fixed-order settings file read
by md() (md_simulation.f90:48-94).

Systems:
  lj_gas     binary Lennard-Jones gas (A: 39.95 amu, eps 0.0104 eV, sigma 3.40 A;
             B: 20.18 amu, eps 0.0031 eV, sigma 2.74 A; A-B Lorentz-Berthelot),
             uniform positions with a minimum separation, lj1g A-A / B-B and lj A-B
  cu_slab    fcc Cu (001) slab under rjl, bottom layers CU_fixed, vacuum above
  gr_on_cu   graphene sheet (tb) on a Cu(111) slab (rjl) coupled by morsec or
             ljc, with an in-plane rotation of the sheet

All randomness comes from numpy's PCG64 seeded generator.
"""
import math
import os

import numpy as np

MASS_COEF = 1.6605389217 / 1.6021765654 * 100.0  # amu*A^2/fs^2 -> eV (md_general.f90:165)
KB = 1.3806488 / 1.6021765654 * 1e-4  # eV/K (md_general.f90:304)


def _fmt_xyz(box, pos, vel, mass, types):
    lines = [f"{len(types):12d}",
             'Lattice="' + "".join(f"{v:16.6f}" for v in
                                   (box[0], 0, 0, 0, box[1], 0, 0, 0, box[2]))
             + ' " Properties=pos:R:3:vel:R:3:mass:R:1:species:S:1']
    fmt = "%27.16f" * 7 + "    %s"
    rows = np.concatenate([np.asarray(pos, float), np.asarray(vel, float), np.asarray(mass, float)[:, None]], axis=1)
    lines.extend(fmt % (*r, t) for r, t in zip(rows.tolist(), types))
    return "\n".join(lines) + "\n"


def write_xyz(path, box, pos, vel, mass, types):
    with open(path, "w") as f:
        f.write(_fmt_xyz(box, pos, vel, mass, types))


def maxwell_velocities(rng, mass, moving, temperature):
    """Gaussian velocities for the `moving` atoms, zero total momentum over them,
    rescaled so that T = 2 KE / (kB 3 N) (md_general.f90:301-310) is exact."""
    n = len(mass)
    vel = np.zeros((n, 3))
    idx = np.nonzero(moving)[0]
    if len(idx) == 0 or temperature <= 0:
        return vel
    m = mass[idx][:, None]
    v = rng.standard_normal((len(idx), 3)) * np.sqrt(KB * temperature / (m * MASS_COEF))
    v -= (m * v).sum(0) / m.sum()
    ke = 0.5 * (m[:, 0] * (v ** 2).sum(1)).sum() * MASS_COEF
    t = 2 * ke / KB / (3 * len(idx))
    v *= math.sqrt(temperature / t)
    vel[idx] = v
    return vel


def _settings_text(*, step_limit, xyz_name, types, groups, all_moving, xyz_moving, z_moving,
                   all_atoms, traj_group, period_traj, integrators, ms_de, nhc, t0,
                   interactions, new_velocities=False, zero_momentum_period=1000000000,
                   changes=(), invert_z_vel=False, logname="md_run.log"):
    L = []
    L.append(f"md_step_limit:\t\t\t\t{step_limit}")
    L.append(f"logfilename:\t\t\t\t{logname}")
    L.append(f"init_xyz_filename:\t\t\t{xyz_name}")
    L.append(f"new_velocities:\t\t\t\t{'T' if new_velocities else 'F'}")
    L.append(f"zero_momentum_period:\t\t{zero_momentum_period}")
    L.append(f"particle_types_num:\t\t\t{len(types)}")
    L.append(f"groups_num:\t\t\t\t\t{len(groups)}")
    for k, g in enumerate(groups, 1):
        names = list(g) + ["#"] * (len(types) - len(g))
        L.append(f"\t{k}\t\t" + "\t".join(names))
    L.append(f"all_moving_atoms_group_num:\t\t{all_moving}")
    L.append(f"xyz_moving_atoms_group_num:\t\t{xyz_moving}")
    L.append(f"z_moving_atoms_group_num:\t\t{z_moving}")
    L.append(f"all_atoms_group_num:\t\t{all_atoms}")
    L.append(f"traj_group_num:\t\t\t\t{traj_group}")
    L.append(f"period_traj:\t\t\t\t{period_traj}")
    L.append(f"change_group_num:\t\t\t{len(changes)}")
    for (gfrom, gto, ts1, ts2, frec) in changes:
        L.append(f"change_groups:\t{gfrom}\t{gto}")
        L.append(f"change_steps:\t{ts1}\t{ts2}\t{frec}")
    L.append(f"invert_z_vel:\t\t\t\t{'T' if invert_z_vel else 'F'}")
    L.append(f"integrators_num:\t\t\t{len(integrators)}")
    L.append(" name    dt         len     snap     log")
    for (name, dt, n, snap, log) in integrators:
        L.append(f" {name:<6s}  {dt:.5f}    {n}\t{snap}    {log}")
    L.append(f"ms_de:\t\t\t\t\t\t{ms_de:g}")
    L.append(f"nhc_num:\t\t\t\t\t{len(nhc)}")
    for (g, t, m, q1) in nhc:
        L.append(f"{g}\t{t:.6g}\t{m}\t{q1:.10g}")
    L.append(f"initial_temperature:\t\t{t0:g}")
    L.append(f"interactions_num:\t\t\t{len(interactions)}")
    for (name, pfile, lists) in interactions:
        L.append(f"{name}\t{pfile}")
        for (g1, g2, nmax, rc, per) in lists:
            L.append(f"{g1}\t{g2}\t{nmax}\t\t{rc:g}\t\t{per}")
    return "\n".join(L) + "\n"


def _write(d, name, text):
    with open(os.path.join(d, name), "w") as f:
        f.write(text)


def _uniform_min_sep(rng, n, box, dmin, max_tries=200):
    """n points uniform in the periodic box with pairwise minimum-image distance >= dmin
    (random sequential addition with a cell grid)."""
    box = np.asarray(box, float)
    nc = np.maximum(1, np.floor(box / dmin).astype(int))
    cs = box / nc
    cells = {}
    pts = np.empty((n, 3))
    k = 0
    tries = 0
    while k < n:
        tries += 1
        if tries > max_tries * n:
            raise RuntimeError("could not place atoms with the requested minimum separation")
        p = rng.random(3) * box
        c = np.floor(p / cs).astype(int) % nc
        ok = True
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    key = tuple((c + (dx, dy, dz)) % nc)
                    for j in cells.get(key, ()):
                        d = pts[j] - p
                        d -= box * np.round(d / box)
                        if d @ d < dmin * dmin:
                            ok = False
                            break
                    if not ok:
                        break
                if not ok:
                    break
            if not ok:
                break
        if ok:
            pts[k] = p
            cells.setdefault(tuple(c), []).append(k)
            k += 1
    return pts


def _uniform_min_sep_batched(rng, n, box, dmin):
    """Uniform positions with a minimum separation, drawn in vectorised rounds:
    candidates closer than dmin to an accepted point are dropped, then of each
    too-close pair among the survivors the later one.  Uses scipy's periodic k-d
    tree; much faster than the one-at-a-time sampler for tens of thousands of atoms."""
    from scipy.spatial import cKDTree
    box = np.asarray(box, float)
    pts = np.empty((0, 3))
    for _ in range(10000):
        need = n - len(pts)
        if need <= 0:
            break
        cand = rng.random((max(64, int(need * 1.5)), 3)) * box
        if len(pts):
            dist, _ = cKDTree(pts, boxsize=box).query(cand, k=1)
            cand = cand[dist >= dmin]
        if len(cand) > 1:
            pairs = cKDTree(cand, boxsize=box).query_pairs(dmin, output_type="ndarray")
            if len(pairs):
                bad = np.zeros(len(cand), bool)
                bad[pairs.max(axis=1)] = True
                cand = cand[~bad]
        pts = np.concatenate([pts, cand[:need]])
    if len(pts) < n:
        raise RuntimeError("could not place atoms with the requested minimum separation")
    return pts


def lj_gas(d, n_a=2000, n_b=2000, box=60.0, seed=12345, temperature=100.0, r1=6.5, r2=7.5,
           rc_list=8.5, period=10, nmax=64, integrators=None, step_limit=None, log_period=100,
           nhc_tau=100.0, min_sep=2.5, ms_de=1e-8, interleave=True, xyz_name="AB.xyz",
           settings_name="md_run_settings.txt", fast_sampler=False, period_traj=100000000):
    """Binary LJ gas (A-B Lorentz-Berthelot) in a periodic cube; writes AB.xyz, the three
    parameter files and md_run_settings.txt into directory d.  Returns the settings name."""
    os.makedirs(d, exist_ok=True)
    rng = np.random.default_rng(seed)
    n = n_a + n_b
    sampler = _uniform_min_sep_batched if fast_sampler else _uniform_min_sep
    pos = sampler(rng, n, (box, box, box), min_sep)
    types = np.array(["A"] * n_a + ["B"] * n_b)
    if interleave:
        types = types[rng.permutation(n)]
    mass = np.where(types == "A", 39.95, 20.18)
    vel = maxwell_velocities(rng, mass, np.ones(n, bool), temperature)
    write_xyz(os.path.join(d, xyz_name), (box, box, box), pos, vel, mass, list(types))
    eps_a, sig_a, eps_b, sig_b = 0.0104, 3.40, 0.0031, 2.74
    eps_ab, sig_ab = math.sqrt(eps_a * eps_b), (sig_a + sig_b) / 2
    _write(d, "parameters_LJ_A-A.txt", f"{eps_a}\t{sig_a}\n{r1}\t{r2}\n")
    _write(d, "parameters_LJ_B-B.txt", f"{eps_b}\t{sig_b}\n{r1}\t{r2}\n")
    _write(d, "parameters_LJ_A-B.txt", f"{eps_ab:.12g}\t{sig_ab:.12g}\n{r1}\t{r2}\n")
    if integrators is None:
        integrators = [("nvt", 0.5, 1000, 100000000, log_period),
                       ("nve", 0.5, 1000, 100000000, log_period),
                       ("nvms", 0.5, 100000, 100000000, log_period)]
    if step_limit is None:
        step_limit = sum(i[2] for i in integrators)
    q1 = 3 * n * KB * temperature * nhc_tau ** 2
    text = _settings_text(
        step_limit=step_limit, xyz_name=xyz_name, types=["A", "B"],
        groups=[["A", "B"], ["A"], ["B"], []], all_moving=1, xyz_moving=1, z_moving=4,
        all_atoms=1, traj_group=3, period_traj=period_traj, integrators=integrators, ms_de=ms_de,
        nhc=[(1, temperature, 3, q1)], t0=temperature,
        interactions=[("lj", "parameters_LJ_A-B.txt", [(2, 3, nmax, rc_list, period),
                                                       (3, 2, nmax, rc_list, period)]),
                      ("lj1g", "parameters_LJ_A-A.txt", [(2, 2, nmax, rc_list, period)]),
                      ("lj1g", "parameters_LJ_B-B.txt", [(3, 3, nmax, rc_list, period)])])
    _write(d, settings_name, text)
    return settings_name


def fcc_slab(nx, ny, nz, a=3.615, z0=5.0, vacuum=25.0):
    """fcc (001) slab of nx*ny*nz cubic cells: positions (sorted by layer, then y, x)
    and the box.  Layer k sits at z0 + k*a/2."""
    basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    g = np.stack(np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij"), -1)
    pts = (g.reshape(-1, 1, 3) + basis[None]).reshape(-1, 3) * a
    order = np.lexsort((pts[:, 0], pts[:, 1], pts[:, 2]))
    pts = pts[order]
    pts[:, 2] += z0
    box = (nx * a, ny * a, nz * a + vacuum)
    return pts, box


def cu_slab(d, nx=32, ny=32, nz=16, a=3.615, fixed_layers=2, seed=2024, temperature=300.0,
            disp=0.05, dt=1.0, steps=10000, log_period=100, rc_list=5.5, period=10, nmax=64,
            r1=4.5, r2=5.0, vacuum=25.0, integrator="nve", nhc_tau=100.0, xyz_name="cu_slab.xyz",
            settings_name="md_run_settings.txt"):
    """Cu fcc (001) slab under rjl; the bottom `fixed_layers` (001) layers are CU_fixed
    and excluded from the moving groups."""
    os.makedirs(d, exist_ok=True)
    rng = np.random.default_rng(seed)
    pos, box = fcc_slab(nx, ny, nz, a, vacuum=vacuum)
    n = len(pos)
    layer = np.rint((pos[:, 2] - pos[:, 2].min()) / (a / 2)).astype(int)
    fixed = layer < fixed_layers
    pos = pos + rng.uniform(-disp, disp, size=pos.shape)
    pos %= np.asarray(box)
    types = np.where(fixed, "CU_fixed", "CU")
    mass = np.full(n, 63.546)
    vel = maxwell_velocities(rng, mass, ~fixed, temperature)
    write_xyz(os.path.join(d, xyz_name), box, pos, vel, mass, list(types))
    # Cu parameters of the rjl (second-moment tight-binding) form
    _write(d, "parameters_RJL_Cu.txt", f"0.0855\t1.224\t10.96\t2.278\t2.556\n{r1}\t{r2}\n")
    nmov = int((~fixed).sum())
    q1 = 3 * nmov * KB * temperature * nhc_tau ** 2
    text = _settings_text(
        step_limit=steps, xyz_name=xyz_name, types=["CU", "CU_fixed"],
        groups=[["CU", "CU_fixed"], ["CU"], []], all_moving=2, xyz_moving=2, z_moving=3,
        all_atoms=1, traj_group=2, period_traj=100000000,
        integrators=[(integrator, dt, steps, 100000000, log_period)], ms_de=1e-8,
        nhc=[(2, temperature, 3, q1)], t0=temperature,
        interactions=[("rjl", "parameters_RJL_Cu.txt", [(1, 1, nmax, rc_list, period)])])
    _write(d, settings_name, text)
    return settings_name


def cu_deposit(d, nx=6, ny=6, nz=4, a=3.615, fixed_layers=1, z_layers=1, n_dep=4, seed=31,
               temperature=300.0, disp=0.05, dt=1.0, integrators=None, log_period=5, rc_list=5.5, period=10,
               nmax=64, vacuum=25.0, change=(3, 30, 5), invert_z_vel=True, dep_speed=0.02,
               xyz_name="cu_dep.xyz", settings_name="md_run_settings.txt"):
    """Cu fcc (001) slab under rjl with the reference's less common step-loop
    paths switched on:
      * the top `z_layers` (001) layers are CU_z, moved only along z
        (integrate_verlet_z_*, molecular_static_1D_velocities);
      * `n_dep` CU_dep atoms (a small cluster, 2.6 A apart) sit in the band
        0.8-0.9 Lz where invert_z_velocities reflects z velocities; they join the
        xyz-moving group one at a time through change_particle_group_N
        (change = (ts1, ts2, frec)): group 4 [CU, CU_dep] starts with the size
        of group 2 [CU];
      * the bottom `fixed_layers` layers are CU_fixed.
    Groups: 1 all, 2 CU, 3 CU_z, 4 CU + CU_dep (xyz-moving), 5 all moving
    (temperature), 6 CU_dep (trajectory)."""
    os.makedirs(d, exist_ok=True)
    rng = np.random.default_rng(seed)
    pos, box = fcc_slab(nx, ny, nz, a, vacuum=vacuum)
    layer = np.rint((pos[:, 2] - pos[:, 2].min()) / (a / 2)).astype(int)
    top = layer.max()
    types = np.where(layer < fixed_layers, "CU_fixed", np.where(layer > top - z_layers, "CU_z", "CU"))
    pos = pos + rng.uniform(-disp, disp, size=pos.shape)
    mass = np.full(len(pos), 63.546)
    vel = maxwell_velocities(rng, mass, types != "CU_fixed", temperature)
    vel[types == "CU_z", :2] = 0.0
    # the deposited cluster: a square of side 2.6 A in the band, half of it in the
    # lower half of the band moving up (inverted at once), half moving down
    zb = 0.85 * box[2]
    dep = np.array([[box[0] / 2 + 2.6 * (k % 2), box[1] / 2 + 2.6 * ((k // 2) % 2), zb + (1.0 if k % 2 else -1.0)]
                    for k in range(n_dep)])
    dvel = np.zeros((n_dep, 3))
    dvel[:, 2] = dep_speed * np.where(np.arange(n_dep) % 2 == 0, 1.0, -1.0)
    pos = np.concatenate([pos, dep]) % np.asarray(box)
    vel = np.concatenate([vel, dvel])
    mass = np.concatenate([mass, np.full(n_dep, 63.546)])
    types = list(types) + ["CU_dep"] * n_dep
    write_xyz(os.path.join(d, xyz_name), box, pos, vel, mass, types)
    _write(d, "parameters_RJL_Cu.txt", "0.0855\t1.224\t10.96\t2.278\t2.556\n4.5\t5.0\n")
    if integrators is None:
        integrators = [("nvt", dt, 20, 100000000, log_period), ("nve", dt, 20, 100000000, log_period),
                       ("nvms", dt, 20, 100000000, log_period)]
    nmov = sum(1 for t in types if t == "CU")
    q1 = 3 * nmov * KB * temperature * 100.0 ** 2
    text = _settings_text(
        step_limit=sum(i[2] for i in integrators), xyz_name=xyz_name, types=["CU", "CU_fixed", "CU_z", "CU_dep"],
        groups=[["CU", "CU_fixed", "CU_z", "CU_dep"], ["CU"], ["CU_z"], ["CU", "CU_dep"], ["CU", "CU_z", "CU_dep"],
                ["CU_dep"]],
        all_moving=5, xyz_moving=4, z_moving=3, all_atoms=1, traj_group=6, period_traj=10,
        integrators=integrators, ms_de=1e-12, nhc=[(2, temperature, 3, q1)], t0=temperature,
        changes=[(2, 4) + tuple(change)] if change else [], invert_z_vel=invert_z_vel,
        interactions=[("rjl", "parameters_RJL_Cu.txt", [(1, 1, nmax, rc_list, period)])])
    _write(d, settings_name, text)
    return settings_name


def graphene_sheet(nx, ny, a=2.46, strain=(1.0, 1.0)):
    """Rectangular graphene cell of nx x ny (a x a*sqrt(3)) cells, 4 atoms each;
    C-C distance a/sqrt(3).  Returns positions (z=0) and the (Lx, Ly) periods."""
    s3 = math.sqrt(3.0)
    basis = np.array([[0.0, 0.0], [a / 2, a / (2 * s3)], [a / 2, a * s3 / 2], [0.0, a * s3 / 2 + a / (2 * s3)]])
    g = np.stack(np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij"), -1).reshape(-1, 1, 2)
    xy = (g * np.array([a, a * s3]) + basis[None]).reshape(-1, 2)
    xy *= np.asarray(strain)
    pos = np.zeros((len(xy), 3))
    pos[:, :2] = xy
    return pos, (nx * a * strain[0], ny * a * s3 * strain[1])


def fcc111_slab(nx, ny, layers, a_s, stretch=(1.0, 1.0)):
    """fcc (111) slab, ABC stacked, nx x ny rectangular (a_s x a_s*sqrt(3)) cells per
    layer (2 atoms each), layer spacing a_s*sqrt(2/3).  Layer 0 at z=0, sorted by
    layer.  Returns positions and the layer index of every atom."""
    s3 = math.sqrt(3.0)
    cell = np.array([[0.0, 0.0], [a_s / 2, a_s * s3 / 2]])
    g = np.stack(np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij"), -1).reshape(-1, 1, 2)
    base = (g * np.array([a_s, a_s * s3]) + cell[None]).reshape(-1, 2)
    shifts = [np.array([0.0, 0.0]), np.array([a_s / 2, a_s / (2 * s3)]), np.array([a_s, a_s / s3])]
    dz = a_s * math.sqrt(2.0 / 3.0)
    pts, lay = [], []
    for k in range(layers):
        xy = base + shifts[k % 3]
        p = np.zeros((len(xy), 3))
        p[:, :2] = xy * np.asarray(stretch)
        p[:, 2] = k * dz
        pts.append(p)
        lay.append(np.full(len(xy), k))
    return np.concatenate(pts), np.concatenate(lay)


def commensurate_rotation(theta_deg, a=2.46, max_len=400.0):
    """Smallest graphene lattice vector m*a1 + n*a2 within max_len whose angle is closest
    to -theta (so rotating the sheet by theta puts it on the x axis).  Returns (m, n,
    angle in degrees, |v|)."""
    best = None
    for m in range(1, int(max_len / a) + 2):
        for n in range(0, m + 1):
            L = a * math.sqrt(m * m + m * n + n * n)
            if L > max_len:
                break
            ang = math.degrees(math.atan2(n * math.sqrt(3) / 2, m + n / 2))
            err = abs(ang - theta_deg)
            if best is None or err < best[0] - 1e-9:
                best = (err, m, n, ang, L)
    return best[1], best[2], best[3], best[4]


def rotated_graphene(m, n, reps_y=1, a=2.46):
    """Graphene rotated so that lattice vector m*a1 + n*a2 lies on x: the rectangular
    periodic cell |v| x sqrt(3)|v|*reps_y/g (exactly commensurate).  Returns
    positions (z=0), (Lx, Ly) and the rotation angle in degrees."""
    s3 = math.sqrt(3.0)
    a1 = np.array([a, 0.0])
    a2 = np.array([a / 2, a * s3 / 2])
    v = m * a1 + n * a2
    w = (m + 2 * n) * a1 - (2 * m + n) * a2  # perpendicular lattice vector, |w| = sqrt(3)|v|
    g = math.gcd(m + 2 * n, 2 * m + n)
    w = w / g
    ang = math.atan2(v[1], v[0])
    R = np.array([[math.cos(-ang), -math.sin(-ang)], [math.sin(-ang), math.cos(-ang)]])
    Lx, Ly = float(np.linalg.norm(v)), float(np.linalg.norm(w)) * reps_y
    basis = np.array([[0.0, 0.0], (a1 + a2) / 3])
    # enumerate lattice points covering the rotated rectangle
    corners = np.array([[0, 0], [Lx, 0], [0, Ly], [Lx, Ly]]) @ R  # back to lattice frame (R^T = R^-1)
    M = np.array([a1, a2]).T
    inv = np.linalg.inv(M)
    cf = corners @ inv.T
    lo = np.floor(cf.min(0)).astype(int) - 2
    hi = np.ceil(cf.max(0)).astype(int) + 2
    ii, jj = np.meshgrid(np.arange(lo[0], hi[0] + 1), np.arange(lo[1], hi[1] + 1), indexing="ij")
    pts = (ii.reshape(-1, 1) * a1 + jj.reshape(-1, 1) * a2)
    allp = np.concatenate([pts + b for b in basis])
    rot = allp @ R.T
    eps = 1e-6
    keep = (rot[:, 0] >= -eps) & (rot[:, 0] < Lx - eps) & (rot[:, 1] >= -eps) & (rot[:, 1] < Ly - eps)
    rot = rot[keep]
    rot[:, 0] = np.mod(rot[:, 0], Lx)
    rot[:, 1] = np.mod(rot[:, 1], Ly)
    pos = np.zeros((len(rot), 3))
    pos[:, :2] = rot
    return pos, (Lx, Ly), math.degrees(ang)


TB_CARBON = (6.325, 1.29, 1.5, 1.315, 0.80469, 0.011304, 19.0, 2.5)  # D S beta r0 delta a0 c0 d0

# rebosc carbon (REBOsolidcarbon.f90:7-25 file layout: A Q alpha / B(3) / beta(3) / T /
# g(6) / R1 R2).  Pair terms: the carbon set of Brenner et al., J. Phys.: Condens.
# Matter 14 (2002) 783.  g: the quintic through that paper's six angular knots
# G(-1, -2/3, -1/2, -1/3, 0, 1) = (-0.01, 0.028207, 0.052804, 0.097321, 0.3, 8.0).
# T: a small dihedral weight chosen here.  Switch 1.7-2.0 A.
REBO_CARBON = dict(
    A=10953.544162170, Q=0.3134602960833, alpha=4.7465390606595,
    B=(12388.79197798, 17.56740646509, 30.71493208065), beta=(4.7204523127, 1.4332132499, 1.3826912506),
    T=-0.004048375,
    g=(0.29999999999999905, 1.0055917166666617, 1.7516746249999886, 2.2404813333333253, 1.943325375000013,
       0.7589269500000115),
    R=(1.7, 2.0))


def rebo_parameters_text(p=REBO_CARBON):
    return (f"{p['A']!r}\t{p['Q']!r}\t{p['alpha']!r}\n" + "\t".join(map(repr, p["B"])) + "\n" +
            "\t".join(map(repr, p["beta"])) + f"\n{p['T']!r}\n" + "\t".join(map(repr, p["g"])) +
            f"\n{p['R'][0]!r}\t{p['R'][1]!r}\n")


def graphene_rebo(d, nx=8, ny=5, seed=11, temperature=300.0, corrugation=0.15, dt=0.5, steps=100,
                  log_period=10, integrator="nve", period=10, nmax=6, rc_list=2.3, vacuum=20.0,
                  xyz_name="gr_rebo.xyz", settings_name="md_run_settings.txt"):
    """A free graphene sheet under rebosc, atoms displaced by up to `corrugation` A
    (so bond angles and dihedrals are not ideal)."""
    os.makedirs(d, exist_ok=True)
    rng = np.random.default_rng(seed)
    gpos, (Lx, Ly) = graphene_sheet(nx, ny)
    gpos[:, 2] = vacuum / 2
    pos = gpos + rng.uniform(-corrugation, corrugation, size=gpos.shape)
    pos[:, 0] %= Lx
    pos[:, 1] %= Ly
    n = len(pos)
    types = ["C"] * n
    mass = np.full(n, 12.011)
    moving = np.ones(n, bool)
    vel = maxwell_velocities(rng, mass, moving, temperature)
    write_xyz(os.path.join(d, xyz_name), (Lx, Ly, vacuum), pos, vel, mass, types)
    _write(d, "parameters_REBO_C.txt", rebo_parameters_text())
    q1 = 3 * n * KB * temperature * 100.0 ** 2
    text = _settings_text(
        step_limit=steps, xyz_name=xyz_name, types=["C"], groups=[["C"], []], all_moving=1, xyz_moving=1,
        z_moving=2, all_atoms=1, traj_group=1, period_traj=100000000,
        integrators=[(integrator, dt, steps, 100000000, log_period)], ms_de=1e-8,
        nhc=[(1, temperature, 3, q1)], t0=temperature,
        interactions=[("rebosc", "parameters_REBO_C.txt", [(1, 1, nmax, rc_list, period)])])
    _write(d, settings_name, text)
    return settings_name


def gr_on_cu(d, n_gx=10, n_gy=6, n_cx=9, n_cy=5, layers=4, fixed_layers=1, a_cu=3.615, height=3.0, vacuum=25.0,
             seed=7, temperature=300.0, disp=0.02, coupling="morsec", simplified=False, dt=0.5, steps=100,
             log_period=10, integrator="nvt", period=10, rotation=None, nhc_tau=100.0, xyz_name="gr_cu.xyz",
             morse=(0.1, 2.2, 1.7, 2.0), morse_r12=(7.0, 8.0), ljc=(0.0168, 2.2, 2.0), ljc_r12=(7.0, 8.0),
             list_skin=0.5, tb_list=(4, 2.0), settings_name="md_run_settings.txt", carbon="tb", cu_nmax=64):
    """Graphene sheet (tb) on a Cu(111) slab (rjl), coupled by morsec or ljc.

    Without `rotation` the sheet has n_gx x n_gy rectangular cells and the Cu
    lattice (n_cx x n_cy cells per layer) is stretched to the same periods.  With
    rotation=(m, n, reps_y) the sheet is the exactly periodic rotated cell of
    rotated_graphene and the Cu counts are chosen to fit it."""
    os.makedirs(d, exist_ok=True)
    rng = np.random.default_rng(seed)
    a_s = a_cu / math.sqrt(2.0)
    if rotation is None:
        gpos, (Lx, Ly) = graphene_sheet(n_gx, n_gy)
    else:
        m, n, reps = rotation
        gpos, (Lx, Ly), _ = rotated_graphene(m, n, reps)
        n_cx = max(1, int(round(Lx / a_s)))
        n_cy = max(1, int(round(Ly / (a_s * math.sqrt(3)))))
    stretch = (Lx / (n_cx * a_s), Ly / (n_cy * a_s * math.sqrt(3)))
    cpos, lay = fcc111_slab(n_cx, n_cy, layers, a_s, stretch)
    z0 = 5.0
    cpos[:, 2] += z0
    ztop = cpos[:, 2].max()
    gpos[:, 2] = ztop + height
    Lz = gpos[:, 2].max() + vacuum
    box = (Lx, Ly, Lz)
    pos = np.concatenate([gpos, cpos])
    types = np.array(["C"] * len(gpos) + [("CU_fixed" if l < fixed_layers else "CU") for l in lay])
    pos = pos + rng.uniform(-disp, disp, size=pos.shape) * (types != "CU_fixed")[:, None]
    pos[:, 0] %= Lx
    pos[:, 1] %= Ly
    mass = np.where(types == "C", 12.011, 63.546)
    moving = types != "CU_fixed"
    vel = maxwell_velocities(rng, mass, moving, temperature)
    write_xyz(os.path.join(d, xyz_name), box, pos, vel, mass, list(types))
    _write(d, "parameters_TB_C.txt", " ".join(f"{v}" for v in TB_CARBON) + "\n1.7\t2.0\n")
    _write(d, "parameters_REBO_C.txt", rebo_parameters_text())
    _write(d, "parameters_RJL_Cu.txt", "0.0855\t1.224\t10.96\t2.278\t2.556\n4.5\t5.0\n")
    if coupling == "morsec":
        _write(d, "parameters_coupling.txt",
               f"{morse[0]}\t{morse[1]}\t{morse[2]}\t{morse[3]}\n{morse_r12[0]}\t{morse_r12[1]}\n"
               f"{'T' if simplified else 'F'}\n")
        rc_c = morse_r12[1] + list_skin
    else:
        _write(d, "parameters_coupling.txt",
               f"{ljc[0]}\t{ljc[1]}\t{ljc[2]}\n{ljc_r12[0]}\t{ljc_r12[1]}\n{'T' if simplified else 'F'}\n")
        rc_c = ljc_r12[1] + list_skin
    nmov = int(moving.sum())
    q1 = 3 * nmov * KB * temperature * nhc_tau ** 2
    text = _settings_text(
        step_limit=steps, xyz_name=xyz_name, types=["C", "CU", "CU_fixed"],
        groups=[["C"], ["CU", "CU_fixed"], ["CU"], ["C", "CU"], ["C", "CU", "CU_fixed"], []],
        all_moving=4, xyz_moving=4, z_moving=6, all_atoms=5, traj_group=1, period_traj=100000000,
        integrators=[(integrator, dt, steps, 100000000, log_period)], ms_de=1e-8,
        nhc=[(4, temperature, 3, q1)], t0=temperature,
        interactions=[(carbon, "parameters_TB_C.txt" if carbon == "tb" else "parameters_REBO_C.txt",
                       [(1, 1, tb_list[0], tb_list[1], period)]),
                      ("rjl", "parameters_RJL_Cu.txt", [(2, 2, cu_nmax, 5.5, period)]),
                      (coupling, "parameters_coupling.txt", [(1, 2, 160, rc_c, period), (2, 1, 160, rc_c, period),
                                                             (1, 1, 3, 1.8, period)])])
    _write(d, settings_name, text)
    return settings_name


def _batch_replica(d, name, kind, n, T, sub, steps, log_period):
    if kind == "lj":
        n_a = n // 2
        box = (n / (4000.0 / 60.0 ** 3)) ** (1.0 / 3.0)
        sf = lj_gas(d, n_a=n_a, n_b=n - n_a, box=box, seed=sub, temperature=T,
                    integrators=[("nve", 0.5, steps, 100000000, log_period)], xyz_name=name + ".xyz",
                    settings_name=name + "_settings.txt", fast_sampler=True)
    else:
        nz = max(4, int(round((n / 4.0) ** (1.0 / 3.0))))
        nxy = max(4, int(round(math.sqrt(n / (4.0 * nz)))))
        # nmax 96: near 1,200 K the 5.5 A shell of a Cu atom fluctuates past 64
        sf = cu_slab(d, nx=nxy, ny=nxy, nz=nz, seed=sub, temperature=T, steps=steps, log_period=log_period,
                     integrator="nve", xyz_name=name + ".xyz", settings_name=name + "_settings.txt", nmax=96)
        n = 4 * nxy * nxy * nz
    return dict(name=name, kind=kind, n=n, temperature=T, settings=sf)


def batch_systems(d, n_rep=512, seed=4242, n_min=500, n_max=20000, t_min=100.0, t_max=1200.0, steps=5000,
                  log_period=10, list_name="batch_list.txt", workers=1):
    """The batched configuration: n_rep independent replicas, each an LJ gas (A-B,
    as lj_gas, dt 0.5 fs) or a Cu rjl slab (as cu_slab, dt 1 fs) with a 50/50 draw,
    sizes uniform in [n_min, n_max] atoms and temperatures uniform in [t_min, t_max]
    K, all nve for `steps` steps.  Writes one settings file and .xyz per replica,
    the shared parameter files, and the settings list (the -ilist format: count,
    then settings file and output prefix per line).  All draws come from `seed`
    first, so `workers` processes (spawned) produce the same files.  Returns the
    list name and the replica descriptions."""
    os.makedirs(d, exist_ok=True)
    rng = np.random.default_rng(seed)
    jobs = []
    for k in range(n_rep):
        n = int(rng.integers(n_min, n_max + 1))
        T = float(rng.uniform(t_min, t_max))
        sub = int(rng.integers(0, 2 ** 31 - 1))
        kind = "lj" if rng.random() < 0.5 else "rjl"
        jobs.append((d, f"rep{k:04d}", kind, n, T, sub, steps, log_period))
    if workers > 1:
        import concurrent.futures as cf
        import multiprocessing as mp
        with cf.ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn")) as ex:
            reps = list(ex.map(_batch_replica, *zip(*jobs), chunksize=4))
    else:
        reps = [_batch_replica(*j) for j in jobs]
    lines = [f"{r['settings']}\t{r['name']}_" for r in reps]
    _write(d, list_name, f"{n_rep}\n" + "\n".join(lines) + "\n")
    return list_name, reps
