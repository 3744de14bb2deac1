"""CPU reference (FP64 numpy) of the learned form, for the tests only.

It restates the learned potential of the CUDA library from its definition: the
Behler-Parrinello descriptors (32 radial Gaussians, 16 angular functions
2^(1-zeta) (1 + lambda cos)^zeta exp(-eta (r_ij^2 + r_ik^2)) fc fc with
fc = (cos(pi r / rc) + 1)/2), normalised, fed to a 48-64-64-1 SiLU network per
atom.  Energies are summed over the atoms of the interaction's group with the
minimum image of md_general.f90:423-441; forces come from central differences of
that energy, so they check the library's analytic gradient independently.  The
model file layout is the library's (magic, count, then per network its kind, the
descriptor set and the weights as little-endian float32).  No counterpart exists
in the reference, so this is not pinned to it: it pins the library's gradient to
its own energy.
"""
import numpy as np

NR, NA, NG, NH = 32, 16, 48, 64
DESC_FLOATS = 2 + NR + NR + 2 + 4 + 2 + NG + NG + 5
NET_FLOATS = NH * NG + NH + NH * NH + NH + NH + 1


def load_models(path):
    raw = open(path, "rb").read()
    assert raw[:8] == b"PFMDMLP2", "not a learned-potential file"
    n = int(np.frombuffer(raw, np.int32, 1, 8)[0])
    off, out = 12, []
    for _ in range(n):
        kind = int(np.frombuffer(raw, np.int32, 1, off)[0])
        off += 4
        d = np.frombuffer(raw, np.float32, DESC_FLOATS, off).astype(np.float64)
        off += 4 * DESC_FLOATS
        w = np.frombuffer(raw, np.float32, NET_FLOATS, off).astype(np.float64)
        off += 4 * NET_FLOATS
        k = 0

        def take(m):
            nonlocal k
            v = d[k:k + m]
            k += m
            return v
        desc = dict(rc_rad=take(1)[0], rc_ang=take(1)[0], rs=take(NR), eta_r=take(NR), eta_a=take(2),
                    zeta=take(4), lam=take(2), mean=take(NG), inv_std=take(NG), bA=take(1)[0], bp=take(1)[0],
                    br0=take(1)[0], bR1=take(1)[0], bR2=take(1)[0])
        k = 0

        def tw(m):
            nonlocal k
            v = w[k:k + m]
            k += m
            return v
        net = dict(W1=tw(NH * NG).reshape(NH, NG), b1=tw(NH), W2=tw(NH * NH).reshape(NH, NH), b2=tw(NH),
                   w3=tw(NH), b3=tw(1)[0])
        out.append(dict(kind=kind, desc=desc, net=net))
    return out


def _fc(r, rc):
    return 0.5 * (np.cos(np.pi * r / rc) + 1.0) * (r < rc)


def descriptors(pos, box, idx, desc):
    """G (len(idx) x 48) of the atoms idx among themselves."""
    p = pos[idx]
    box = np.asarray(box, float)
    n = len(idx)
    G = np.zeros((n, NG))
    for a in range(n):
        d = p - p[a]
        d -= box * np.round(d / box)
        r = np.sqrt((d * d).sum(1))
        r[a] = np.inf
        m = r < desc["rc_rad"]
        rr = r[m]
        G[a, :NR] = (np.exp(-desc["eta_r"][None, :] * (rr[:, None] - desc["rs"][None, :]) ** 2)
                     * _fc(rr, desc["rc_rad"])[:, None]).sum(0)
        ma = r < desc["rc_ang"]
        u, ru = d[ma], r[ma]
        fa = _fc(ru, desc["rc_ang"])
        for j in range(len(ru)):
            for k in range(j + 1, len(ru)):
                cs = u[j] @ u[k] / (ru[j] * ru[k])
                for il in range(2):
                    t = max(1.0 + desc["lam"][il] * cs, 0.0)
                    for iz in range(4):
                        z = desc["zeta"][iz]
                        for ie in range(2):
                            G[a, NR + (il * 4 + iz) * 2 + ie] += (2.0 ** (1 - z) * t ** z *
                                                                  np.exp(-desc["eta_a"][ie] * (ru[j] ** 2 + ru[k] ** 2))
                                                                  * fa[j] * fa[k])
    return G


def _silu(x):
    return x / (1.0 + np.exp(-x))


def atom_energies(G, model):
    d, w = model["desc"], model["net"]
    x = (G - d["mean"]) * d["inv_std"]
    a1 = _silu(x @ w["W1"].T + w["b1"])
    a2 = _silu(a1 @ w["W2"].T + w["b2"])
    return a2 @ w["w3"] + w["b3"]


# the model's pair terms besides the network (learned.h): the close-contact wall
# (k/2) (r_core - r)^2 per atom and partner below r_core (kCoreK, core_radius)
# and, for rjl networks, the baseline bA sum_j exp(-bp (r/br0 - 1)) fc(r) of each
# atom (the rjl repulsion, RosatoGuillopeLegrand.f90:23-49, with the cosine
# switch of cut_off_function.f90:6-28)
CORE_K = 20.0
CORE_R = {0: 1.15, 1: 2.2}


def _pairs_of(p, box, a):
    d = p - p[a]
    d -= box * np.round(d / box)
    r = np.sqrt((d * d).sum(1))
    r[a] = np.inf
    return d, r


def _base_phi(desc, r):
    """phi(r) and dphi/dr of the baseline (zero when bA = 0)."""
    if desc["bA"] <= 0.0:
        return np.zeros_like(r), np.zeros_like(r)
    R1, R2 = desc["bR1"], desc["bR2"]
    k = 3.14159265358979 / (R2 - R1)
    x = np.clip(r - R1, 0.0, None)
    fc = np.where(r <= R1, 1.0, np.where(r < R2, 0.5 * (1.0 + np.cos(k * x)), 0.0))
    dfc = np.where((r > R1) & (r < R2), -0.5 * k * np.sin(k * x), 0.0)
    e = np.exp(-desc["bp"] * (r / desc["br0"] - 1.0))
    return e * fc, e * (dfc - desc["bp"] / desc["br0"] * fc)


def pair_row_energies(pos, box, idx, model):
    """Wall and baseline energy of each atom of idx (its own partners' share)."""
    p = pos[idx]
    box = np.asarray(box, float)
    rc, d = CORE_R[model["kind"]], model["desc"]
    e = np.zeros(len(idx))
    for a in range(len(idx)):
        _, r = _pairs_of(p, box, a)
        x = rc - r[r < rc]
        e[a] = 0.5 * CORE_K * (x * x).sum()
        m = r < max(d["bR2"], 0.0)
        e[a] += d["bA"] * _base_phi(d, r[m])[0].sum()
    return e


def core_energy(pos, box, idx, model):
    return float(pair_row_energies(pos, box, idx, model).sum())


def pair_forces(pos, box, idx, model, n_atoms):
    """-d(wall + baseline energy)/dx (n_atoms x 3)."""
    p = pos[idx]
    box = np.asarray(box, float)
    rc, d = CORE_R[model["kind"]], model["desc"]
    f = np.zeros((n_atoms, 3))
    for a in range(len(idx)):
        dv, r = _pairs_of(p, box, a)
        m = r < rc
        f[idx[a]] -= ((2.0 * CORE_K * (rc - r[m]) / r[m])[:, None] * dv[m]).sum(0)
        m = r < max(d["bR2"], 0.0)
        if d["bA"] > 0.0 and m.any():
            _, dph = _base_phi(d, r[m])
            f[idx[a]] += ((2.0 * d["bA"] * dph / r[m])[:, None] * dv[m]).sum(0)
    return f


def energy(pos, box, idx, model):
    return (float(atom_energies(descriptors(pos, box, idx, model["desc"]), model).sum())
            + core_energy(pos, box, idx, model))


def forces_fd(pos, box, idx, model, atoms, h=1e-4):
    """-dE/dx by central differences for the given atoms (rows of the result)."""
    f = np.zeros((len(atoms), 3))
    for n, a in enumerate(atoms):
        for c in range(3):
            pp, pm = pos.copy(), pos.copy()
            pp[a, c] += h
            pm[a, c] -= h
            f[n, c] = -(energy(pp, box, idx, model) - energy(pm, box, idx, model)) / (2 * h)
    return f


# ---- descriptor Jacobian, network gradient and the training loss ----------
# The training loss of the library's learned form (learned.h: launch_train_grad)
#   L(W) = wE * mean_rows (E_row - t_row)^2 + wF * sum_atoms |F - F_ref|^2 / (3 N)
# with F = -dE/dx of the summed network energies, restated here in FP64 so that
# tests can check the library's gradient of L with respect to the network's
# weights (FP32 CUDA-core and BF16 tensor-core kernels) by central differences
# of this L.

def _fc_d(r, rc):
    """fc and dfc/dr of the cosine cut-off, zero beyond rc."""
    inside = r < rc
    k = np.pi / rc
    return (0.5 * (np.cos(k * r) + 1.0) * inside, -0.5 * k * np.sin(k * r) * inside)


def descriptors_jacobian(pos, box, idx, desc):
    """G (n x 48, un-normalised) of the atoms idx among themselves and
    J = dG/dx (n x 48 x N x 3) over all N atoms of pos."""
    box = np.asarray(box, float)
    N = len(pos)
    n = len(idx)
    G = np.zeros((n, NG))
    J = np.zeros((n, NG, N, 3))
    p = pos[idx]
    rs, er = desc["rs"], desc["eta_r"]
    for a in range(n):
        d = p - p[a]
        d -= box * np.round(d / box)
        r = np.sqrt((d * d).sum(1))
        r[a] = np.inf
        ia = idx[a]
        # radial
        m = np.nonzero(r < desc["rc_rad"])[0]
        rr, dd = r[m], d[m]
        fc, dfc = _fc_d(rr, desc["rc_rad"])
        ex = np.exp(-er[None, :] * (rr[:, None] - rs[None, :]) ** 2)  # (m, NR)
        G[a, :NR] = (ex * fc[:, None]).sum(0)
        dg = ex * (-2.0 * er[None, :] * (rr[:, None] - rs[None, :]) * fc[:, None] + dfc[:, None])  # dg/dr
        unit = dd / rr[:, None]
        for q, j in enumerate(m):
            contrib = dg[q][:, None] * unit[q][None, :]  # (NR, 3)
            J[a, :NR, idx[j]] += contrib
            J[a, :NR, ia] -= contrib
        # angular
        m = np.nonzero(r < desc["rc_ang"])[0]
        if len(m) < 2:
            continue
        u, ru = d[m], r[m]
        fa, dfa = _fc_d(ru, desc["rc_ang"])
        jj, kk = np.triu_indices(len(m), 1)
        U, V, RU, RV = u[jj], u[kk], ru[jj], ru[kk]
        cs = (U * V).sum(1) / (RU * RV)
        dcs_du = V / (RU * RV)[:, None] - cs[:, None] * U / (RU ** 2)[:, None]
        dcs_dv = U / (RU * RV)[:, None] - cs[:, None] * V / (RV ** 2)[:, None]
        for il in range(2):
            lam = desc["lam"][il]
            t = 1.0 + lam * cs
            pos_t = t > 0
            t = np.where(pos_t, t, 0.0)
            for iz in range(4):
                z = desc["zeta"][iz]
                c0 = 2.0 ** (1 - z)
                tz = t ** z
                dtz = np.where(pos_t, z * t ** (z - 1) * lam, 0.0)  # d t^z / d cs
                for ie in range(2):
                    eta = desc["eta_a"][ie]
                    E = np.exp(-eta * (RU ** 2 + RV ** 2))
                    Bq = E * fa[jj] * fa[kk]
                    col = NR + (il * 4 + iz) * 2 + ie
                    G[a, col] += (c0 * tz * Bq).sum()
                    dB_du = Bq[:, None] * (-2.0 * eta * U) + (E * dfa[jj] * fa[kk])[:, None] * U / RU[:, None]
                    dB_dv = Bq[:, None] * (-2.0 * eta * V) + (E * fa[jj] * dfa[kk])[:, None] * V / RV[:, None]
                    gu = c0 * (dtz[:, None] * dcs_du * Bq[:, None] + tz[:, None] * dB_du)
                    gv = c0 * (dtz[:, None] * dcs_dv * Bq[:, None] + tz[:, None] * dB_dv)
                    for q in range(len(jj)):
                        J[a, col, idx[m[jj[q]]]] += gu[q]
                        J[a, col, idx[m[kk[q]]]] += gv[q]
                        J[a, col, ia] -= gu[q] + gv[q]
    return G, J


def net_vector(model):
    """The network's weights as one vector in the library's Net layout
    (W1, b1, W2, b2, w3, b3)."""
    w = model["net"]
    return np.concatenate([w["W1"].ravel(), w["b1"], w["W2"].ravel(), w["b2"], w["w3"], [w["b3"]]])


def with_net_vector(model, v):
    k = 0

    def take(m):
        nonlocal k
        out = v[k:k + m]
        k += m
        return out
    net = dict(W1=take(NH * NG).reshape(NH, NG), b1=take(NH), W2=take(NH * NH).reshape(NH, NH), b2=take(NH),
               w3=take(NH), b3=take(1)[0])
    return dict(kind=model["kind"], desc=model["desc"], net=net)


def energies_and_dEdG(G, model):
    """Row energies and dE_row/dG (un-normalised descriptor units)."""
    d, w = model["desc"], model["net"]
    x = (G - d["mean"]) * d["inv_std"]
    z1 = x @ w["W1"].T + w["b1"]
    a1 = _silu(z1)
    z2 = a1 @ w["W2"].T + w["b2"]
    a2 = _silu(z2)
    E = a2 @ w["w3"] + w["b3"]

    def dsilu(z):
        s = 1.0 / (1.0 + np.exp(-z))
        return s * (1.0 + z * (1.0 - s))
    gz2 = w["w3"][None, :] * dsilu(z2)
    gz1 = (gz2 @ w["W2"]) * dsilu(z1)
    return E, (gz1 @ w["W1"]) * d["inv_std"]


def training_loss(model, G, J, targets, f_ref, w_energy=1.0, w_force=1.0, e_core=None, f_core=None):
    """L(W) at a configuration: G, J from descriptors_jacobian, per-row energy
    targets and reference forces (N x 3).  The model's energies and forces are
    the network's plus the close-contact wall's (e_core per row, f_core per atom;
    constants of the weights)."""
    E, g = energies_and_dEdG(G, model)
    if e_core is not None:
        E = E + e_core
    loss = w_energy * np.mean((E - targets) ** 2)
    if w_force:
        F = -np.einsum("rf,rfac->ac", g, J)
        if f_core is not None:
            F = F + f_core
        loss += w_force * ((F - f_ref) ** 2).sum() / (3 * len(f_ref))
    return loss


def rjl_atom_energies(pos, box, idx, par):
    """Per-atom rjl energies A0 sum exp(-p(r/r0-1)) fc - xi sqrt(sum exp(-2q(r/r0-1)) fc)
    with the cosine switch fc between R1 and R2 (r <= R2), over the atoms idx
    (RosatoGuillopeLegrand.f90:23-49; cut_off_function.f90:6-16 with its pi)."""
    A0, xi, p, q, r0, R1, R2 = par
    box = np.asarray(box, float)
    P = pos[idx]
    out = np.zeros(len(idx))
    for a in range(len(idx)):
        d = P - P[a]
        d -= box * np.round(d / box)
        r = np.sqrt((d * d).sum(1))
        r[a] = np.inf
        r = r[r <= R2]
        fc = np.where(r < R1, 1.0, 0.5 * (1.0 + np.cos(3.14159265358979 * (r - R1) / (R2 - R1))))
        x = r / r0 - 1.0
        out[a] = A0 * (np.exp(-p * x) * fc).sum() - xi * np.sqrt((np.exp(-2 * q * x) * fc).sum())
    return out
