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
DESC_FLOATS = 2 + NR + NR + 2 + 4 + 2 + NG + NG
NET_FLOATS = NH * NG + NH + NH * NH + NH + NH + 1


def load_models(path):
    raw = open(path, "rb").read()
    assert raw[:8] == b"PFMDMLP1", "not a learned-potential file"
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
                    zeta=take(4), lam=take(2), mean=take(NG), inv_std=take(NG))
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


def energy(pos, box, idx, model):
    return float(atom_energies(descriptors(pos, box, idx, model["desc"]), model).sum())


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
