"""Learned form: networks trained on the plain kernels' per-atom energies stand in
for tb and rjl; the analytic forces are checked against finite differences of the
library's own energy and of the FP64 CPU reference (oracle/learned_ref.py), and the
classical kernels check and replace the networks when they drift."""
import numpy as np
import pytest

import pfmds_gb300 as pf
from pfmds_gb300 import configs
from oracle import learned_ref

pytestmark = pytest.mark.gpu


def _gr(d, T=600.0):
    configs.gr_on_cu(str(d), n_gx=6, n_gy=4, n_cx=6, n_cy=3, layers=3, steps=10 ** 6, log_period=10,
                     integrator="nve", tb_list=(32, 4.5), temperature=T)
    return str(d)


def _train(d, out, frames=40, stride=5, iters=8, model_in=None, force_weight=1.0):
    s = pf.Simulation(d, form="plain", out_period=10 ** 9)
    r, fr = s.learned_train(out, frames=frames, stride=stride, iters=iters, lr=2e-3, model_in=model_in,
                            force_weight=force_weight)
    s.close()
    return r, fr


def test_training_lowers_energy_and_force_errors(tmp_path, built):
    d = _gr(tmp_path)
    m0, m1 = str(tmp_path / "m0.bin"), str(tmp_path / "m1.bin")
    r0, f0 = _train(d, m0, frames=1, stride=0, iters=1)
    r1, f1 = _train(d, m1, frames=60, stride=5, iters=8, model_in=m0)
    assert np.isnan(r0[2]) and np.isnan(r1[2])  # the coupling keeps its classical kernel
    assert (r1[:2] < r0[:2]).all(), (r0, r1)
    assert (r1[:2] < 0.05).all(), r1  # eV per atom
    assert f1 < f0, (f0, f1)  # eV/A, learned against plain forces
    ms = learned_ref.load_models(m1)
    assert sorted(m["kind"] for m in ms) == [0, 1]


def test_energy_matches_cpu_reference_and_forces_its_gradient(tmp_path, built):
    d = _gr(tmp_path)
    m = str(tmp_path / "m.bin")
    _train(d, m, frames=10, stride=5, iters=4)
    s = pf.Simulation(d, form="precision", out_period=10 ** 9)
    s.learned_use(m, check_period=0)
    e = s.compute()
    p, _, f = s.state()
    box = np.array([float(x) for x in open(tmp_path / "gr_cu.xyz").read().splitlines()[1].split('"')[1].split()])[[0, 4, 8]]
    types = [ln.split()[-1] for ln in open(tmp_path / "gr_cu.xyz").read().splitlines()[2:]]
    models = {mm["kind"]: mm for mm in learned_ref.load_models(m)}
    c_idx = np.array([i for i, t in enumerate(types) if t == "C"])
    cu_idx = np.array([i for i, t in enumerate(types) if t.startswith("CU")])
    e_tb = learned_ref.energy(p, box, c_idx, models[0])
    e_rjl = learned_ref.energy(p, box, cu_idx, models[1])
    assert e[0] == pytest.approx(e_tb, abs=2e-5 * len(c_idx))
    assert e[1] == pytest.approx(e_rjl, abs=2e-5 * len(cu_idx))
    # forces: central differences of the library's potential energy (all three
    # interactions) for a few atoms of each kind
    h = 2e-3
    for a in list(c_idx[:3]) + list(cu_idx[-3:]):
        for c in range(3):
            pp, pm = p.copy(), p.copy()
            pp[a, c] += h
            pm[a, c] -= h
            s.set_state(pp)
            ep = s.compute().sum()
            s.set_state(pm)
            em = s.compute().sum()
            fd = -(ep - em) / (2 * h)
            assert abs(fd - f[a, c]) < 2e-3 + 2e-2 * abs(f[a, c]), (a, c, fd, f[a, c])
    s.close()


def test_learned_forces_match_cpu_reference_gradient(tmp_path, built):
    # rjl alone: the library's learned forces against FP64 finite differences of
    # the CPU reference energy
    configs.cu_slab(str(tmp_path), nx=3, ny=3, nz=3, steps=10 ** 6, log_period=10, temperature=800.0)
    m = str(tmp_path / "m.bin")
    s = pf.Simulation(str(tmp_path), form="plain", out_period=10 ** 9)
    s.learned_train(m, frames=8, stride=4, iters=4, lr=2e-3)
    s.close()
    assert np.isfinite(learned_ref.load_models(m)[0]["net"]["W1"]).all()
    s = pf.Simulation(str(tmp_path), form="precision", out_period=10 ** 9)
    s.learned_use(m, check_period=0)
    s.compute()
    p, _, f = s.state()
    box = configs.fcc_slab(3, 3, 3, 3.615, vacuum=25.0)[1]
    model = learned_ref.load_models(m)[0]
    idx = np.arange(len(p))
    atoms = [0, 17, 50, 100]
    ref = learned_ref.forces_fd(p, box, idx, model, atoms, h=1e-4)
    scale = np.abs(ref).max()
    assert np.abs(f[atoms] - ref).max() < 2e-3 * max(scale, 1.0), (f[atoms], ref)
    s.close()


def test_close_contact_wall_matches_cpu_reference(tmp_path, built):
    # two Cu atoms pushed to 1.8 A, inside the rjl network's 2.2 A wall: the
    # library's energy and forces (network plus wall) against the FP64 CPU
    # reference's energy and its central differences
    configs.cu_slab(str(tmp_path), nx=3, ny=3, nz=3, steps=10 ** 6, log_period=10, temperature=300.0)
    m = str(tmp_path / "m.bin")
    s = pf.Simulation(str(tmp_path), form="plain", out_period=10 ** 9)
    s.learned_train(m, frames=4, stride=2, iters=2, lr=2e-3)
    s.close()
    s = pf.Simulation(str(tmp_path), form="precision", out_period=10 ** 9)
    s.learned_use(m, check_period=0)
    s.compute()
    p, _, _ = s.state()
    box = configs.fcc_slab(3, 3, 3, 3.615, vacuum=25.0)[1]
    d = p - p[40]
    d -= box * np.round(d / box)
    r = np.sqrt((d * d).sum(1))
    r[40] = np.inf
    j = int(np.argmin(r))
    p[j] = p[40] + d[j] / r[j] * 1.8
    s.set_state(p)
    e = s.compute()
    _, _, f = s.state()
    model = learned_ref.load_models(m)[0]
    idx = np.arange(len(p))
    assert model["desc"]["bA"] > 0.0  # the rjl repulsion as the baseline
    fc = learned_ref.pair_forces(p, box, idx, model, len(p))
    assert np.abs(fc[40]).max() > 10.0  # the wall alone: 2 k (r_core - r) = 16 eV/A
    assert e[0] == pytest.approx(learned_ref.energy(p, box, idx, model), abs=2e-5 * len(p))
    ref = learned_ref.forces_fd(p, box, idx, model, [40, j], h=1e-4)
    scale = np.abs(ref).max()
    assert np.abs(f[[40, j]] - ref).max() < 2e-3 * max(scale, 1.0), (f[[40, j]], ref)
    s.close()


def test_checked_run_stays_within_the_bound(tmp_path, built):
    # every 10 steps the classical kernels judge the network: the run either stays
    # learned with the force RMSE under the bound or falls back at the first check
    # that exceeds it; either way it completes
    d = _gr(tmp_path)
    m = str(tmp_path / "m.bin")
    _train(d, m, frames=60, stride=5, iters=8)
    s = pf.Simulation(d, form="precision", out_period=10 ** 9)
    s.learned_use(m, check_period=10, max_rmse=0.5)
    s.advance(31)
    st = s.learned_status()
    assert st["checks"] >= 1 and st["last_rmse"] > 0.0
    if st["fallen_back"]:
        assert not st["active"] and st["last_rmse"] > 0.5
    else:
        assert st["active"] and st["checks"] == 3 and st["last_rmse"] <= 0.5
    s.close()


def test_fallback_to_classical_kernels(tmp_path, built):
    d = _gr(tmp_path)
    m = str(tmp_path / "m.bin")
    _train(d, m, frames=2, stride=2, iters=1)
    s = pf.Simulation(d, form="precision", out_period=10 ** 9)
    s.learned_use(m, check_period=5, max_rmse=1e-9)
    s.advance(11)
    st = s.learned_status()
    assert st["fallen_back"] and not st["active"] and st["checks"] == 1
    # after the fallback the run uses the classical kernels: the same forces as a
    # run that never loaded a network, from the same state
    p, v, f = s.state()
    c = pf.Simulation(d, form="precision", out_period=10 ** 9)
    c.set_state(p, v)
    c.compute()
    s.compute()
    fs, fc = s.state()[2], c.state()[2]
    # the same kernels, but not the same FP32 summation order: the learned
    # context rebuilds the tb list at every update step in cell order, the other
    # filters it from its outer list (another order), and the threads per row are
    # tuned per context.  tb's force sums cancel strongly, so the two agree to
    # the precision form's own error scale (force RMSE against FP64 about 1e-5
    # relative), three orders of magnitude below the network's error: forces of
    # the network would fail this check.
    assert np.abs(fs - fc).max() < 1e-5 * np.abs(fc).max()
    s.close()
    c.close()


def test_tensor_core_network_matches_fp32(tmp_path, built):
    """The tcgen05 BF16 network against the FP32 CUDA-core one on the same model
    and configuration: energies and forces within BF16 rounding."""
    d = _gr(tmp_path)
    m = str(tmp_path / "m.bin")
    _train(d, m, frames=20, stride=5, iters=4)
    out = {}
    for tc in (False, True):
        s = pf.Simulation(d, form="precision", out_period=10 ** 9)
        s.learned_use(m, check_period=0, tensor_cores=tc)
        e = s.compute()
        out[tc] = (e, s.state()[2])
        s.close()
    (e32, f32), (e16, f16) = out[False], out[True]
    n = len(f32)
    assert np.all(np.abs(e16[:2] - e32[:2]) < 2e-3 * n), (e16, e32)  # eV over the system
    rel = np.sqrt(((f16 - f32) ** 2).mean()) / np.sqrt((f32 ** 2).mean())
    assert rel < 3e-2, rel


def test_tensor_core_training_gradient_matches_fp32(tmp_path, built):
    """The tcgen05 training kernel (BF16 operands, FP32 accumulation) gives the
    gradient of the FP32 kernel, block by block (W1, b1, W2, b2, w3, b3), to BF16
    accuracy, and repeats bit for bit."""
    d = _gr(tmp_path)
    m = str(tmp_path / "m.bin")
    _train(d, m, frames=6, stride=5, iters=4)
    s = pf.Simulation(d, form="plain", out_period=10 ** 9)
    s.advance(3)
    g32, l32 = s.learned_gradient(m, force_weight=1.0, tensor_cores=False, n_networks=2)
    gtc, ltc = s.learned_gradient(m, force_weight=1.0, tensor_cores=True, n_networks=2)
    gtc2, _ = s.learned_gradient(m, force_weight=1.0, tensor_cores=True, n_networks=2)
    assert np.array_equal(gtc, gtc2)
    np.testing.assert_allclose(ltc, l32, rtol=3e-2)
    NH, NG = 64, 48
    cuts = np.cumsum([0, NH * NG, NH, NH * NH, NH, NH, 1])
    for k in range(2):
        for a, b in zip(cuts[:-1], cuts[1:]):
            x, y = gtc[k, a:b].astype(np.float64), g32[k, a:b].astype(np.float64)
            if b - a == 1:
                # b3: twice the mean energy residual, which training drives towards
                # zero; BF16 moves each row's energy by up to about 2e-3 eV
                assert abs(x[0] - y[0]) < 4e-3 + 5e-2 * abs(y[0]), (k, x, y)
                continue
            rel = np.linalg.norm(x - y) / max(np.linalg.norm(y), 1e-30)
            assert rel < 5e-2, (k, a, b, rel)


def test_tensor_core_training_lowers_energy_and_force_errors(tmp_path, built):
    d = _gr(tmp_path)
    m0, m1 = str(tmp_path / "m0.bin"), str(tmp_path / "m1.bin")
    r0, f0 = _train(d, m0, frames=1, stride=0, iters=1)
    s = pf.Simulation(d, form="plain", out_period=10 ** 9)
    r1, f1 = s.learned_train(m1, frames=60, stride=5, iters=8, lr=2e-3, model_in=m0, tensor_cores=True)
    s.close()
    assert (r1[:2] < r0[:2]).all(), (r0, r1)
    assert (r1[:2] < 0.05).all(), r1
    assert f1 < f0, (f0, f1)


def test_training_gradient_matches_fp64_loss(tmp_path, built):
    """The library's training-loss gradient -- FP32 CUDA-core kernel and BF16
    tensor-core kernel -- against central differences of the FP64 loss of
    oracle/learned_ref.py (energies against per-atom rjl energies, forces
    against the oracle's FP64 forces), along random directions within each block
    of the network's weights and across all of them."""
    from oracle.pyoracle import Oracle
    d = str(tmp_path)
    configs.cu_slab(d, nx=3, ny=3, nz=3, steps=10 ** 6, log_period=10, temperature=800.0)
    m = str(tmp_path / "m.bin")
    s = pf.Simulation(d, form="plain", out_period=10 ** 9)
    s.learned_train(m, frames=20, stride=5, iters=4, lr=2e-3)
    s.close()
    s = pf.Simulation(d, form="plain", out_period=10 ** 9)  # the input configuration
    g32, loss32 = s.learned_gradient(m, force_weight=1.0)
    gtc, losstc = s.learned_gradient(m, force_weight=1.0, tensor_cores=True)
    s.close()
    o = Oracle(d, out_period=1, threads=1)
    o.step()
    pos, _, f_ref = o.state()
    lines = open(tmp_path / "cu_slab.xyz").read().splitlines()
    box = np.array([float(x) for x in lines[1].split('"')[1].split()])[[0, 4, 8]]
    par = [float(x) for x in open(tmp_path / "parameters_RJL_Cu.txt").read().split()]
    idx = np.arange(len(pos))
    model = learned_ref.load_models(m)[0]
    G, J = learned_ref.descriptors_jacobian(pos, box, idx, model["desc"])
    t = learned_ref.rjl_atom_energies(pos, box, idx, par)
    v0 = learned_ref.net_vector(model)

    ec = learned_ref.pair_row_energies(pos, box, idx, model)
    fc = learned_ref.pair_forces(pos, box, idx, model, len(pos))

    def loss(v):
        return learned_ref.training_loss(learned_ref.with_net_vector(model, v), G, J, t, f_ref, e_core=ec, f_core=fc)

    E, _ = learned_ref.energies_and_dEdG(G, model)
    assert loss32[0] == pytest.approx(((E + ec - t) ** 2).sum(), rel=2e-3)
    blocks = {"W1": (0, 3072), "b1": (3072, 3136), "W2": (3136, 7232), "b2": (7232, 7296), "w3": (7296, 7360),
              "b3": (7360, 7361), "all": (0, learned_ref.NET_FLOATS)}
    rng = np.random.default_rng(7)
    h = 1e-5
    report = {}
    for name, (a, b) in blocks.items():
        for _ in range(3 if b - a > 1 else 1):
            dvec = np.zeros(learned_ref.NET_FLOATS)
            dvec[a:b] = rng.standard_normal(b - a)
            dvec /= np.linalg.norm(dvec)
            fd = (loss(v0 + h * dvec) - loss(v0 - h * dvec)) / (2 * h)
            gn = np.abs(np.concatenate([g32[0][a:b], [fd]])).max()
            e32 = abs(float(g32[0] @ dvec) - fd)
            etc = abs(float(gtc[0] @ dvec) - fd)
            report.setdefault(name, []).append((fd, e32, etc))
            assert e32 <= 2e-3 * (abs(fd) + 1e-2 * gn), (name, fd, float(g32[0] @ dvec))
            assert etc <= 6e-2 * (abs(fd) + 1e-2 * gn), (name, fd, float(gtc[0] @ dvec))
    print("loss gradient along directions (fd, |fp32 - fd|, |tc - fd|):", report)
