"""The FP64 restatement of the learned form's training loss (oracle/learned_ref.py)
checked against itself by central differences: the descriptor Jacobian against
differences of the descriptors, dE/dG against differences of the network, and
the rjl per-atom energies against the oracle's interaction energy.  The GPU
tests compare the library's loss gradient with this restatement."""
import numpy as np
import pytest

from oracle import learned_ref as lr
from pfmds_gb300 import configs
from oracle.pyoracle import Oracle


def _desc(rc_rad=5.0, rc_ang=3.0):
    return dict(rc_rad=rc_rad, rc_ang=rc_ang, rs=np.linspace(0.8, rc_rad - 0.4, lr.NR),
                eta_r=np.full(lr.NR, 4.0), eta_a=np.array([0.0, 0.2]), zeta=np.array([1.0, 2.0, 4.0, 8.0]),
                lam=np.array([1.0, -1.0]), mean=np.zeros(lr.NG), inv_std=np.ones(lr.NG))


def _cluster(n=14, seed=3):
    rng = np.random.default_rng(seed)
    box = np.array([12.0, 12.0, 12.0])
    pos = 6.0 + rng.uniform(-2.6, 2.6, size=(n, 3))
    return pos, box


def _model(seed=5):
    rng = np.random.default_rng(seed)
    net = dict(W1=rng.normal(0, 0.2, (lr.NH, lr.NG)), b1=rng.normal(0, 0.1, lr.NH),
               W2=rng.normal(0, 0.15, (lr.NH, lr.NH)), b2=rng.normal(0, 0.1, lr.NH),
               w3=rng.normal(0, 0.2, lr.NH), b3=0.3)
    d = _desc()
    d["mean"] = rng.normal(0, 0.5, lr.NG)
    d["inv_std"] = rng.uniform(0.5, 2.0, lr.NG)
    return dict(kind=1, desc=d, net=net)


def test_descriptor_jacobian_against_differences():
    pos, box = _cluster()
    idx = np.arange(len(pos))
    d = _desc()
    G, J = lr.descriptors_jacobian(pos, box, idx, d)
    np.testing.assert_allclose(G, lr.descriptors(pos, box, idx, d), rtol=1e-12, atol=1e-12)
    h = 1e-5
    for a in (0, 5, 9):
        for c in range(3):
            pp, pm = pos.copy(), pos.copy()
            pp[a, c] += h
            pm[a, c] -= h
            fd = (lr.descriptors(pp, box, idx, d) - lr.descriptors(pm, box, idx, d)) / (2 * h)
            np.testing.assert_allclose(J[:, :, a, c], fd, rtol=1e-6, atol=1e-7)


def test_network_gradient_against_differences():
    m = _model()
    rng = np.random.default_rng(1)
    G = rng.uniform(0.0, 3.0, (6, lr.NG))
    E, g = lr.energies_and_dEdG(G, m)
    np.testing.assert_allclose(E, lr.atom_energies(G, m), rtol=1e-13)
    h = 1e-6
    for f in (0, 17, 40, 47):
        Gp, Gm = G.copy(), G.copy()
        Gp[:, f] += h
        Gm[:, f] -= h
        fd = (lr.atom_energies(Gp, m) - lr.atom_energies(Gm, m)) / (2 * h)
        np.testing.assert_allclose(g[:, f], fd, rtol=1e-6, atol=1e-9)


def test_net_vector_round_trip():
    m = _model()
    v = lr.net_vector(m)
    assert v.shape == (lr.NET_FLOATS,)
    m2 = lr.with_net_vector(m, v)
    for k in m["net"]:
        np.testing.assert_array_equal(np.asarray(m2["net"][k]), np.asarray(m["net"][k]))


def test_rjl_atom_energies_sum_to_the_oracle(tmp_path):
    configs.cu_slab(str(tmp_path), nx=3, ny=3, nz=3, steps=10, log_period=1)
    o = Oracle(str(tmp_path), out_period=1, threads=1)
    o.step()
    pos = o.state()[0]
    lines = open(tmp_path / "cu_slab.xyz").read().splitlines()
    box = np.array([float(x) for x in lines[1].split('"')[1].split()])[[0, 4, 8]]
    par = [float(x) for x in open(tmp_path / "parameters_RJL_Cu.txt").read().split()]
    e = lr.rjl_atom_energies(pos, box, np.arange(len(pos)), par)
    assert e.sum() == pytest.approx(o.energies()["inter"][0], rel=1e-12)


def test_pair_terms_forces_are_their_gradient():
    # a cluster with pairs inside both walls and within the baseline's range:
    # the wall and baseline forces against central differences of their energy
    rng = np.random.default_rng(3)
    pos = rng.uniform(0.0, 5.0, size=(14, 3))
    box = np.array([30.0, 30.0, 30.0])
    idx = np.arange(14)
    m = _model()
    for kind, base in ((0, 0.0), (1, 0.0855)):
        mk = dict(m, kind=kind, desc=dict(m["desc"], bA=base, bp=10.96, br0=2.556, bR1=4.0, bR2=5.0))
        f = lr.pair_forces(pos, box, idx, mk, 14)
        assert np.abs(f).max() > 0.0
        h = 1e-6
        for a in (0, 5, 13):
            for c in range(3):
                pp, pm = pos.copy(), pos.copy()
                pp[a, c] += h
                pm[a, c] -= h
                fd = -(lr.core_energy(pp, box, idx, mk) - lr.core_energy(pm, box, idx, mk)) / (2 * h)
                assert f[a, c] == pytest.approx(fd, rel=1e-6, abs=1e-6)
    two = np.array([[1.0, 1.0, 1.0], [2.8, 1.0, 1.0]])
    mk = dict(m, kind=1, desc=dict(m["desc"], bA=0.0855, bp=10.96, br0=2.556, bR1=4.0, bR2=5.0))
    expect = lr.CORE_K * (lr.CORE_R[1] - 1.8) ** 2 + 2 * 0.0855 * np.exp(-10.96 * (1.8 / 2.556 - 1.0))
    assert lr.core_energy(two, box, np.arange(2), mk) == pytest.approx(expect)
