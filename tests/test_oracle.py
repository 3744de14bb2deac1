"""The CPU oracle against known answers and physics invariants (CPU only).

The reference cannot be built here (Fortran, no compiler) and ships no fixtures,
so the oracle is pinned by: hand-derived values of the switch functions and the
minimum-image rule, two-atom energies restated independently in numpy from the
reference's formulas, finite-difference forces (the reference's own numerical
force uses central differences, md_interactions.f90:273-310), zero total force,
energy conservation under nve, the Nose-Hoover conserved quantity under nvt,
and the nvms exit.
"""
import math
import os

import numpy as np
import pytest

from pfmds_gb300 import configs
from oracle import pyoracle as po
from oracle.pyoracle import Oracle, OracleError

PI_T = 3.14159265358979


# ---------------------------------------------------------------- switches
def test_cosine_switch_known_values():
    R1, R2 = 4.5, 5.0
    assert po.f_cut_cos(4.0, R1, R2) == 1.0
    assert po.f_cut_cos(R1, R1, R2) == 1.0  # r < R1 is strict; cos(0) = 1
    assert po.f_cut_cos(4.75, R1, R2) == pytest.approx(0.5 * (1 + math.cos(PI_T / 2)), abs=1e-15)
    assert po.f_cut_cos(R2, R1, R2) == 0.0
    assert po.df_cut_cos(4.0, R1, R2) == 0.0
    # f'/r at the midpoint: -sin(pi/2) * pi / (R2-R1) / r / 2
    assert po.df_cut_cos(4.75, R1, R2) == pytest.approx(-PI_T / 0.5 / 4.75 / 2, rel=1e-14)
    assert po.df_cut_cos(5.0, R1, R2) == 0.0


def test_quintic_switch_and_missing_factor():
    R1, R2 = 6.5, 8.5  # R2 - R1 = 2 exposes the missing 1/(R2-R1) of f_dfr_cut
    assert po.f_cut_poly(7.5, R1, R2) == pytest.approx(0.5, abs=1e-15)
    f, dfr = po.f_dfr_cut(7.5, R1, R2)
    assert f == pytest.approx(0.5, abs=1e-15)
    # dfr = r x^2 (-30 + 60x - 30x^2) at x = 1/2: r * 0.25 * (-7.5), no 1/(R2-R1)
    assert dfr == pytest.approx(7.5 * 0.25 * -7.5, rel=1e-14)
    # clamped beyond the range; exactly zero at and past R2
    assert po.f_dfr_cut(9.0, R1, R2) == (0.0, 0.0)
    assert po.f_dfr_cut(1.0, R1, R2) == (1.0, 0.0)


def test_minimum_image_tie_rule():
    box = np.array([10.0, 10.0, 10.0])
    # dr = +h maps to -h, dr = -h stays -h (md_general.f90:434-436)
    dr, dr2 = po.find_distance([0, 0, 0], [5.0, 0, 0], box)
    assert dr[0] == -5.0
    dr, dr2 = po.find_distance([5.0, 0, 0], [0, 0, 0], box)
    assert dr[0] == -5.0
    dr, dr2 = po.find_distance([0.5, 9.5, 1.0], [9.5, 0.5, 8.0], box)
    assert np.allclose(dr, [-1.0, 1.0, -3.0]) and dr2 == pytest.approx(11.0)


# ---------------------------------------------------------------- two atoms
def _two_atoms(d, name, types, r, box=30.0, params=None, rlist=9.0):
    os.makedirs(d, exist_ok=True)
    pos = np.array([[10.0, 10.0, 10.0], [10.0 + r, 10.0, 10.0]])
    configs.write_xyz(os.path.join(d, "two.xyz"), (box, box, box), pos, np.zeros((2, 3)),
                      np.array([30.0, 30.0]), types)
    with open(os.path.join(d, "p.txt"), "w") as f:
        f.write(params)
    names = sorted(set(types))
    groups = [names, [names[0]], [names[-1]], []]
    g12 = (2, 3) if len(names) == 2 else (1, 1)
    lists = {"lj": [(g12[0], g12[1], 8, rlist, 10), (g12[1], g12[0], 8, rlist, 10)],
             "lj1g": [(1, 1, 8, rlist, 10)], "rjl": [(1, 1, 8, rlist, 10)]}[name]
    text = configs._settings_text(step_limit=1, xyz_name="two.xyz", types=names, groups=groups, all_moving=1,
                                  xyz_moving=1, z_moving=4, all_atoms=1, traj_group=1, period_traj=10 ** 8,
                                  integrators=[("nve", 1.0, 1, 10 ** 8, 1)], ms_de=1e-8, nhc=[], t0=0.0,
                                  interactions=[(name, "p.txt", lists)])
    with open(os.path.join(d, "md_run_settings.txt"), "w") as f:
        f.write(text)
    return d


@pytest.mark.parametrize("r", [3.0, 3.8, 6.9, 7.3])
def test_lj1g_pair_energy_and_force(tmp_path, r):
    eps, sig, R1, R2 = 0.0104, 3.40, 6.5, 7.5
    d = _two_atoms(str(tmp_path), "lj1g", ["A", "A"], r, params=f"{eps} {sig}\n{R1} {R2}\n")
    o = Oracle(d)
    e = o.eval(True)[0]
    c6, c12 = 4 * eps * sig ** 6, 4 * eps * sig ** 12
    x = min(max((r - R1) / (R2 - R1), 0.0), 1.0)
    f = 1 + x ** 3 * (-10 + 15 * x - 6 * x * x)
    u = r ** -6
    assert e == pytest.approx(u * (c12 * u - c6) * f, rel=1e-12)
    dfdr = x * x * (-30 + 60 * x - 30 * x * x) / (R2 - R1)  # exact derivative (R2-R1 = 1 here)
    dEdr = (-12 * c12 * u * u / r + 6 * c6 * u / r) * f + u * (c12 * u - c6) * dfdr
    p, v, frc = o.state()
    assert frc[1, 0] == pytest.approx(-dEdr, rel=1e-10, abs=1e-14)
    assert frc[0, 0] == pytest.approx(dEdr, rel=1e-10, abs=1e-14)


@pytest.mark.parametrize("r", [2.4, 3.6, 4.7, 5.2])
def test_rjl_dimer_energy(tmp_path, r):
    A0, xi, p_, q, r0, R1, R2 = 0.0855, 1.224, 10.96, 2.278, 2.556, 4.5, 5.0
    d = _two_atoms(str(tmp_path), "rjl", ["CU", "CU"], r, params=f"{A0} {xi} {p_} {q} {r0}\n{R1} {R2}\n",
                   rlist=5.5)
    e = Oracle(d).eval(True)[0]
    fc = 1.0 if r < R1 else (0.5 * (1 + math.cos(PI_T * (r - R1) / (R2 - R1))) if r < R2 else 0.0)
    per_atom = A0 * math.exp(-p_ * (r / r0 - 1)) * fc - xi * math.sqrt(math.exp(-2 * q * (r / r0 - 1)) * fc)
    assert e == pytest.approx(2 * per_atom, rel=1e-12, abs=1e-15)


# ---------------------------------------------------------------- gradients
def _fd_check(d, atoms, h=1e-5, tol=2e-5):
    o = Oracle(d, threads=1)
    o.eval(True)
    p, v, f = o.state()
    worst = 0.0
    for a in atoms:
        for k in range(3):
            pp = p.copy()
            pp[a, k] += h
            o.set_state(pp)
            ep = o.eval(False).sum()
            pm = p.copy()
            pm[a, k] -= h
            o.set_state(pm)
            em = o.eval(False).sum()
            g = -(ep - em) / (2 * h)
            worst = max(worst, abs(g - f[a, k]) / (abs(f[a, k]) + 1e-2))
    assert worst < tol, worst
    return f


def test_fd_lj_gas(tmp_path):
    configs.lj_gas(str(tmp_path), n_a=100, n_b=100, box=22.0)
    f = _fd_check(str(tmp_path), [0, 17, 99, 150, 199])
    assert np.abs(f.sum(0)).max() < 1e-12


def test_fd_rjl_slab(tmp_path):
    configs.cu_slab(str(tmp_path), nx=4, ny=4, nz=3)
    f = _fd_check(str(tmp_path), [0, 60, 100, 191])
    assert np.abs(f.sum(0)).max() < 1e-10


@pytest.mark.parametrize("coupling,simplified", [("morsec", False), ("ljc", False), ("morsec", True)])
def test_fd_graphene_on_cu(tmp_path, coupling, simplified):
    configs.gr_on_cu(str(tmp_path), n_gx=6, n_gy=4, n_cx=6, n_cy=3, layers=3, coupling=coupling,
                     simplified=simplified)
    # carbon atoms carry the tb bond order and the normal-derivative terms
    f = _fd_check(str(tmp_path), [0, 5, 40, 96, 130], h=2e-6, tol=5e-5)
    if not simplified:
        assert np.abs(f.sum(0)).max() < 1e-8


def test_lj1g_quirk_forces_inconsistent_when_switch_width_is_not_one(tmp_path):
    # f_dfr_cut lacks 1/(R2-R1) (cut_off_poly.f90:41); with R2-R1 = 2 the switch
    # region's forces are not -dE/dr.  Atoms 7.0 A apart sit inside it.
    d = _two_atoms(str(tmp_path), "lj1g", ["A", "A"], 7.0, params="0.0104 3.40\n6.5 8.5\n")
    o = Oracle(d)
    o.eval(True)
    p, v, f = o.state()
    h = 1e-5
    pp = p.copy()
    pp[1, 0] += h
    o.set_state(pp)
    ep = o.eval(True)[0]
    pm = p.copy()
    pm[1, 0] -= h
    o.set_state(pm)
    em = o.eval(True)[0]
    g = -(ep - em) / (2 * h)
    assert abs(g - f[1, 0]) > 1e-3 * abs(g)


# ---------------------------------------------------------------- dynamics
def test_nve_energy_conservation(tmp_path):
    configs.lj_gas(str(tmp_path), n_a=150, n_b=150, box=24.0, integrators=[("nve", 0.5, 400, 10 ** 8, 50)])
    o = Oracle(str(tmp_path), out_period=50, threads=2)
    o.step()
    e0 = o.energies()["conserved"]
    es = []
    while not o.run(50):
        es.append(o.energies()["conserved"])
    drift = max(abs(e - e0) for e in es) / 300
    assert drift < 2e-5  # eV per atom over 200 fs


def test_nvt_conserved_quantity_and_temperature(tmp_path):
    configs.lj_gas(str(tmp_path), n_a=150, n_b=150, box=24.0, temperature=100.0,
                   integrators=[("nvt", 0.5, 600, 10 ** 8, 50)])
    o = Oracle(str(tmp_path), out_period=50, threads=2)
    o.step()
    e0 = o.energies()["conserved"]
    while not o.run(50):
        e = o.energies()
        assert abs(e["conserved"] - e0) / 300 < 5e-5
    assert e["nhc"] != 0.0


def test_nvms_converges_and_exits(tmp_path):
    configs.cu_slab(str(tmp_path), nx=3, ny=3, nz=2, steps=5000, integrator="nvms", log_period=10)
    s = open(tmp_path / "md_run_settings.txt").read().replace("ms_de:\t\t\t\t\t\t1e-08", "ms_de:\t\t\t\t\t\t1e-07")
    open(tmp_path / "md_run_settings.txt", "w").write(s)
    o = Oracle(str(tmp_path), out_period=10 ** 6, threads=1)
    pe = []
    while not o.step():
        pe.append(o.energies()["pe"])
    assert o.md_step < 5001
    assert "potential energy diffrence is small enough" in o.output()
    assert pe[-1] < pe[0]


# ---------------------------------------------------------------- lists
def test_lists_match_brute_force_and_lessnnum(tmp_path):
    configs.lj_gas(str(tmp_path), n_a=120, n_b=80, box=20.0, rc_list=7.0)
    o = Oracle(str(tmp_path), threads=1)
    o.step()
    p, v, f = o.state()
    box = np.array([20.0] * 3)
    nl = o.nlist(1, 0)  # lj1g A-A: group 2 (A atoms, ascending)
    with open(os.path.join(tmp_path, "AB.xyz")) as fh:
        types = [ln.split()[-1] for ln in fh.read().splitlines()[2:]]
    a_idx = [i for i, t in enumerate(types) if t == "A"]
    for row, i in enumerate(a_idx):
        d = p[a_idx] - p[i]
        d -= box * np.round(d / box)
        r2 = (d ** 2).sum(1)
        expect = [k for k in range(len(a_idx)) if a_idx[k] != i and r2[k] < 49.0]
        got = list(nl["nlist"][row, :nl["nnum"][row]])
        assert got == expect
        assert nl["lessnnum"][row] == sum(1 for k in expect if a_idx[k] < i)


def test_overflow_and_out_of_cell_errors(tmp_path):
    configs.lj_gas(str(tmp_path), n_a=100, n_b=100, box=20.0, nmax=5)
    with pytest.raises(OracleError) as ei:
        Oracle(str(tmp_path)).step()
    assert ei.value.code == 1 and "too many neighbours" in str(ei.value)
    d2 = tmp_path / "oob"
    configs.lj_gas(str(d2), n_a=10, n_b=10, box=20.0, min_sep=3.0)
    o = Oracle(str(d2))
    p, v, f = o.state()
    p[3, 1] = 25.0
    o.set_state(p)
    with pytest.raises(OracleError) as ei:
        o.step()
    assert ei.value.code == 2
    assert "particle out of cell" in o.output()


def test_wrong_nhc_parameters(tmp_path):
    configs.lj_gas(str(tmp_path), n_a=10, n_b=10, box=20.0, min_sep=3.0)
    s = open(tmp_path / "md_run_settings.txt").read().replace("1\t100\t3\t", "1\t-100\t3\t")
    open(tmp_path / "md_run_settings.txt", "w").write(s)
    with pytest.raises(OracleError) as ei:
        Oracle(str(tmp_path))
    assert "wrong nhc parameters" in str(ei.value)
