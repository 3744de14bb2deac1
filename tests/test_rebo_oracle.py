"""rebosc in the oracle: its forces are the reference's central differences on a
third-order truncated list (calculate_forces_numerically,
md_interactions.f90:273-310).  They must equal central differences of the full
energy, which pins the truncation restatement."""
import numpy as np

from oracle.pyoracle import Oracle
from pfmds_gb300 import configs


def test_truncated_list_forces_are_the_full_energy_gradient(tmp_path, built):
    sf = configs.graphene_rebo(str(tmp_path), nx=8, ny=5, seed=3)
    o = Oracle(str(tmp_path), sf, write_files=False)
    e0 = o.eval(True)[0]
    assert -7.5 < e0 / o.natoms < -6.0  # eV per atom of a strained sheet
    p, _, f = o.state()
    assert np.abs(f.sum(0)).max() < 1e-5
    h = 1e-5
    for a in (0, 7, 33, 101):
        for k in range(3):
            pp = p.copy()
            pp[a, k] += h
            o.set_state(pp)
            ep = o.eval(True)[0]
            pp[a, k] -= 2 * h
            o.set_state(pp)
            em = o.eval(True)[0]
            assert abs(f[a, k] + (ep - em) / (2 * h)) < 1e-6, (a, k)
    o.set_state(p)
