"""Skin-triggered list rebuilds of the precision form: a list keeps its rows at an
update step while no atom moved too far, every pair within the interaction's
cut-off stays in it, and the run follows the one rebuilt at every update step."""
import numpy as np
import pytest

import pfmds_gb300 as pf
from pfmds_gb300 import configs

pytestmark = pytest.mark.gpu


def _pairs_within(p, box, rc):
    """Set of (i, j) atom pairs closer than rc (minimum image), i != j."""
    from scipy.spatial import cKDTree
    t = cKDTree(np.mod(p, box), boxsize=box)
    return {(i, j) for i, j in t.query_pairs(rc)} | {(j, i) for i, j in t.query_pairs(rc)}


def test_skin_lists_skip_rebuilds_and_stay_complete(tmp_path, built):
    configs.cu_slab(str(tmp_path), nx=8, ny=8, nz=6, steps=400, log_period=10, temperature=300.0)
    d = str(tmp_path)
    box = np.array([float(x) for x in (tmp_path / "cu_slab.xyz").read_text().splitlines()[1].split('"')[1].split()])[[0, 4, 8]]
    s = pf.Simulation(d, form="precision", out_period=10 ** 6)
    r = pf.Simulation(d, form="precision", out_period=10 ** 6, skin_lists=False)
    assert r.nlist_builds()[0] == -1
    for k in range(20):
        s.advance(10)
        r.advance(10)
        if k % 5 == 4:
            p = s.state()[0]
            lst = s.nlist(0, 0)
            have = {(int(lst["pidx"][i]), int(j)) for i in range(len(lst["nnum"]))
                    for j in lst["pidx"][lst["nlist"][i, :lst["nnum"][i]]]}
            need = _pairs_within(p, box, 5.0)  # rjl cut-off R2
            assert need <= have, len(need - have)
    b = s.nlist_builds()[0]
    assert 1 <= b < 20, b  # 21 update steps in 200 steps
    ps, _, fs = s.state()
    pr, _, fr = r.state()
    dd = np.abs(ps - pr)
    assert np.minimum(dd, box - dd).max() < 1e-4
    assert np.sqrt(((fs - fr) ** 2).mean()) / np.sqrt((fr ** 2).mean()) < 1e-3
    assert s.energies()["conserved"] == pytest.approx(r.energies()["conserved"], rel=1e-6)


def test_two_level_rebuild_holds_every_pair_within_the_list_radius(tmp_path, built):
    """A rebuild filters the rows of the wider outer list, built steps earlier at
    other positions: the result holds exactly the pairs within the list radius
    now (up to FP32 rounding at the radius)."""
    configs.cu_slab(str(tmp_path), nx=8, ny=8, nz=6, steps=400, log_period=10, temperature=600.0)
    d = str(tmp_path)
    box = np.array([float(x) for x in (tmp_path / "cu_slab.xyz").read_text().splitlines()[1].split('"')[1].split()])[[0, 4, 8]]
    s = pf.Simulation(d, form="precision", out_period=10 ** 6)
    s.advance(150)
    s.time_kernel("lists", reps=1)  # every list rebuilt at the current positions
    p = s.state()[0]
    lst = s.nlist(0, 0)
    have = {(int(lst["pidx"][i]), int(j)) for i in range(len(lst["nnum"]))
            for j in lst["pidx"][lst["nlist"][i, :lst["nnum"][i]]]}
    assert _pairs_within(p, box, 5.5 - 1e-3) <= have <= _pairs_within(p, box, 5.5 + 1e-3)
    s.close()


@pytest.mark.parametrize("graphs", [True, False])
def test_fused_kick_drift_is_bitwise_the_separate_one(tmp_path, built, graphs):
    """The force kernel that also runs the next step's kick and drift gives the
    same trajectory, bit for bit, as the separate kick-drift kernel, across list
    rebuilds, energy steps and segment ends."""
    configs.cu_slab(str(tmp_path), nx=8, ny=8, nz=6, steps=400, log_period=10, temperature=300.0)
    d = str(tmp_path)
    runs = []
    for fuse in (True, False):
        s = pf.Simulation(d, form="precision", out_period=10 ** 6, fuse_steps=fuse, use_graphs=graphs)
        energies = []
        for n in (7, 30, 1, 45):
            s.advance(n)
            e = s.energies()
            energies.append((e["ke"], e["pe"], e["conserved"]))
        runs.append(s.state() + (energies,))
        s.close()
    for a, b in zip(runs[0][:3], runs[1][:3]):
        assert np.array_equal(a, b)
    assert runs[0][3] == runs[1][3]
