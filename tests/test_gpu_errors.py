"""Error paths of the CUDA library, each raised on the device as a status word and
mapped to the reference's message; none faults the GPU.  The oracle raises the same
code on the same input."""
import numpy as np
import pytest

import pfmds_gb300 as pf
from pfmds_gb300 import configs
from oracle.pyoracle import Oracle, OracleError

pytestmark = pytest.mark.gpu
FORMS = ["plain", "precision"]


@pytest.mark.parametrize("form", FORMS)
def test_list_overflow(tmp_path, built, form):
    # 'error: too many neighbours' (md_neighbours.f90:80)
    configs.lj_gas(str(tmp_path), n_a=100, n_b=100, box=20.0, nmax=5)
    with pytest.raises(OracleError) as eo:
        Oracle(str(tmp_path)).step()
    s = pf.Simulation(str(tmp_path), form=form)
    with pytest.raises(pf.PfmdError) as ei:
        s.advance(1)
    assert ei.value.code == pf.PFMD_E_NLIST_OVERFLOW == eo.value.code
    assert "too many neighbours" in str(ei.value)


@pytest.mark.parametrize("form", FORMS)
def test_out_of_cell(tmp_path, built, form):
    # check_positions (md_general.f90:342-364)
    configs.lj_gas(str(tmp_path), n_a=10, n_b=10, box=20.0, min_sep=3.0)
    s = pf.Simulation(str(tmp_path), form=form)
    p, v, f = s.state()
    p[3, 1] = 25.0
    s.set_state(p)
    with pytest.raises(pf.PfmdError) as ei:
        s.advance(1)
    assert ei.value.code == pf.PFMD_E_OUT_OF_CELL
    assert "particle out of cell" in str(ei.value)


@pytest.mark.parametrize("form", FORMS)
def test_out_of_cell_after_drift(tmp_path, built, form):
    # an atom that moves more than one box length in one nve step: the single
    # shift (md_integrators.f90:20-24) leaves it outside and the next step stops
    configs.lj_gas(str(tmp_path), n_a=10, n_b=10, box=20.0, min_sep=3.0,
                   integrators=[("nve", 0.5, 100, 10 ** 8, 10)])
    o = Oracle(str(tmp_path))
    s = pf.Simulation(str(tmp_path), form=form)
    p, v, f = s.state()
    v[5, 0] = 100.0  # A/fs: 50 A in one 0.5 fs step, more than one 20 A box
    o.set_state(vel=v)
    s.set_state(vel=v)
    with pytest.raises(OracleError) as eo:
        o.run(4)
    with pytest.raises(pf.PfmdError) as ei:
        s.advance(4)
    assert ei.value.code == pf.PFMD_E_OUT_OF_CELL == eo.value.code
    assert s.md_step == o.md_step


@pytest.mark.parametrize("form", FORMS)
def test_graphene_nearest_neighbour_count(tmp_path, built, form):
    # find_gr_nearest_neighbors needs exactly 3 (graphenenorm.f90:26,30): lift one
    # carbon atom out of the sheet so that its neighbours see only two
    configs.gr_on_cu(str(tmp_path), n_gx=6, n_gy=4, n_cx=6, n_cy=3, layers=3, steps=20)
    o = Oracle(str(tmp_path))
    s = pf.Simulation(str(tmp_path), form=form)
    p, v, f = s.state()
    p[0, 2] += 4.0
    o.set_state(p)
    s.set_state(p)
    with pytest.raises(OracleError) as eo:
        o.step()
    with pytest.raises(pf.PfmdError) as ei:
        s.advance(1)
    assert ei.value.code == pf.PFMD_E_GR_NN == eo.value.code


def test_context_reports_state_after_error(tmp_path, built):
    configs.lj_gas(str(tmp_path), n_a=100, n_b=100, box=20.0, nmax=5)
    s = pf.Simulation(str(tmp_path), form="plain")
    with pytest.raises(pf.PfmdError):
        s.advance(1)
    # the context stays usable for reading back and is destroyed cleanly
    p, v, f = s.state()
    assert np.isfinite(p).all()
    s.close()
