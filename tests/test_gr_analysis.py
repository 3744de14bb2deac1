"""Graphene-on-copper analysis (graphene_on_surface_analysis.f90:8-29,
position_analysis md_general.f90:400-421): the library's host implementation
against the numpy restatement, directly and through run_gr_analysis."""
import numpy as np
import pytest

import pfmds_gb300 as pf
from pfmds_gb300 import configs
from tests.helpers import moire_fit_ref as ref


def _system(d, name, seed, height):
    configs.gr_on_cu(str(d), n_gx=7, n_gy=5, n_cx=6, n_cy=3, layers=3, seed=seed, height=height,
                     xyz_name=name, settings_name=name + "_settings.txt")
    return d / name


def test_analysis_matches_restatement(tmp_path, built):
    p = _system(tmp_path, "a.xyz", 3, 3.1)
    for z in (0.0, 6.0, 9.5):
        a1, a2 = pf.gr_on_cu_analysis(p, z)
        r1, r2 = ref.gr_on_cu_analysis(str(p), z)
        assert np.allclose(a1, r1, rtol=0, atol=1e-12, equal_nan=True)
        assert np.allclose(a2, r2, rtol=0, atol=1e-12, equal_nan=True)
    # above every atom: no atom counted, so the mean is 0/0 as in the reference
    a1, a2 = pf.gr_on_cu_analysis(p, 500.0)
    assert np.isnan(a1[0]) and a1[1] == 1000.0 and a1[2] == 500.0


def test_run_gr_analysis_writes_the_list(tmp_path, built):
    names = ["a.xyz", "b.xyz"]
    for k, nm in enumerate(names):
        _system(tmp_path, nm, 5 + k, 3.0 + 0.3 * k)
    (tmp_path / "filelist.txt").write_text("2\n" + "\n".join(names) + "\n")
    assert pf.run_gr_analysis(["-path", f"{tmp_path}/", "-fl", "filelist.txt", "-o", "res.txt", "-z", "1.0"]) == 0
    rows = (tmp_path / "res.txt").read_text().splitlines()
    assert len(rows) == 2
    for nm, row in zip(names, rows):
        t = row.split()
        assert t[0] == nm
        r1, r2 = ref.gr_on_cu_analysis(str(tmp_path / nm), 1.0)
        assert np.allclose([float(v) for v in t[1:]], r1 - r2[0], rtol=0, atol=1e-12)


def test_missing_file_is_an_io_error(tmp_path, built):
    with pytest.raises(pf.PfmdError) as ei:
        pf.gr_on_cu_analysis(tmp_path / "nope.xyz", 0.0)
    assert ei.value.code == pf.PFMD_E_IO
