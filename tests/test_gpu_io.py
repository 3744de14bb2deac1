"""Snapshot and trajectory files written by the background writer (the default)
are the files written at each event, byte for byte, and are complete when
finish() returns; a write error surfaces as PFMD_E_IO."""
import os

import pytest

import pfmds_gb300 as pf
from pfmds_gb300 import configs

pytestmark = pytest.mark.gpu


def _case(d, snap=3, traj=2):
    configs.cu_slab(str(d), nx=6, ny=6, nz=4, steps=40, log_period=5)
    sf = d / "md_run_settings.txt"
    t = sf.read_text().replace("period_traj:\t\t\t\t100000000", f"period_traj:\t\t\t\t{traj}")
    sf.write_text(t.replace("100000000", str(snap)))
    return str(d)


def test_background_files_equal_files_written_at_the_event(tmp_path, built):
    d = _case(tmp_path)
    for mode in (0, 1):
        s = pf.Simulation(d, form="plain", out_period=10 ** 6, write_files=True, prefix=f"{d}/m{mode}_",
                          async_io=bool(mode))
        s.advance(10 ** 6)
        s.finish()
        s.close()
    a = sorted(f for f in os.listdir(d) if f.startswith("m0_"))
    b = sorted(f for f in os.listdir(d) if f.startswith("m1_"))
    assert [f[3:] for f in a] == [f[3:] for f in b]
    assert sum(f.startswith("m0_snapshot_") for f in a) == 13 and "m0_traj_02.xyz" in a
    for x, y in zip(a, b):
        tx, ty = (tmp_path / x).read_bytes(), (tmp_path / y).read_bytes()
        if x.endswith(".log"):  # the closing record starts with the prefix
            tx, ty = tx.splitlines()[:-1], ty.splitlines()[:-1]
        assert tx == ty, x


def test_write_error_is_reported(tmp_path, built):
    d = _case(tmp_path)
    os.mkdir(tmp_path / "x_snapshot_000009.xyz")  # a directory where a snapshot goes
    s = pf.Simulation(d, form="plain", out_period=10 ** 6, write_files=True, prefix=f"{d}/x_")
    with pytest.raises(pf.PfmdError) as ei:
        s.advance(10 ** 6)
        s.finish()
    assert ei.value.code == pf.PFMD_E_IO and "cannot open" in str(ei.value)
