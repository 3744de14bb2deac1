"""The library's output files and output-unit text against records derived from
the Fortran WRITE statements (tests/helpers/fortran_records.py), which is
written independently of the library's formatter: log records, output blocks,
the settings echo, the closing record, snapshots and trajectory frames, in
both arithmetic forms and on a system with a Nose-Hoover chain."""
import os

import pytest

import pfmds_gb300 as pf
from pfmds_gb300 import configs
from tests.helpers import fortran_records as fr
from tests.helpers.record_check import Expect

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("form", ["plain", "precision"])
def test_library_records(tmp_path, built, monkeypatch, form):
    d = str(tmp_path)
    configs.lj_gas(d, n_a=150, n_b=150, box=24.0, log_period=5, period_traj=10,
                   integrators=[("nvt", 0.5, 20, 20, 5), ("nve", 0.5, 20, 15, 5)])
    monkeypatch.chdir(d)
    out_path = os.path.join(d, "out.txt")
    fd = os.open(out_path, os.O_WRONLY | os.O_CREAT | os.O_TRUNC, 0o644)
    try:
        e = Expect(d)
        s = pf.Simulation(d, form=form, out_period=10, write_files=True, out_fd=fd, async_io=False)
        for step in range(0, 41):
            s.advance(1)
            e.sample(s, step, 10)
        s.finish()
        en = s.energies()
        closing = fr.closing_record("", 40, s.sim_time, en["pe"] + en["ke"], en["pe"], en["ke"],
                                    en["temperature"], en["inter"])
        s.close()
    finally:
        os.close(fd)
    e.check_log(os.path.join(d, "md_run.log"))
    e.check_files(d)
    with open(out_path) as f:
        text = f.read()
    e.check_out(text)
    with open(os.path.join(d, "md_run.log")) as f:
        assert f.read().rstrip("\n").split("\n")[-1] == closing
    assert closing in text.split("\n")
