"""The oracle's output files and output-unit text against records derived from
the Fortran WRITE statements (tests/helpers/fortran_records.py), which is
written independently of the C++ formatter the oracle and the library share.

Covers the log record '(A6,i9,7f24.6)' + f20.9 energies, the output block of
md_simulation.f90:211-229, the settings echo of md_simulation.f90:48-94, the
closing record '(A32,i9,5f20.9)', snapshot files '(7f27.16,A,A)' and
trajectory frames '(7f10.4,A,A)'."""
import os

import pytest

from pfmds_gb300 import configs
from oracle.pyoracle import Oracle
from tests.helpers import fortran_records as fr
from tests.helpers.record_check import Expect


@pytest.mark.parametrize("x,w,d,exp", [
    # hand-evaluated Fw.d fields
    (0.5, 24, 6, "                0.500000"),
    (-87.53056589483532, 24, 6, "              -87.530566"),
    (1e-7, 24, 6, "                0.000000"),
    (-1e-7, 24, 6, "               -0.000000"),
    (0.5, 3, 2, ".50"),
    (123456.0, 5, 1, "*****"),
    (39.95, 27, 16, "        39.9500000000000028"),  # 39.95 is 39.95000000000000284217... in binary
])
def test_fw_d(x, w, d, exp):
    assert fr.F(x, w, d) == exp


@pytest.mark.parametrize("x,w,d,exp", [
    (311.2829142496041, 21, 9, "      3.112829142E+02"),
    (1e-8, 16, 6, "    1.000000E-08"),
    (0.0, 16, 6, "    0.000000E+00"),
    (2.5e-150, 16, 6, "    2.500000-150"),
])
def test_esw_d(x, w, d, exp):
    assert fr.ES(x, w, d) == exp


def test_a_edit():
    assert fr.A("md_step_limit:", 32, 128) == "md_step_limit:" + " " * 18
    assert fr.A("nve", 6) == "   nve"
    assert fr.A("nve", 6, 32) == "nve   "
    assert fr.A("CU_fixed", 12, 32) == "CU_fixed    "
    assert fr.list_int(4000) == "        4000"


def _run_oracle(d, steps, out_period):
    e = Expect(d)
    o = Oracle(d, out_period=out_period, threads=1, write_files=True)
    o.step()
    e.sample(o, 0, out_period)
    for s in range(1, steps + 1):
        o.step()
        e.sample(o, s, out_period)
    o.finish()
    return e, o


def test_oracle_records(tmp_path, monkeypatch):
    d = str(tmp_path)
    configs.lj_gas(d, n_a=150, n_b=150, box=24.0, log_period=5, period_traj=10,
                   integrators=[("nvt", 0.5, 20, 20, 5), ("nve", 0.5, 20, 15, 5)])
    monkeypatch.chdir(d)
    e, o = _run_oracle(d, 40, 10)
    e.check_log(os.path.join(d, "md_run.log"))
    e.check_files(d)
    e.check_out(o.output())
    # the closing record follows the last log record in the log file
    with open(os.path.join(d, "md_run.log")) as f:
        last = f.read().rstrip("\n").split("\n")[-1]
    en = o.energies()
    assert last == fr.closing_record("", 40, o.sim_time, en["pe"] + en["ke"], en["pe"], en["ke"],
                                     en["temperature"], en["inter"])
