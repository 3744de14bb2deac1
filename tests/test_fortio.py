"""Fortran edit-descriptor and list-directed I/O emulation (pfmds_gb300/csrc/fortio.h).

Expected strings follow the Fortran rules for Aw, Iw, Iw.m, Lw, Fw.d (leading zero
only when it fits, asterisks on overflow) and ESw.d (E+dd, or +ddd without the
letter for three-digit exponents), and gfortran's list-directed forms."""
import ctypes as C
import os
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    out = tmp_path_factory.mktemp("shim") / "libshim.so"
    subprocess.run(["g++", "-O1", "-std=c++17", "-shared", "-fPIC",
                    os.path.join(HERE, "helpers", "fortio_shim.cpp"), "-o", str(out)], check=True)
    L = C.CDLL(str(out))
    L.sh_to_real.restype = C.c_double
    L.sh_to_real.argtypes = [C.c_char_p]
    return L


def call(L, name, *args):
    buf = C.create_string_buffer(512)
    cargs = []
    for a in args:
        if isinstance(a, float):
            cargs.append(C.c_double(a))
        elif isinstance(a, str):
            cargs.append(a.encode())
        else:
            cargs.append(C.c_longlong(a) if name in ("sh_fmt_i", "sh_fmt_i0", "sh_list_int") and a is args[0]
                         else C.c_int(a))
    getattr(L, name)(*cargs, buf, 512)
    return buf.value.decode()


@pytest.mark.parametrize("x,w,d,exp", [
    (1.5, 24, 6, " " * 16 + "1.500000"),
    (0.0, 10, 2, "      0.00"),
    (-1.769128065752, 20, 9, " " * 8 + "-1.769128066"),
    (0.5, 10, 4, "    0.5000"),
    (-0.5, 10, 4, "   -0.5000"),
    (0.5, 4, 2, "0.50"),
    (0.5, 3, 2, ".50"),
    (-0.5, 3, 2, "***"),
    (1e10, 10, 2, "**********"),
    (-1e-12, 24, 6, " " * 15 + "-0.000000"),
    (60.0, 16, 6, "       60.000000"),
    (12.345678901234567, 27, 16, f"{12.345678901234567:27.16f}"),
])
def test_fmt_f(shim, x, w, d, exp):
    assert call(shim, "sh_fmt_f", x, w, d) == exp


@pytest.mark.parametrize("x,w,d,exp", [
    (1e-8, 16, 6, "    1.000000E-08"),
    (-224763.06126861525, 21, 9, "     -2.247630613E+05"),
    (0.0, 16, 6, "    0.000000E+00"),
    (1e-100, 12, 3, "   1.000-100"),
    (7.296673e-17, 16, 6, "    7.296673E-17"),
])
def test_fmt_es(shim, x, w, d, exp):
    assert call(shim, "sh_fmt_es", x, w, d) == exp


def test_integers_logicals_characters(shim):
    assert call(shim, "sh_fmt_i", 1000, 12) == "        1000"
    assert call(shim, "sh_fmt_i", 123456, 3) == "***"
    assert call(shim, "sh_fmt_i0", 100, 6, 6) == "000100"
    assert call(shim, "sh_fmt_i0", 3, 2, 2) == "03"
    assert call(shim, "sh_fmt_l", 1, 8) == "       T"
    # A6 with trim('nvt') right-justifies; A6 of a character(32) variable keeps its
    # leftmost 6 characters (the padding included)
    assert call(shim, "sh_fmt_a", "nvt", 6, -1) == "   nvt"
    assert call(shim, "sh_fmt_a", "nvt", 6, 32) == "nvt   "
    assert call(shim, "sh_fmt_a", "md_step_limit:", 32, 128) == "md_step_limit:" + " " * 18
    assert call(shim, "sh_fmt_a", "neib", 8, -1) == "    neib"


def test_list_directed_output(shim):
    # default INTEGER: 12 columns; REAL(8): 17 significant digits that read back exactly
    # (the blank layout around list-directed reals is processor dependent)
    assert call(shim, "sh_list_int", 8) == "           8"
    for v in (1.5, -1.0345396527657869e-3, 224763.06126861525, 0.0, 1e-300):
        s = call(shim, "sh_list_real", v)
        assert len(s) >= 25 and float(s.replace("E-", "e-").replace("E+", "e+")) == v


def test_list_directed_input(shim):
    assert call(shim, "sh_read_items", "md_step_limit:  1000  trailing\nnext", 2) == "md_step_limit:|1000"
    # a READ statement continues on the following records
    assert call(shim, "sh_read_items", "1 2\n3\n4", 3) == "1|2|3"
    # commas, quotes, a null value and the slash terminator
    assert call(shim, "sh_read_items", "'a b', 5,, 7", 4) == "a b|5|<unset>|7"
    assert call(shim, "sh_read_items", "1 2 / 3", 3) == "1|2|<unset>"
    assert call(shim, "sh_read_items", "Lattice=\" 16.0 0.0", 3) == "Lattice=\"|16.0|0.0"


@pytest.mark.parametrize("s,v", [("1.e-8", 1e-8), ("1d-8", 1e-8), ("1.0D+00", 1.0), ("+5", 5.0), (".5", 0.5),
                                 ("1.5-3", 1.5e-3), ("2.278", 2.278), ("-0.25e1", -2.5)])
def test_real_input(shim, s, v):
    assert shim.sh_to_real(s.encode()) == v


@pytest.mark.parametrize("x,w,d", [(0.5, 27, 16), (-0.5, 27, 16), (0.25, 3, 2), (-0.25, 4, 2), (-0.25, 3, 2),
                                   (123.456, 10, 4), (-1e9, 10, 4), (0.0, 10, 4), (-0.0, 27, 16),
                                   (1.0 / 3.0, 27, 16), (99999.99999, 10, 4), (float("nan"), 10, 4),
                                   (float("-inf"), 27, 16)])
def test_xyz_writer_f_matches_fmt_f(shim, x, w, d):
    assert call(shim, "sh_put_f", x, w, d) == call(shim, "sh_fmt_f", x, w, d)


@pytest.mark.parametrize("n", [5, 20000])
def test_threaded_snapshot_text_matches_line_by_line(shim, n):
    shim.sh_snapshot_matches.argtypes = [C.c_int, C.c_double]
    assert shim.sh_snapshot_matches(n, 0.731) == 1
