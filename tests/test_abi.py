"""The C ABI library without a GPU: it loads, exports every entry point that
include/pfmd.h declares, reads the reference's input files (errors mapped to the
reference's messages) and fails loudly when no device exists."""
import ctypes as C
import os
import re

import pytest

import pfmds_gb300 as pf
from pfmds_gb300 import configs
from oracle.pyoracle import Oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    text = open(os.path.join(ROOT, "include", "pfmd.h")).read()
    return sorted(set(re.findall(r"\b(pfmd_[a-z_0-9]+)\s*\(", text)))


def test_header_and_python_mirror_agree(built):
    assert declared() == sorted(pf.EXPORTS)


def test_library_exports_every_declared_symbol(built):
    L = pf.load()
    for name in declared():
        assert hasattr(L, name), name


def test_library_and_executable_exist(built):
    assert os.path.exists(pf.LIB_PATH)
    assert os.access(pf.EXE_PATH, os.X_OK)


def _no_gpu():
    try:
        import torch
        return not torch.cuda.is_available()
    except ImportError:
        return True


def _create(d, **kw):
    """pfmd_create_from_files with the output unit on a pipe; returns (rc, text, msg)."""
    L = pf.load()
    r, w = os.pipe()
    o = pf.default_options(out_fd=w, **kw)
    h = C.c_void_p()
    rc = L.pfmd_create_from_files((d + "/").encode(), b"md_run_settings.txt", C.byref(o), C.byref(h))
    os.close(w)
    text = b""
    while True:
        chunk = os.read(r, 1 << 16)
        if not chunk:
            break
        text += chunk
    os.close(r)
    msg = L.pfmd_errmsg(h).decode()
    L.pfmd_destroy(h)
    return rc, text.decode(), msg


@pytest.mark.skipif(not _no_gpu(), reason="checks the no-device path")
def test_no_device_fails_loudly_after_reading_inputs(tmp_path, built):
    configs.lj_gas(str(tmp_path), n_a=20, n_b=20, box=20.0)
    rc, text, msg = _create(str(tmp_path))
    assert rc == pf.PFMD_E_CUDA and "no CUDA device" in msg
    # the set-up echo is identical to the oracle's (md_simulation.f90:48-93)
    o = Oracle(str(tmp_path))
    echo = o.output().split("PREPARATIONS TIME")[0]
    assert text == echo[: len(text)] and len(text) > 0
    assert "settings_filename: md_run_settings.txt" in text
    assert text.count("\n") == echo.count("\n")


def test_parse_errors(tmp_path, built):
    configs.lj_gas(str(tmp_path), n_a=20, n_b=20, box=20.0)
    s = open(tmp_path / "md_run_settings.txt").read()
    open(tmp_path / "md_run_settings.txt", "w").write(s.replace("lj1g\tparameters_LJ_B-B", "lj9\tparameters_LJ_B-B"))
    rc, text, msg = _create(str(tmp_path))
    assert rc == pf.PFMD_E_PARAM and "unknown interaction name" in msg
    os.remove(tmp_path / "AB.xyz")
    rc, text, msg = _create(str(tmp_path))
    assert rc == pf.PFMD_E_IO and "AB.xyz" in msg
    rc, text, msg = _create(str(tmp_path / "missing"))
    assert rc == pf.PFMD_E_IO


def test_wrong_nhc_parameters_message(tmp_path, built):
    configs.lj_gas(str(tmp_path), n_a=20, n_b=20, box=20.0)
    s = open(tmp_path / "md_run_settings.txt").read().replace("1\t100\t3\t", "1\t-100\t3\t")
    open(tmp_path / "md_run_settings.txt", "w").write(s)
    rc, text, msg = _create(str(tmp_path))
    assert rc == pf.PFMD_E_PARAM and msg == "error: wrong nhc parameters"


def test_strerror_names(built):
    assert pf.strerror(pf.PFMD_E_NLIST_OVERFLOW) == "PFMD_E_NLIST_OVERFLOW"
    assert pf.strerror(pf.PFMD_E_GR_NN) == "PFMD_E_GR_NN"


def test_array_pointer_arguments():
    """The per-step calls pass arrays as void* through the buffer protocol, and
    by address when the array is read-only: both name the array's first double."""
    import numpy as np
    libc = C.CDLL(None)
    libc.memcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t]
    libc.memcpy.restype = C.c_void_p
    src = np.arange(6.0)
    ro = src.copy()
    ro.flags.writeable = False
    for a in (src, ro):
        dst = np.zeros(6)
        libc.memcpy(pf._addr(dst), pf._addr(a), 48)
        assert np.array_equal(dst, a)
