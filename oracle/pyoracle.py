"""ctypes wrapper of the CPU oracle (liboracle.so) -- TEST INFRASTRUCTURE ONLY.

The oracle is a C++ FP64 restatement of PFMDS's md() hot path (see oracle.cpp);
parity against the Fortran reference itself is unpinned because no Fortran
compiler is available.  Tests, the smoke entry point and the benchmark's CPU
baseline use this module; the product never does.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

_ERR = {0: "ok", 1: "PFMD_E_NLIST_OVERFLOW", 2: "PFMD_E_OUT_OF_CELL", 3: "PFMD_E_GR_NN",
        4: "PFMD_E_PARAM", 5: "PFMD_E_CUDA", 6: "PFMD_E_TIMEOUT", 7: "PFMD_E_IO"}


class OracleError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{_ERR.get(code, code)}: {msg}")
        self.code = code


def lib():
    global _LIB
    if _LIB is None:
        from . import build_oracle  # noqa: F401  (package-relative when imported as oracle.pyoracle)
        path = build_oracle.build()
        L = C.CDLL(path)
        dp, ip, vp = C.POINTER(C.c_double), C.POINTER(C.c_int), C.c_void_p
        L.orc_create.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.c_int,
                                 C.c_int, C.POINTER(vp)]
        L.orc_step.argtypes = [vp, ip]
        L.orc_run.argtypes = [vp, C.c_longlong, ip]
        L.orc_finish.argtypes = [vp]
        L.orc_destroy.argtypes = [vp]
        L.orc_md_step.argtypes = [vp]
        L.orc_md_step.restype = C.c_longlong
        L.orc_natoms.argtypes = [vp]
        L.orc_get_state.argtypes = [vp, dp, dp, dp]
        L.orc_set_state.argtypes = [vp, dp, dp]
        L.orc_sim_time.argtypes = [vp]
        L.orc_sim_time.restype = C.c_double
        L.orc_ninteractions.argtypes = [vp]
        L.orc_nl_shape.argtypes = [vp, C.c_int, C.c_int, ip, ip]
        L.orc_get_nl.argtypes = [vp, C.c_int, C.c_int, ip, ip, ip, ip, dp]
        L.orc_get_gr_norm.argtypes = [vp, C.c_int, dp]
        L.orc_energies.argtypes = [vp, dp, dp, dp, dp, dp, dp]
        L.orc_eval.argtypes = [vp, C.c_int, dp]
        L.orc_errmsg.argtypes = [vp]
        L.orc_errmsg.restype = C.c_char_p
        L.orc_output.argtypes = [vp]
        L.orc_output.restype = C.c_char_p
        L.orc_run_md_simulation.argtypes = [C.c_int, C.POINTER(C.c_char_p)]
        for f in ("orc_f_cut_cos", "orc_df_cut_cos", "orc_f_cut_poly"):
            getattr(L, f).argtypes = [C.c_double] * 3
            getattr(L, f).restype = C.c_double
        L.orc_f_dfr_cut.argtypes = [C.c_double] * 3 + [dp, dp]
        L.orc_find_distance.argtypes = [dp, dp, dp, dp, dp]
        _LIB = L
    return _LIB


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


class Oracle:
    """One md() run of the oracle: set-up on construction, then step()/run()."""

    def __init__(self, input_path, settings="md_run_settings.txt", prefix="", out_period=1,
                 threads=0, seed=1, write_files=False):
        L = lib()
        self._h = C.c_void_p()
        ip = input_path if input_path.endswith("/") or not input_path else input_path + "/"
        rc = L.orc_create(ip.encode(), settings.encode(), prefix.encode(), out_period, threads,
                          seed, 1 if write_files else 0, C.byref(self._h))
        self._check(rc)
        self.finished = False

    def _check(self, rc):
        if rc:
            raise OracleError(rc, lib().orc_errmsg(self._h).decode())

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_destroy(self._h)
            self._h = None

    def step(self):
        f = C.c_int(0)
        self._check(lib().orc_step(self._h, C.byref(f)))
        self.finished = bool(f.value)
        return self.finished

    def run(self, n):
        f = C.c_int(0)
        self._check(lib().orc_run(self._h, n, C.byref(f)))
        self.finished = bool(f.value)
        return self.finished

    def finish(self):
        self._check(lib().orc_finish(self._h))

    @property
    def md_step(self):
        return lib().orc_md_step(self._h)

    @property
    def natoms(self):
        return lib().orc_natoms(self._h)

    @property
    def sim_time(self):
        return lib().orc_sim_time(self._h)

    def state(self):
        n = self.natoms
        p, v, f = (np.zeros((n, 3)) for _ in range(3))
        lib().orc_get_state(self._h, _dp(p), _dp(v), _dp(f))
        return p, v, f

    def set_state(self, pos=None, vel=None):
        p = None if pos is None else np.ascontiguousarray(pos, dtype=np.float64)
        v = None if vel is None else np.ascontiguousarray(vel, dtype=np.float64)
        lib().orc_set_state(self._h, None if p is None else _dp(p), None if v is None else _dp(v))

    @property
    def n_interactions(self):
        return lib().orc_ninteractions(self._h)

    def nlist(self, inter, lst):
        n, m = C.c_int(), C.c_int()
        self._check(lib().orc_nl_shape(self._h, inter, lst, C.byref(n), C.byref(m)))
        n, m = n.value, m.value
        nnum = np.zeros(n, np.int32)
        less = np.zeros(n, np.int32)
        pidx = np.zeros(n, np.int32)
        nl = np.zeros((n, m), np.int32)
        r = np.zeros((n, m))
        self._check(lib().orc_get_nl(self._h, inter, lst, _ip(nnum), _ip(less), _ip(pidx), _ip(nl), _dp(r)))
        return dict(nnum=nnum, lessnnum=less, pidx=pidx, nlist=nl, moddr=r)

    def gr_norm(self, inter, n_rows):
        g = np.zeros((n_rows, 3))
        self._check(lib().orc_get_gr_norm(self._h, inter, _dp(g)))
        return g

    def energies(self):
        e = np.zeros(max(1, self.n_interactions))
        vals = [C.c_double() for _ in range(5)]
        lib().orc_energies(self._h, _dp(e), *[C.byref(v) for v in vals])
        pe, ke, t, enhc, econs = (v.value for v in vals)
        return dict(inter=e[:self.n_interactions].copy(), pe=pe, ke=ke, temperature=t, nhc=enhc,
                    conserved=econs)

    def eval(self, rebuild=True):
        e = np.zeros(max(1, self.n_interactions))
        self._check(lib().orc_eval(self._h, 1 if rebuild else 0, _dp(e)))
        return e[:self.n_interactions].copy()

    def output(self):
        return lib().orc_output(self._h).decode()


def run_md_simulation(args):
    """Run the oracle's run_md_simulation command line in-process."""
    L = lib()
    argv = (C.c_char_p * (len(args) + 1))(*([b"oracle_md"] + [a.encode() for a in args]))
    return L.orc_run_md_simulation(len(args) + 1, argv)


def f_cut_cos(r, R1, R2):
    return lib().orc_f_cut_cos(r, R1, R2)


def df_cut_cos(r, R1, R2):
    return lib().orc_df_cut_cos(r, R1, R2)


def f_cut_poly(r, R1, R2):
    return lib().orc_f_cut_poly(r, R1, R2)


def f_dfr_cut(r, R1, R2):
    f, d = C.c_double(), C.c_double()
    lib().orc_f_dfr_cut(r, R1, R2, C.byref(f), C.byref(d))
    return f.value, d.value


def find_distance(v1, v2, box):
    v1 = np.ascontiguousarray(v1, float)
    v2 = np.ascontiguousarray(v2, float)
    b = np.ascontiguousarray(box, float)
    dr = np.zeros(3)
    dr2 = C.c_double()
    lib().orc_find_distance(_dp(v1), _dp(v2), _dp(b), _dp(dr), C.byref(dr2))
    return dr, dr2.value
