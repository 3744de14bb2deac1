"""GB300 (sm_103a) implementation of PFMDS's MD force-and-integration hot path.

The compute path is the CUDA library built in-tree (pfmds_gb300/_build/libpfmd.so,
C ABI declared in include/pfmd.h).  This module is a thin ctypes mirror of that
ABI, named after the reference's md() and run_md_simulation: it loads the library
and fails loudly when it is missing; there is no CPU fallback.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libpfmd.so")
EXE_PATH = os.path.join(HERE, "_build", "run_md_simulation")

PFMD_OK = 0
PFMD_E_NLIST_OVERFLOW = 1
PFMD_E_OUT_OF_CELL = 2
PFMD_E_GR_NN = 3
PFMD_E_PARAM = 4
PFMD_E_CUDA = 5
PFMD_E_TIMEOUT = 6
PFMD_E_IO = 7
PFMD_E_STATE = 8
FORMS = {"plain": 0, "precision": 1}
NET_FLOATS = 7361  # floats per network of the learned form (PFMD_LEARNED_NET_FLOATS)

# every entry point include/pfmd.h declares
EXPORTS = ("pfmd_default_options", "pfmd_create_from_files", "pfmd_destroy", "pfmd_errmsg", "pfmd_strerror",
           "pfmd_advance", "pfmd_finish", "pfmd_md", "pfmd_run_md_simulation", "pfmd_natoms", "pfmd_md_step",
           "pfmd_get_state", "pfmd_set_state", "pfmd_energies", "pfmd_compute", "pfmd_ninteractions",
           "pfmd_nlist_shape", "pfmd_get_nlist", "pfmd_nlist_load", "pfmd_get_gr_norm", "pfmd_set_group_n",
           "pfmd_get_stream", "pfmd_kernel_launches", "pfmd_advance_timed", "pfmd_time_kernel",
           "pfmd_flush_l2", "pfmd_batch_create", "pfmd_batch_destroy", "pfmd_batch_errmsg", "pfmd_batch_info",
           "pfmd_batch_replica", "pfmd_batch_run", "pfmd_batch_run_list", "pfmd_batch_graphs", "pfmd_batch_tune", "pfmd_batch_set_tpa", "pfmd_batch_get_state",
           "pfmd_batch_energies", "pfmd_batch_energy_history", "pfmd_learned_train", "pfmd_learned_use",
           "pfmd_learned_check", "pfmd_learned_status", "pfmd_learned_gradient", "pfmd_nlist_builds", "pfmd_rjl_forces_noalloc",
           "pfmd_gr_on_cu_analysis", "pfmd_run_gr_analysis", "pfmd_run_gr_moire_fitting", "pfmd_debug_waits",
           "pfmd_batch_create_entries", "pfmd_batch_accepts")

_LIB = None


class PfmdError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{strerror(code)}: {msg}")
        self.code = code


class Options(C.Structure):
    _fields_ = [("form", C.c_int), ("rand_seed", C.c_int), ("out_period", C.c_int), ("out_fd", C.c_int),
                ("all_out_fd", C.c_int), ("write_files", C.c_int), ("output_prefix", C.c_char_p),
                ("num_threads", C.c_int), ("device", C.c_int), ("use_graphs", C.c_int),
                ("threads_per_row", C.c_int), ("async_io", C.c_int), ("skin_lists", C.c_int),
                ("fuse_steps", C.c_int)]


def load(path=LIB_PATH):
    """Loads libpfmd.so (build it with pfmds_gb300._build.build() or __graft_entry__.build())."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(path):
        raise ImportError(f"pfmds_gb300: CUDA library {path} is missing; run pfmds_gb300._build.build()")
    L = C.CDLL(path)
    vp, ip, dp, llp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_longlong)
    L.pfmd_default_options.argtypes = [C.POINTER(Options)]
    L.pfmd_default_options.restype = None
    L.pfmd_create_from_files.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(Options), C.POINTER(vp)]
    L.pfmd_destroy.argtypes = [vp]
    L.pfmd_destroy.restype = None
    L.pfmd_errmsg.argtypes = [vp]
    L.pfmd_errmsg.restype = C.c_char_p
    L.pfmd_strerror.argtypes = [C.c_int]
    L.pfmd_strerror.restype = C.c_char_p
    L.pfmd_advance.argtypes = [vp, C.c_longlong, ip]
    L.pfmd_finish.argtypes = [vp]
    L.pfmd_md.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(Options)]
    L.pfmd_run_md_simulation.argtypes = [C.c_int, C.POINTER(C.c_char_p)]
    L.pfmd_run_gr_analysis.argtypes = [C.c_int, C.POINTER(C.c_char_p)]
    L.pfmd_run_gr_moire_fitting.argtypes = [C.c_int, C.POINTER(C.c_char_p)]
    L.pfmd_gr_on_cu_analysis.argtypes = [C.c_char_p, C.c_double, dp, dp]
    L.pfmd_natoms.argtypes = [vp, ip]
    L.pfmd_md_step.argtypes = [vp, llp, dp]
    # the array arguments of the per-step calls as plain pointers (see _addr)
    L.pfmd_get_state.argtypes = [vp, vp, vp, vp]
    L.pfmd_set_state.argtypes = [vp, vp, vp]
    L.pfmd_energies.argtypes = [vp, vp, dp, dp, dp, dp, dp]
    L.pfmd_compute.argtypes = [vp, C.c_int, dp]
    L.pfmd_ninteractions.argtypes = [vp, ip]
    L.pfmd_nlist_shape.argtypes = [vp, C.c_int, C.c_int, ip, ip]
    L.pfmd_get_nlist.argtypes = [vp, C.c_int, C.c_int, ip, ip, ip, ip]
    L.pfmd_nlist_load.argtypes = [vp, ip, ip]
    L.pfmd_get_gr_norm.argtypes = [vp, C.c_int, dp]
    L.pfmd_set_group_n.argtypes = [vp, C.c_int, C.c_int]
    L.pfmd_get_stream.argtypes = [vp, C.POINTER(vp)]
    L.pfmd_kernel_launches.argtypes = [vp, llp]
    L.pfmd_advance_timed.argtypes = [vp, C.c_longlong, ip, dp]
    L.pfmd_time_kernel.argtypes = [vp, C.c_char_p, C.c_int, dp, dp]
    L.pfmd_flush_l2.argtypes = [vp, C.c_longlong]
    L.pfmd_batch_create.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(Options), C.POINTER(vp)]
    L.pfmd_batch_destroy.argtypes = [vp]
    L.pfmd_batch_destroy.restype = None
    L.pfmd_batch_errmsg.argtypes = [vp]
    L.pfmd_batch_errmsg.restype = C.c_char_p
    L.pfmd_batch_info.argtypes = [vp, ip, llp, llp]
    L.pfmd_batch_replica.argtypes = [vp, C.c_int, ip, ip, ip]
    L.pfmd_batch_run.argtypes = [vp, C.c_longlong, dp]
    L.pfmd_batch_run_list.argtypes = [vp, C.c_char_p, C.c_int, dp]
    L.pfmd_batch_graphs.argtypes = [vp, ip]
    L.pfmd_nlist_builds.argtypes = [vp, llp, ip]
    L.pfmd_batch_tune.argtypes = [vp, C.c_int, ip]
    L.pfmd_batch_set_tpa.argtypes = [vp, ip]
    L.pfmd_batch_get_state.argtypes = [vp, C.c_int, dp, dp, dp]
    L.pfmd_batch_energies.argtypes = [vp, dp, dp]
    L.pfmd_batch_energy_history.argtypes = [vp, dp, llp, ip]
    L.pfmd_learned_train.argtypes = [vp, C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                     C.c_int, dp, dp]
    L.pfmd_learned_gradient.argtypes = [vp, C.c_char_p, C.c_double, C.c_int, C.POINTER(C.c_float), dp, dp]
    L.pfmd_learned_use.argtypes = [vp, C.c_char_p, C.c_longlong, C.c_double, C.c_int]
    L.pfmd_learned_check.argtypes = [vp, dp]
    L.pfmd_learned_status.argtypes = [vp, ip, ip, dp, ip]
    # device buffers are passed as integer addresses (c_void_p)
    L.pfmd_debug_waits.argtypes = [C.c_uint, C.c_int]
    L.pfmd_batch_create_entries.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_char_p), C.POINTER(C.c_char_p),
                                            C.POINTER(Options), C.POINTER(vp)]
    L.pfmd_batch_accepts.argtypes = [C.c_char_p, C.c_char_p, llp, ip, llp, C.c_char_p, C.c_int]
    L.pfmd_rjl_forces_noalloc.argtypes = [C.c_int, vp, dp, dp, vp, vp, C.c_int, vp, vp, vp, C.c_char_p, C.c_int]
    _LIB = L
    return L


def debug_waits(spin_limit=0, stall=False):
    """Test hook of the bounded device waits (pfmd_debug_waits): a poll limit
    (0: built-in) and whether the next waits are made impossible."""
    load().pfmd_debug_waits(int(spin_limit), 1 if stall else 0)


def batch_accepts(input_path, settings):
    """(accepted, reason, (steps, list period, zero_momentum_period)) of one
    settings file for the batched kernel (host only)."""
    ip = input_path if (not input_path or input_path.endswith("/")) else input_path + "/"
    st, per, zmp = C.c_longlong(), C.c_int(), C.c_longlong()
    why = C.create_string_buffer(512)
    rc = load().pfmd_batch_accepts(ip.encode(), settings.encode(), C.byref(st), C.byref(per), C.byref(zmp), why,
                                   len(why))
    return rc == PFMD_OK, why.value.decode(), (st.value, per.value, zmp.value)


def strerror(code):
    try:
        return load().pfmd_strerror(code).decode()
    except ImportError:
        return str(code)


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _addr(a):
    """A C-contiguous array's data as a void* argument.  Through the buffer
    protocol when the array is writable (a fraction of the cost of data_as,
    which matters on the per-step calls), else by its address."""
    try:
        return C.byref(C.c_char.from_buffer(a))
    except (TypeError, ValueError):
        return C.c_void_p(a.__array_interface__["data"][0])


def default_options(**kw):
    o = Options()
    load().pfmd_default_options(C.byref(o))
    for k, v in kw.items():
        if k == "form" and isinstance(v, str):
            v = FORMS[v]
        if k == "output_prefix" and isinstance(v, str):
            v = v.encode()
        setattr(o, k, v)
    return o


class Simulation:
    """One md() run on the GPU (md_simulation.f90:19): set-up on construction,
    then advance() through the loop body and finish() for the closing output."""

    def __init__(self, input_path, settings="md_run_settings.txt", form="plain", out_period=1, write_files=False,
                 prefix="", use_graphs=True, out_fd=-1, all_out_fd=-1, seed=1, num_threads=1, device=0,
                 threads_per_row=0, async_io=True, skin_lists=True, fuse_steps=True):
        L = load()
        self._prefix = prefix.encode()
        self.opts = default_options(form=form, out_period=out_period, write_files=1 if write_files else 0,
                                    output_prefix=self._prefix, use_graphs=1 if use_graphs else 0, out_fd=out_fd,
                                    all_out_fd=all_out_fd, rand_seed=seed, num_threads=num_threads, device=device,
                                    threads_per_row=threads_per_row, async_io=1 if async_io else 0,
                                    skin_lists=1 if skin_lists else 0, fuse_steps=1 if fuse_steps else 0)
        self._h = C.c_void_p()
        ip = input_path if (not input_path or input_path.endswith("/")) else input_path + "/"
        rc = L.pfmd_create_from_files(ip.encode(), settings.encode(), C.byref(self.opts), C.byref(self._h))
        if rc:
            msg = L.pfmd_errmsg(self._h).decode()
            L.pfmd_destroy(self._h)
            self._h = None
            raise PfmdError(rc, msg)
        self.finished = False

    def close(self):
        if getattr(self, "_h", None):
            load().pfmd_destroy(self._h)
            self._h = None

    __del__ = close

    def _check(self, rc):
        if rc:
            raise PfmdError(rc, load().pfmd_errmsg(self._h).decode())

    def advance(self, n):
        if getattr(self, "_fin", None) is None:
            self._fin = C.c_int(0)
            self._finref = C.byref(self._fin)
        self._check(load().pfmd_advance(self._h, int(n), self._finref))
        self.finished = bool(self._fin.value)
        return self.finished

    def finish(self):
        self._check(load().pfmd_finish(self._h))

    @property
    def natoms(self):
        n = getattr(self, "_natoms", None)
        if n is None:  # fixed for the context's life
            c = C.c_int()
            self._check(load().pfmd_natoms(self._h, C.byref(c)))
            n = self._natoms = c.value
        return n

    @property
    def md_step(self):
        s, t = C.c_longlong(), C.c_double()
        self._check(load().pfmd_md_step(self._h, C.byref(s), C.byref(t)))
        return s.value

    @property
    def sim_time(self):
        s, t = C.c_longlong(), C.c_double()
        self._check(load().pfmd_md_step(self._h, C.byref(s), C.byref(t)))
        return t.value

    def state(self, out=None):
        """Positions, velocities and forces (n x 3 each); `out` may supply three
        C-contiguous float64 arrays to fill (pinned host memory, for instance)."""
        n = self.natoms
        p, v, f = out if out is not None else (np.zeros((n, 3)) for _ in range(3))
        for a in (p, v, f):
            if a.shape != (n, 3) or a.dtype != np.float64 or not a.flags.c_contiguous:
                raise ValueError("state(): out arrays must be C-contiguous float64 of shape (natoms, 3)")
        self._check(load().pfmd_get_state(self._h, _addr(p), _addr(v), _addr(f)))
        return p, v, f

    def set_state(self, pos=None, vel=None):
        n = self.natoms
        p = None if pos is None else np.ascontiguousarray(pos, dtype=np.float64)
        v = None if vel is None else np.ascontiguousarray(vel, dtype=np.float64)
        for a in (p, v):
            if a is not None and a.size != 3 * n:
                raise ValueError("set_state(): arrays must hold natoms x 3 values")
        self._check(load().pfmd_set_state(self._h, None if p is None else _addr(p), None if v is None else _addr(v)))

    @property
    def n_interactions(self):
        k = getattr(self, "_nint", None)
        if k is None:  # fixed for the context's life
            c = C.c_int()
            self._check(load().pfmd_ninteractions(self._h, C.byref(c)))
            k = self._nint = c.value
        return k

    def energies(self):
        ni = self.n_interactions
        e = np.zeros(max(1, ni))
        if getattr(self, "_evals", None) is None:
            self._evals = [C.c_double() for _ in range(5)]
            self._erefs = [C.byref(v) for v in self._evals]
        self._check(load().pfmd_energies(self._h, _addr(e), *self._erefs))
        pe, ke, t, enhc, econs = (v.value for v in self._evals)
        return dict(inter=e[:ni].copy(), pe=pe, ke=ke, temperature=t, nhc=enhc, conserved=econs)

    def compute(self, rebuild=True):
        e = np.zeros(max(1, self.n_interactions))
        self._check(load().pfmd_compute(self._h, 1 if rebuild else 0, _dp(e)))
        return e[:self.n_interactions].copy()

    def nlist(self, inter, lst):
        n, m = C.c_int(), C.c_int()
        self._check(load().pfmd_nlist_shape(self._h, inter, lst, C.byref(n), C.byref(m)))
        n, m = n.value, m.value
        nnum = np.zeros(n, np.int32)
        less = np.zeros(n, np.int32)
        pidx = np.zeros(n, np.int32)
        nl = np.zeros((n, m), np.int32)
        self._check(load().pfmd_get_nlist(self._h, inter, lst, _ip(nnum), _ip(less), _ip(pidx), _ip(nl)))
        return dict(nnum=nnum, lessnnum=less, pidx=pidx, nlist=nl)

    def gr_norm(self, inter):
        n, m = C.c_int(), C.c_int()
        self._check(load().pfmd_nlist_shape(self._h, inter, 2, C.byref(n), C.byref(m)))
        g = np.zeros((n.value, 3))
        self._check(load().pfmd_get_gr_norm(self._h, inter, _dp(g)))
        return g

    def nlist_load(self):
        buf = np.zeros(64, np.int32)
        cnt = C.c_int()
        self._check(load().pfmd_nlist_load(self._h, _ip(buf), C.byref(cnt)))
        return buf[:cnt.value].copy()

    def nlist_builds(self):
        """Rebuilds of every list so far (-1: a list rebuilt at every update step)."""
        buf = np.zeros(64, np.int64)
        cnt = C.c_int()
        self._check(load().pfmd_nlist_builds(self._h, buf.ctypes.data_as(C.POINTER(C.c_longlong)), C.byref(cnt)))
        return buf[:cnt.value].copy()

    def set_group_n(self, group, n):
        self._check(load().pfmd_set_group_n(self._h, group, n))

    def learned_train(self, model_out, frames, stride=10, iters=4, lr=1e-3, model_in=None, force_weight=1.0,
                      tensor_cores=False):
        """Online training from this plain-form run (tensor_cores: the training
        kernels on tcgen05); returns the per-interaction per-atom energy RMSE (eV)
        of the last frame (NaN where no network) and the learned-against-plain force
        RMSE (eV/A) on it."""
        r = np.zeros(max(1, self.n_interactions))
        fr = C.c_double()
        self._check(load().pfmd_learned_train(self._h, model_in.encode() if model_in else None,
                                              model_out.encode() if model_out else None, frames, stride, iters, lr,
                                              force_weight, 1 if tensor_cores else 0, _dp(r), C.byref(fr)))
        return r[:self.n_interactions].copy(), fr.value

    def learned_gradient(self, model_in=None, force_weight=1.0, tensor_cores=False, n_networks=1, timed=False):
        """(gradient, loss[, device ms]): the training-loss gradient of each network
        at this configuration (rows of NET_FLOATS floats), its summed squared energy
        error and, with timed, the device time of the gradient kernels."""
        g = np.zeros((n_networks, NET_FLOATS), np.float32)
        loss = np.zeros(n_networks)
        ms = C.c_double()
        self._check(load().pfmd_learned_gradient(self._h, model_in.encode() if model_in else None, force_weight,
                                                 1 if tensor_cores else 0,
                                                 g.ctypes.data_as(C.POINTER(C.c_float)), _dp(loss), C.byref(ms)))
        return (g, loss, ms.value) if timed else (g, loss)

    def learned_use(self, model_path, check_period=100, max_rmse=0.05, tensor_cores=False):
        self._check(load().pfmd_learned_use(self._h, model_path.encode(), check_period, max_rmse,
                                            1 if tensor_cores else 0))

    def learned_check(self):
        r = C.c_double()
        self._check(load().pfmd_learned_check(self._h, C.byref(r)))
        return r.value

    def learned_status(self):
        a, n, f = C.c_int(), C.c_int(), C.c_int()
        r = C.c_double()
        self._check(load().pfmd_learned_status(self._h, C.byref(a), C.byref(n), C.byref(r), C.byref(f)))
        return dict(active=bool(a.value), checks=n.value, last_rmse=r.value, fallen_back=bool(f.value))

    @property
    def stream(self):
        s = C.c_void_p()
        self._check(load().pfmd_get_stream(self._h, C.byref(s)))
        return s.value or 0

    def advance_timed(self, n):
        """advance(n) and the device milliseconds between its first and last kernel."""
        f, ms = C.c_int(0), C.c_double(0.0)
        self._check(load().pfmd_advance_timed(self._h, int(n), C.byref(f), C.byref(ms)))
        self.finished = bool(f.value)
        return ms.value

    def time_kernel(self, name, reps=20):
        """(average ms per launch, algorithmic bytes per launch) of one kernel group."""
        ms, b = C.c_double(), C.c_double()
        self._check(load().pfmd_time_kernel(self._h, name.encode(), int(reps), C.byref(ms), C.byref(b)))
        return ms.value, b.value

    def flush_l2(self, nbytes=256 << 20):
        self._check(load().pfmd_flush_l2(self._h, int(nbytes)))

    @property
    def kernel_launches(self):
        n = C.c_longlong()
        self._check(load().pfmd_kernel_launches(self._h, C.byref(n)))
        return n.value


def md(input_path, settings="md_run_settings.txt", **kw):
    """The whole md() call (create, advance to the end, finish)."""
    L = load()
    prefix = kw.pop("prefix", "")
    o = default_options(output_prefix=prefix.encode(), **kw)
    ip = input_path if (not input_path or input_path.endswith("/")) else input_path + "/"
    return L.pfmd_md(ip.encode(), settings.encode(), C.byref(o))


class Batch:
    """Batched form: every replica of a settings list (the -ilist format of
    run_md_simulation_mpi) in one device state, advanced together by one
    persistent kernel (precision form)."""

    def __init__(self, input_path, list_file, device=0):
        L = load()
        self.opts = default_options(form="precision", device=device)
        self._h = C.c_void_p()
        ip = input_path if (not input_path or input_path.endswith("/")) else input_path + "/"
        rc = L.pfmd_batch_create(ip.encode(), list_file.encode(), C.byref(self.opts), C.byref(self._h))
        if rc:
            msg = L.pfmd_batch_errmsg(self._h).decode()
            L.pfmd_batch_destroy(self._h)
            self._h = None
            raise PfmdError(rc, msg)

    def close(self):
        if getattr(self, "_h", None):
            load().pfmd_batch_destroy(self._h)
            self._h = None

    __del__ = close

    def _check(self, rc):
        if rc:
            raise PfmdError(rc, load().pfmd_batch_errmsg(self._h).decode())

    def info(self):
        r, n, s = C.c_int(), C.c_longlong(), C.c_longlong()
        self._check(load().pfmd_batch_info(self._h, C.byref(r), C.byref(n), C.byref(s)))
        return r.value, n.value, s.value

    @property
    def n_replicas(self):
        return self.info()[0]

    def replica(self, r):
        a, n, k = C.c_int(), C.c_int(), C.c_int()
        self._check(load().pfmd_batch_replica(self._h, r, C.byref(a), C.byref(n), C.byref(k)))
        return dict(atom0=a.value, n=n.value, kind=("lj", "rjl")[k.value])

    def run(self, nsteps):
        ms = C.c_double()
        self._check(load().pfmd_batch_run(self._h, nsteps, C.byref(ms)))
        return ms.value

    def graphs(self):
        """CUDA graphs held for runs (-1: runs launch directly)."""
        n = C.c_int()
        self._check(load().pfmd_batch_graphs(self._h, C.byref(n)))
        return n.value

    def run_list(self, out_path="", all_out=None):
        """Run every entry to the end of its nve stage and write each entry's
        files (log, snapshots, trajectory, final .xyz) under out_path + its
        prefix; the closing records go to the file all_out when given.  Returns
        the device time in ms."""
        ms = C.c_double()
        f = open(all_out, "w") if all_out else None
        try:
            if f:
                f.flush()
            self._check(load().pfmd_batch_run_list(self._h, out_path.encode(), f.fileno() if f else -1,
                                                   C.byref(ms)))
        finally:
            if f:
                f.close()
        return ms.value

    def tune(self, steps=10):
        t = np.zeros(6, np.int32)
        self._check(load().pfmd_batch_tune(self._h, steps, _ip(t)))
        return t.tolist()

    def set_tpa(self, tpa):
        t = np.ascontiguousarray(tpa, dtype=np.int32)
        self._check(load().pfmd_batch_set_tpa(self._h, _ip(t)))

    def state(self, r):
        n = self.replica(r)["n"]
        p, v, f = (np.zeros((n, 3)) for _ in range(3))
        self._check(load().pfmd_batch_get_state(self._h, r, _dp(p), _dp(v), _dp(f)))
        return p, v, f

    def energies(self):
        R = self.n_replicas
        ep, ek = np.zeros(R), np.zeros(R)
        self._check(load().pfmd_batch_energies(self._h, _dp(ep), _dp(ek)))
        return ep, ek

    def history(self):
        """(rows, replicas, 2) array of (potential, kinetic) per energy step, and
        the steps between rows; history4() keeps the potential per interaction."""
        h4, per = self.history4()
        return np.stack([h4[..., :3].sum(-1), h4[..., 3]], axis=-1), per

    def history4(self):
        """(rows, replicas, 4): the three interaction energies and the kinetic energy."""
        h5, per = self.history5()
        return h5[..., :4], per

    def history5(self):
        """(rows, replicas, 5): the three interaction energies, the kinetic energy
        and the Nose-Hoover chain's energy (0 for nve replicas)."""
        rows, per = C.c_longlong(), C.c_int()
        self._check(load().pfmd_batch_energy_history(self._h, None, C.byref(rows), C.byref(per)))
        h = np.zeros((max(rows.value, 0), self.n_replicas, 5))
        if rows.value:
            self._check(load().pfmd_batch_energy_history(self._h, _dp(h), C.byref(rows), C.byref(per)))
        return h, per.value


def _argv(name, args):
    return len(args) + 1, (C.c_char_p * (len(args) + 1))(*([name.encode()] + [a.encode() for a in args]))


def run_md_simulation(args):
    """The run_md_simulation command line, in-process."""
    return load().pfmd_run_md_simulation(*_argv("run_md_simulation", args))


def run_gr_moire_fitting(args):
    """The run_gr_moire_fitting command line, in-process (md() runs on the GPU)."""
    return load().pfmd_run_gr_moire_fitting(*_argv("run_gr_moire_fitting", args))


def run_gr_analysis(args):
    """The run_gr_analysis command line, in-process (host only)."""
    return load().pfmd_run_gr_analysis(*_argv("run_gr_analysis", args))


def gr_on_cu_analysis(path, z):
    """(arr1, arr2): mean, minimum and maximum z above z of the carbon and of the
    copper atoms of an .xyz file (host only)."""
    a1, a2 = np.zeros(3), np.zeros(3)
    rc = load().pfmd_gr_on_cu_analysis(str(path).encode(), float(z), _dp(a1), _dp(a2))
    if rc:
        raise PfmdError(rc, f"cannot analyse {path}")
    return a1, a2
