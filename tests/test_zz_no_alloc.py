"""pfmd_rjl_forces_noalloc: rjl forces and energy without any device allocation.

The entry point serves callers that cannot call cudaMalloc -- host codes whose
device memory is all held by their own pool allocator, and loops that cannot
take the device-wide synchronisation that cudaMalloc and cudaFree imply.  The
caller owns every buffer; the entry point's scratch is a fixed array inside the
library.  These tests call it through the C ABI on device buffers that the test
(the caller) owns, and compare it with the context API's own rjl forces and
energy (pfmd_compute) on two calls in a row: the second call sees a different
configuration, so scratch left over from the first call would show.
"""
import ctypes as C

import numpy as np
import pytest

import pfmds_gb300 as pf
from pfmds_gb300 import configs

MAX_ATOMS = 1 << 20  # capacity of the entry point's fixed scratch
NX, NY, NZ, A = 8, 8, 5, 3.615


def _call(n, pos, box, params, nnum, nbr, max_nbr, frc, energy, stream=0):
    err = C.create_string_buffer(256)
    rc = pf.load().pfmd_rjl_forces_noalloc(
        n, pos, box.ctypes.data_as(C.POINTER(C.c_double)), params.ctypes.data_as(C.POINTER(C.c_double)),
        nnum, nbr, max_nbr, frc, energy, stream, err, len(err))
    return rc, err.value.decode()


def test_rejects_sizes_beyond_its_scratch(built):
    # returns before touching the device: runs without a GPU too
    box = np.array([10.0, 10.0, 10.0])
    params = np.array([0.0855, 1.224, 10.96, 2.278, 2.556, 4.5, 5.0])
    rc, msg = _call(MAX_ATOMS + 1, 1, box, params, 1, 1, 8, 1, None)
    assert rc == pf.PFMD_E_PARAM
    assert "1048577" in msg and str(MAX_ATOMS) in msg
    rc, msg = _call(-1, 1, box, params, 1, 1, 8, 1, None)
    assert rc == pf.PFMD_E_PARAM


def _atom_list(sim, n):
    """The context's rjl list as n x max_nbr partner atoms, row i = atom i."""
    nl = sim.nlist(0, 0)
    pidx, nnum, ent = nl["pidx"], nl["nnum"], nl["nlist"]
    assert sorted(pidx.tolist()) == list(range(n))  # one group holds every atom
    m = ent.shape[1]
    nbr = np.full((n, m), -1, np.int32)
    cnt = np.zeros(n, np.int32)
    for r in range(len(pidx)):
        k = nnum[r]
        nbr[pidx[r], :k] = pidx[ent[r, :k]]
        cnt[pidx[r]] = k
    return cnt, nbr


@pytest.mark.gpu
def test_matches_context_forces_on_two_calls(tmp_path, built):
    torch = pytest.importorskip("torch")
    configs.cu_slab(str(tmp_path), nx=NX, ny=NY, nz=NZ, steps=100, log_period=10)
    box = np.asarray(configs.fcc_slab(NX, NY, NZ, A, vacuum=25.0)[1], dtype=np.float64)
    params = np.array([float(x) for x in open(tmp_path / "parameters_RJL_Cu.txt").read().split()])
    assert params.shape == (7,)
    sim = pf.Simulation(str(tmp_path), form="plain")
    n = sim.natoms
    dev = torch.device("cuda:0")
    frc_d = torch.empty((n, 3), dtype=torch.float64, device=dev)
    e_d = torch.empty(1, dtype=torch.float64, device=dev)
    for call, steps in enumerate((0, 15)):
        if steps:
            sim.advance(steps)
        e_ref = sim.compute(rebuild=True)[0]
        pos, _, f_ref = sim.state()
        cnt, nbr = _atom_list(sim, n)
        pos_d = torch.from_numpy(np.ascontiguousarray(pos)).to(dev)
        nnum_d = torch.from_numpy(cnt).to(dev)
        nbr_d = torch.from_numpy(nbr).to(dev)
        frc_d.fill_(float("nan"))
        stream = torch.cuda.current_stream(dev).cuda_stream
        rc, msg = _call(n, pos_d.data_ptr(), box, params, nnum_d.data_ptr(), nbr_d.data_ptr(), nbr.shape[1],
                        frc_d.data_ptr(), e_d.data_ptr(), stream)
        assert rc == pf.PFMD_OK, msg
        torch.cuda.synchronize(dev)
        f = frc_d.cpu().numpy()
        e = float(e_d.cpu()[0])
        scale = np.abs(f_ref).max()
        # the same tolerance as the plain-form parity tests: 1e-9 of the force scale
        assert np.abs(f - f_ref).max() <= 1e-9 * scale, f"call {call + 1}"
        assert abs(e - e_ref) <= 1e-9 * abs(e_ref), f"call {call + 1}: {e} vs {e_ref}"
    sim.close()


@pytest.mark.gpu
def test_rows_longer_than_max_nbr_give_nan(tmp_path, built):
    """A row whose count exceeds max_nbr is cut; its force and the energy come
    back NaN instead of plausible wrong values."""
    torch = pytest.importorskip("torch")
    configs.cu_slab(str(tmp_path), nx=NX, ny=NY, nz=NZ, steps=100, log_period=10)
    box = np.asarray(configs.fcc_slab(NX, NY, NZ, A, vacuum=25.0)[1], dtype=np.float64)
    params = np.array([float(x) for x in open(tmp_path / "parameters_RJL_Cu.txt").read().split()])
    sim = pf.Simulation(str(tmp_path), form="plain")
    n = sim.natoms
    sim.compute(rebuild=True)
    pos = sim.state()[0]
    cnt, nbr = _atom_list(sim, n)
    sim.close()
    width = int(cnt.max()) - 1
    cut = cnt > width
    assert cut.any() and not cut.all()
    dev = torch.device("cuda:0")
    pos_d = torch.from_numpy(np.ascontiguousarray(pos)).to(dev)
    nnum_d = torch.from_numpy(cnt).to(dev)
    nbr_d = torch.from_numpy(np.ascontiguousarray(nbr[:, :width])).to(dev)
    frc_d = torch.zeros((n, 3), dtype=torch.float64, device=dev)
    e_d = torch.zeros(1, dtype=torch.float64, device=dev)
    rc, msg = _call(n, pos_d.data_ptr(), box, params, nnum_d.data_ptr(), nbr_d.data_ptr(), width,
                    frc_d.data_ptr(), e_d.data_ptr(), torch.cuda.current_stream(dev).cuda_stream)
    assert rc == pf.PFMD_OK, msg
    torch.cuda.synchronize(dev)
    f = frc_d.cpu().numpy()
    assert np.isnan(f[cut]).all()
    assert np.isnan(float(e_d.cpu()[0]))
