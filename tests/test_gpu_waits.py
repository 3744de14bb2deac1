"""The bounded device waits give up and report PFMD_E_TIMEOUT.

pfmd_debug_waits lowers the poll limit and makes the waits impossible: the
batched kernel's grid barrier then expects one arrival more than the grid has,
and the tensor-core network kernels wait for an mbarrier phase that no MMA
completes.  Each kernel must give up, record the timeout in its status word and
return (the tensor-core kernels also release their TMEM), so the call fails
with PFMD_E_TIMEOUT within a short time and the CUDA context stays usable."""
import time

import numpy as np
import pytest

import pfmds_gb300 as pf
from pfmds_gb300 import configs

pytestmark = pytest.mark.gpu


@pytest.fixture
def stalled_waits():
    pf.debug_waits(spin_limit=2048, stall=True)
    yield
    pf.debug_waits(0, False)


def _context_still_usable(tmp_path):
    d = str(tmp_path / "after")
    configs.lj_gas(d, n_a=100, n_b=100, box=20.0, integrators=[("nve", 0.5, 20, 10 ** 8, 10)])
    s = pf.Simulation(d, form="precision", out_period=10 ** 9)
    s.advance(21)
    assert np.isfinite(s.state()[0]).all()
    s.close()


def test_batch_grid_barrier_times_out(tmp_path, built, stalled_waits):
    ln, reps = configs.batch_systems(str(tmp_path), n_rep=3, n_min=500, n_max=800, steps=100, log_period=10,
                                     seed=3)
    b = pf.Batch(str(tmp_path), ln)
    t0 = time.perf_counter()
    with pytest.raises(pf.PfmdError) as e:
        b.run(10)
    elapsed = time.perf_counter() - t0
    assert e.value.code == pf.PFMD_E_TIMEOUT
    assert "grid barrier gave up waiting" in str(e.value)
    assert elapsed < 10.0, elapsed
    b.close()
    pf.debug_waits(0, False)
    _context_still_usable(tmp_path)


def _gr(d):
    configs.gr_on_cu(str(d), n_gx=6, n_gy=4, n_cx=6, n_cy=3, layers=3, steps=10 ** 6, log_period=10,
                     integrator="nve", tb_list=(32, 4.5))
    return str(d)


def test_tensor_core_network_wait_times_out(tmp_path, built):
    d = _gr(tmp_path)
    m = str(tmp_path / "m.bin")
    s = pf.Simulation(d, form="plain", out_period=10 ** 9)
    s.learned_train(m, frames=1, stride=0, iters=1, lr=2e-3)
    s.close()
    s = pf.Simulation(d, form="precision", out_period=10 ** 9)
    s.learned_use(m, check_period=0, tensor_cores=True)
    s.compute()  # the network kernel runs when its waits can complete
    pf.debug_waits(spin_limit=2048, stall=True)
    try:
        t0 = time.perf_counter()
        with pytest.raises(pf.PfmdError) as e:
            s.compute()
        elapsed = time.perf_counter() - t0
    finally:
        pf.debug_waits(0, False)
    assert e.value.code == pf.PFMD_E_TIMEOUT
    assert elapsed < 10.0, elapsed
    s.close()
    _context_still_usable(tmp_path)


def test_tensor_core_training_wait_times_out(tmp_path, built):
    d = _gr(tmp_path)
    m = str(tmp_path / "m.bin")
    s = pf.Simulation(d, form="plain", out_period=10 ** 9)
    s.learned_train(m, frames=1, stride=0, iters=1, lr=2e-3)
    s.learned_gradient(m, tensor_cores=True, n_networks=2)  # tb and rjl networks
    pf.debug_waits(spin_limit=2048, stall=True)
    try:
        with pytest.raises(pf.PfmdError) as e:
            s.learned_gradient(m, tensor_cores=True, n_networks=2)
    finally:
        pf.debug_waits(0, False)
    assert e.value.code == pf.PFMD_E_TIMEOUT
    s.close()
    _context_still_usable(tmp_path)
