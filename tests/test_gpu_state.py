"""State transfers through the C ABI: page-locked host arrays are read and written
in place by the conversion kernels, pageable ones through a staging copy; both
give the same bits, and cached energies stay those of the last step."""
import numpy as np
import pytest

import pfmds_gb300 as pf
from pfmds_gb300 import configs

pytestmark = pytest.mark.gpu


def _pinned(n_doubles):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA-enabled torch for page-locked host memory")
    return torch.zeros(n_doubles, dtype=torch.float64, pin_memory=True).numpy()


def test_pinned_and_pageable_state_transfers_match(tmp_path, built):
    configs.cu_slab(str(tmp_path), nx=6, ny=6, nz=4, steps=100, log_period=10, temperature=300.0)
    d = str(tmp_path)
    s = pf.Simulation(d, form="precision", out_period=10 ** 6)
    s.advance(12)
    n = s.natoms
    ref = s.state()
    # the arrays start one double into a larger page-locked block
    block = _pinned(9 * n + 7)
    outs = tuple(block[1 + 3 * n * k: 1 + 3 * n * (k + 1)].reshape(n, 3) for k in range(3))
    got = s.state(out=outs)
    for a, b in zip(ref, got):
        assert np.array_equal(a, b)

    p, v, _ = ref
    v2 = v * 0.99
    outs[0][...] = p
    outs[1][...] = v2
    s.set_state(outs[0], outs[1])  # page-locked: read in place
    s.advance(7)
    a = s.state()
    e_a = s.energies()

    r = pf.Simulation(d, form="precision", out_period=10 ** 6)
    r.advance(12)
    r.set_state(p.copy(), v2.copy())  # pageable: staged
    r.advance(7)
    b = r.state()
    e_b = r.energies()
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    assert e_a["conserved"] == e_b["conserved"] and e_a["ke"] == e_b["ke"]
    s.close()
    r.close()


def test_cached_energies_follow_the_run(tmp_path, built):
    """energies() reuses the control block read at the end of advance() until a
    call that may launch work; reading the state in between keeps it."""
    configs.cu_slab(str(tmp_path), nx=6, ny=6, nz=4, steps=100, log_period=5, temperature=300.0)
    s = pf.Simulation(str(tmp_path), form="precision", out_period=10 ** 6)
    s.advance(10)
    e1 = s.energies()
    s.state()
    assert s.energies()["conserved"] == e1["conserved"]
    s.advance(5)
    e2 = s.energies()
    assert e2["ke"] != e1["ke"]
    e3 = s.compute()
    assert np.allclose(s.energies()["inter"], e3)
    s.close()
