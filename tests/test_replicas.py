"""Several GPUs run independent replicas (no data-path collective): bench.py's
rank helpers take the max of the timed spans and the sum of the atoms over ranks,
and the reference arm runs on rank 0 only.  Checked with two gloo ranks on CPU."""
import multiprocessing as mp
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2",
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    r, w, dist = bench.dist_init()
    span = bench.dist_max(dist, 10.0 * (rank + 1))    # timed spans: the slowest rank counts
    atoms = bench.dist_sum(dist, 1000.0 * (rank + 1))  # work: every rank's atoms
    bench.barrier(dist)
    dist.destroy_process_group()
    q.put((r, w, span, atoms))


def test_rank_helpers_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(timeout=180)
    assert all(p.exitcode == 0 for p in ps)
    got = sorted(q.get(timeout=10) for _ in ps)
    assert got == [(0, 2, 20.0, 3000.0), (1, 2, 20.0, 3000.0)]


def test_single_process_has_no_group():
    sys.path.insert(0, ROOT)
    import bench
    env_ws = os.environ.pop("WORLD_SIZE", None)
    try:
        assert bench.dist_init() == (0, 1, None)
        assert bench.dist_max(None, 3.5) == 3.5 and bench.dist_sum(None, 2.0) == 2.0
    finally:
        if env_ws is not None:
            os.environ["WORLD_SIZE"] = env_ws


def test_reference_arm_prints_on_rank_zero_only(built):
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and r.stdout.strip() == ""
