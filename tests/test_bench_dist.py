"""bench.py's multi-rank helpers on CPU: two gloo ranks (the N>1 bench runs independent replicas, one
per GPU; the only cross-rank operations are a barrier and the max of the per-rank times)."""
import os
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, q):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    dist, r, w, local = bench.dist_setup(world)
    try:
        assert (r, w) == (rank, world) and dist.get_backend() == "gloo"
        bench.barrier(dist)
        q.put((rank, bench.max_over_ranks(dist, 1.5 + rank)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_max_time():
    pytest.importorskip("torch.distributed")
    import torch
    if torch.cuda.is_available():
        pytest.skip("gloo path is the CPU-only path")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    got = dict(q.get(timeout=10) for _ in range(2))
    assert got == {0: 2.5, 1: 2.5}


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    dist, r, w, local = bench.dist_setup(1)
    assert dist is None and (r, w) == (0, 1)
    assert bench.max_over_ranks(None, 3.0) == 3.0
