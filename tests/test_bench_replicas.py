"""The bench's multi-rank logic on CPU: two gloo ranks, each an independent
replica, reduce to one whole-job rate (sum of edges / slowest rank's time)."""

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    w, r, local, pg = bench.dist_init()
    assert (w, r, local) == (world, rank, rank)
    bench.barrier(pg)
    # rank 0: 10 ms for 1e9 edges; rank 1: 20 ms for 3e9 edges
    ms = 10.0 * (rank + 1)
    edges = 1e9 * (2 * rank + 1)
    rate, ms_max = bench.replica_rate(pg, ms, edges)
    out.put((rank, rate, ms_max))
    pg.destroy_process_group()


def test_two_replicas_gloo():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() % 2000)
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for _, rate, ms_max in res:
        assert ms_max == 20.0
        assert rate == pytest.approx(4e9 / 0.020 / 1e9)


def test_single_rank_has_no_group():
    sys.path.insert(0, ROOT)
    import bench
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        os.environ.pop(k, None)
    w, r, local, pg = bench.dist_init()
    assert (w, r, local, pg) == (1, 0, 0, None)
    rate, ms = bench.replica_rate(None, 5.0, 1e9)
    assert ms == 5.0 and rate == pytest.approx(200.0)
