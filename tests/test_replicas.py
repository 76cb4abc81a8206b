"""Replica aggregation of bench.py across ranks, on CPU with two gloo ranks:
the slowest rank's time and the sum of every rank's iterations make the
whole-job value; the reference arm runs on rank 0 only."""
import os
import sys
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    ws, r, _ = bench.dist_env()
    dist = bench.dist_init(ws)
    ms = 100.0 + 50.0 * r            # rank 1 is the slowest
    iters = 20 * (r + 1)
    tmax = bench.allreduce_max(dist, ms)
    total = bench.allreduce_sum(dist, iters)
    bench.barrier(dist)
    ref_rc = None
    if r == 1:
        ref_rc = bench.run_reference(None, ws, r)   # other ranks exit without work
    q.put((r, tmax, total, total / (tmax / 1e3), ref_rc))
    dist.destroy_process_group()


def test_two_gloo_ranks_aggregate():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, tmax, total, value, ref_rc in out:
        assert tmax == 150.0
        assert total == 60
        assert value == pytest.approx(60 / 0.150)
        if r == 1:
            assert ref_rc == 0
