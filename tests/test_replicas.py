"""Replicas across ranks (the step does not shard; N GPUs run N independent
replicas and the bench reports the whole-job rate over the slowest rank):
the timing reduction and barrier of bench.py on two gloo ranks on the CPU."""
import os

import pytest


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", init_method="env://", rank=rank, world_size=world)
    try:
        w, r, _ = bench._dist()
        bench._barrier(w)
        ms = bench._allreduce_max(10.0 + 5.0 * rank, w)  # per-rank timed region (ms)
        q.put((r, w, ms))
    finally:
        dist.destroy_process_group()


def test_two_rank_replica_timing():
    mp = pytest.importorskip("torch.multiprocessing")
    import socket

    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert got == [(0, 2, 15.0), (1, 2, 15.0)]  # both ranks see the slowest rank's time
