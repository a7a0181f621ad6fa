"""Replicas on several ranks (the only multi-GPU form of this path): the job's rate is all ranks'
work over the slowest rank's time. Exercised with world_size 2 over gloo on the CPU."""

import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, times, q):
    import sys

    import torch.distributed as dist

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        bench.barrier(dist)
        tmax = bench.max_over_ranks(times[rank], dist)
        rate = bench.replica_rate(5, times[rank], dist)
        q.put((rank, tmax, rate))
    finally:
        dist.destroy_process_group()


def test_replica_rate_over_two_gloo_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    times = [2.0, 2.5]
    procs = [ctx.Process(target=_rank, args=(r, 2, port, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, tmax, rate in out:
        assert tmax == pytest.approx(2.5)
        assert rate == pytest.approx(2 * 5 / 2.5)


def test_single_process_rate():
    import sys

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench

    assert bench.replica_rate(4, 2.0, None) == pytest.approx(2.0)
