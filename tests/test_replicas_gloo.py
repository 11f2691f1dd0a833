"""Multi-GPU bench path (replicas only: every rank labels its own copy of the
graph, no data-path collective), exercised on CPU with two gloo ranks: the
timing each rank reports must be the maximum over ranks, and the whole-job
throughput counts every replica's labels."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r is slower by r: the job time is the slowest rank's
        got = bench.max_over_ranks(dist, [0.25 + 0.1 * rank, 0.5 + 0.2 * rank], "cpu")
        q.put((rank, got))
    finally:
        dist.destroy_process_group()


def test_timings_are_max_over_two_gloo_ranks():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(world):
        assert res[r] == pytest.approx([0.35, 0.7])


def test_replica_throughput_counts_every_replica():
    assert bench.replica_throughput(1000, 1, 0.5) == pytest.approx(2000.0)
    assert bench.replica_throughput(1000, 4, 0.5) == pytest.approx(8000.0)
