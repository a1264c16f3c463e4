"""The multi-GPU form of the benchmark is replicas only: every rank solves its own copy of
the batch and the job's time is the slowest rank's. This checks that host logic on CPU
with two gloo ranks (no GPU): the max-over-ranks reduction `bench.aggregate_max` and the
whole-job throughput that bench.py derives from it."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        ms = [40.0, 46.5][rank]  # per-replica step time
        worst = bench.aggregate_max(ms, world, None)
        count = 40000
        out[rank] = (worst, world * count / (worst / 1e3))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_replicas_max_over_ranks():
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank, args=(world, _free_port(), out), nprocs=world, start_method="spawn", join=True)
    assert out[0] == out[1]  # every rank sees the same job time
    worst, value = out[0]
    assert worst == 46.5  # the slowest replica's time
    assert value == pytest.approx(2 * 40000 / 0.0465)  # all ranks' solves over that time
