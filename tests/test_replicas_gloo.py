"""CPU, two gloo ranks: the multi-replica host logic of bench.py (one replica per GPU, no collective
on the data path): the timed region is the slowest rank's, and the whole-job throughput counts
every rank's steps."""
from __future__ import annotations

import os
import socket

import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        ms = bench.max_over_ranks(10.0 + 5.0 * rank)        # rank 1 is the slowest replica
        out[rank] = (ms, bench.replica_throughput(world, 20, ms))
    finally:
        dist.destroy_process_group()


def test_two_replicas_max_time_and_total_steps():
    import torch.multiprocessing as mp
    world = 2
    port = _free_port()
    with mp.get_context("spawn").Manager() as man:
        out = man.dict()
        mp.start_processes(_rank, args=(world, port, out), nprocs=world, start_method="spawn", join=True)
        res = dict(out)
    assert set(res) == {0, 1}
    for ms, value in res.values():
        assert ms == 15.0
        assert value == pytest.approx(2 * 20 / 0.015)


def test_single_process_is_identity():
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.replica_throughput(1, 10, 100.0) == pytest.approx(100.0)
