"""The benchmark's multi-rank path on the CPU: two gloo ranks. The design is
replicas (each GPU runs the whole workload; no collective on the data path),
so what crosses ranks is the timing: every rank takes the slowest rank's
times (an all-reduce MAX) and the whole-job rate is every rank's steps over
that time."""

import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        # rank r's step and end-to-end times: r + 1 and 3 - r seconds
        got = bench.max_over_ranks([rank + 1.0, 3.0 - rank])
        dist.barrier()
        out[rank] = (got, bench.aggregate_rate(4, world, got[0]))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_times():
    world = 2
    port = _free_port()
    with mp.get_context("spawn").Manager() as manager:
        out = manager.dict()
        mp.start_processes(_rank, args=(world, port, out), nprocs=world, start_method="spawn")
        results = dict(out)
    for rank in range(world):
        got, rate = results[rank]
        assert got == [2.0, 3.0]  # max(1, 2) and max(3, 2)
        assert rate == 4 * 2 / 2.0


def test_one_rank_keeps_its_own_times():
    import bench

    assert bench.max_over_ranks([1.5, 2.5]) == [1.5, 2.5]
    assert bench.aggregate_rate(10, 1, 2.0) == 5.0
