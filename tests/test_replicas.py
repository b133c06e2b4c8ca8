"""The replicas path of bench.py under two ranks on CPU (gloo): each rank
times its own batch, every rank learns the slowest rank's time, and the
whole-job throughput counts all ranks' solves over that time.  The data
path has no collective; only this timing uses one."""
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


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks(10.0 + 5.0 * rank, world, torch.device("cpu"))
        out[rank] = (ms, bench.replica_value(4096, world, ms))
    finally:
        dist.destroy_process_group()


def test_two_ranks_take_the_slowest_time():
    world, port = 2, _free_port()
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.start_processes(_rank, args=(world, port, out), nprocs=world, join=True, start_method="spawn")
        res = dict(out)
    assert res[0][0] == res[1][0] == 15.0
    assert res[0][1] == res[1][1] == pytest.approx(4096 * 2 / 0.015)


def test_single_rank_is_unchanged():
    assert bench.max_over_ranks(7.5, 1, None) == 7.5
    assert bench.replica_value(100, 1, 10.0) == pytest.approx(1e4)
