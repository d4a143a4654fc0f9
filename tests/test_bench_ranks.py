"""The replica aggregation of bench.py under torch.distributed, on CPU with two
gloo ranks: every rank gets the slowest rank's time, and the job rate counts the
units of all ranks over that time."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = bench._max_over_ranks(10.0 * (rank + 1), torch.device("cpu"), world)
    out[rank] = (ms, bench._job_rate(1000, 5, world, ms))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    world = 2
    port = _free_port()
    with mp.get_context("spawn").Manager() as mgr:   # no fork of this multi-threaded process
        out = mgr.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0] == res[1]
    ms, rate = res[0]
    assert ms == 20.0
    assert rate == pytest.approx(1000 * 5 * 2 / 0.020)


def test_one_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench._max_over_ranks(12.5, None, 1) == 12.5
    assert bench._job_rate(10, 3, 1, 1000.0) == pytest.approx(30.0)
