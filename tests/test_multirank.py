"""The N > 1 path of bench.py on CPU ranks (gloo, world size 2): every rank
gets the slowest rank's time, and the whole-job rate counts the units of all
ranks over that time (replicas only: no data moves between ranks)."""
import os
import socket
import sys

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = [40.0, 50.0][rank]                 # rank 1 is the slower one
    rate, ms_max = bench.job_rate(1000, ms, world, "cpu")
    out[rank] = (rate, ms_max, bench.max_over_ranks(rank + 0.5, world, "cpu"))
    dist.barrier()
    dist.destroy_process_group()


def test_job_rate_two_ranks():
    world = 2
    out = mp.Manager().dict()
    mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
    for r in range(world):
        rate, ms_max, mx = out[r]
        assert ms_max == 50.0
        assert rate == pytest.approx(world * 1000 / 0.050)
        assert mx == 1.5


def test_job_rate_one_rank():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.job_rate(1000, 40.0, 1, "cpu") == (1000 / 0.040, 40.0)
