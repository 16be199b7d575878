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


# ---- replicas only: each rank steps its own system, nothing is exchanged ---------

def _replica(lib, index):
    """Replica `index` of a small Lennard-Jones batch (one per rank): 500 atoms,
    density and seed from the index, 20 velocity-Verlet steps with energies."""
    import ctypes as C

    import numpy as np
    from mdrun import fcc_lattice, velocity_verlet
    N, rho = 500, 0.75 + 0.05 * index
    L = (N / rho) ** (1.0 / 3.0)
    md = lib.system(1, 1, 2.5, 0.3, N)
    lib.EmDee_set_pair_model(md, 1, 1, lib.EmDee_pair_lj_cut(1.0, 1.0), 0.0)
    lib.upload(md, "box", np.array([L]))
    lib.upload(md, "coordinates", fcc_lattice(N, L, 0.05, 100 + index))
    lib.EmDee_random_momenta(C.byref(md), 1.2, True, 200 + index)
    velocity_verlet(lib, md, 0.005, 20, 1)
    R = lib.download(md, "coordinates", (N, 3))
    return (md.Energy.Potential, md.Virial.Total, md.Kinetic.Total, md.Builds, R.tobytes())


def _replica_rank(rank, world, port, so, out):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from emdee_gb300.emdee import EmDee
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = _replica(EmDee(so), rank)
    gathered = [None] * world
    dist.all_gather_object(gathered, mine)   # results only, for the check below
    out[rank] = gathered
    dist.destroy_process_group()


def test_replicas_per_rank_match_single_rank(oracle_path):
    """Two gloo ranks, one system each (the oracle library on the CPU): every
    rank's result equals, bit for bit, the same replica run by one process."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from emdee_gb300.emdee import EmDee
    world = 2
    out = mp.Manager().dict()
    mp.spawn(_replica_rank, args=(world, _free_port(), oracle_path, out), nprocs=world, join=True)
    lib = EmDee(oracle_path)
    single = [_replica(lib, r) for r in range(world)]
    assert single[0][0] != single[1][0]   # the replicas differ
    for r in range(world):
        assert out[r] == single
