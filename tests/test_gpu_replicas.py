"""Replica batches (EmDee_replicas_*, no counterpart in the reference): every
replica advanced by the persistent batch kernel must follow the same
trajectory as the same system stepped alone -- by the CPU oracle through the
reference's loop (test/common/contained.f90:63-72) and by the GPU library's own
single-system path -- with the same neighbor-list rebuilds.  The batch is
deterministic: two runs of k steps equal one run of 2k steps bit for bit."""
import ctypes as C

import numpy as np
import pytest

from emdee_gb300.emdee import EmDee, MIXED
from emdee_gb300.workloads import fcc
from mdrun import velocity_verlet

pytestmark = pytest.mark.gpu

SPECS = [(2048, 0.85, 1.5), (256, 0.90, 0.8), (1000, 0.70, 2.0), (500, 0.80, 1.2), (1372, 0.88, 1.0),
         (300, 0.75, 1.9)]
SEED, DT, STEPS, NPROP = 86245, 0.005, 40, 10


@pytest.fixture(scope="module")
def gpu():
    import emdee_gb300
    from emdee_gb300.build import build
    build()
    return emdee_gb300.load()


@pytest.fixture(scope="module")
def oracle(oracle_path):
    return EmDee(oracle_path)


def make(lib, N, rho, T, k, precision=None):
    R, L = fcc(N, rho, 0.05, SEED + k)
    md = lib.system(1, 1, 2.5, 0.3, N)
    if precision is not None:
        lib.EmDee_set_precision(md, precision)
    lib.EmDee_set_pair_model(md, 1, 1, lib.EmDee_pair_lj_cut(1.0, 1.0), 0.0)
    lib.upload(md, "box", np.array([L]))
    lib.upload(md, "coordinates", R)
    lib.EmDee_random_momenta(C.byref(md), T, True, SEED + k)
    return md


def batch(gpu, mds):
    arr = (C.POINTER(type(mds[0])) * len(mds))(*[C.pointer(m) for m in mds])
    return gpu.lib.EmDee_replicas_create(len(mds), C.cast(arr, C.c_void_p)), arr


def state(lib, md, N):
    return (np.array([md.Energy.Potential, md.Virial.Total, md.Kinetic.Total]), md.Builds,
            lib.download(md, "coordinates", (N, 3)))


def test_replicas_match_oracle_and_single_system(gpu, oracle):
    mds = [make(gpu, N, rho, T, k, MIXED) for k, (N, rho, T) in enumerate(SPECS)]
    b, keep = batch(gpu, mds)
    gpu.lib.EmDee_replicas_run(b, STEPS, DT, NPROP)
    assert gpu.lib.EmDee_replicas_block_size(b) in (256, 512, 1024)
    assert gpu.lib.EmDee_replicas_pair_threads(b) in (1, 2)
    for k, (N, rho, T) in enumerate(SPECS):
        got = state(gpu, mds[k], N)
        for lib, prec in ((oracle, None), (gpu, MIXED)):
            md = make(lib, N, rho, T, k, prec)
            velocity_verlet(lib, md, DT, STEPS, NPROP)
            ref = state(lib, md, N)
            rel = np.abs(got[0] - ref[0]) / np.abs(ref[0])
            print(N, "batch vs", "oracle" if lib is oracle else "single GPU", "U, W, K rel", rel,
                  "max |dR|", np.abs(got[2] - ref[2]).max(), "builds", got[1], ref[1])
            assert rel.max() < 1e-4
            assert np.abs(got[2] - ref[2]).max() < 1e-4
            assert got[1] == ref[1]
    gpu.lib.EmDee_replicas_destroy(b)


def test_replicas_are_deterministic(gpu):
    out = []
    for split in (False, True):
        mds = [make(gpu, N, rho, T, k, MIXED) for k, (N, rho, T) in enumerate(SPECS[:3])]
        b, keep = batch(gpu, mds)
        if split:
            gpu.lib.EmDee_replicas_run(b, STEPS // 2, DT, NPROP)
            gpu.lib.EmDee_replicas_run(b, STEPS // 2, DT, NPROP)
        else:
            gpu.lib.EmDee_replicas_run(b, STEPS, DT, NPROP)
        out.append([(gpu.download(m, "coordinates", (N, 3)), gpu.download(m, "momenta", (N, 3)), m.Builds,
                     m.Energy.Potential) for m, (N, _, _) in zip(mds, SPECS[:3])])
        gpu.lib.EmDee_replicas_destroy(b)
    for a, c in zip(out[0], out[1]):
        assert np.array_equal(a[0], c[0]) and np.array_equal(a[1], c[1]) and a[2] == c[2] and a[3] == c[3]


def test_single_system_continues_after_batch(gpu, oracle):
    N, rho, T = SPECS[0]
    md = make(gpu, N, rho, T, 0, MIXED)
    b, keep = batch(gpu, [md])
    gpu.lib.EmDee_replicas_run(b, STEPS // 2, DT, NPROP)
    gpu.lib.EmDee_replicas_destroy(b)
    velocity_verlet(gpu, md, DT, STEPS // 2, NPROP)
    ref = make(oracle, N, rho, T, 0)
    velocity_verlet(oracle, ref, DT, STEPS, NPROP)
    assert abs(md.Energy.Potential - ref.Energy.Potential) < 1e-4 * abs(ref.Energy.Potential)
    assert np.abs(gpu.download(md, "coordinates", (N, 3)) - oracle.download(ref, "coordinates", (N, 3))).max() < 1e-4


def make_binary(lib, N, k, precision=None):
    """80:20 Lennard-Jones mixture (eps_AB 1.5, sigma_AB 0.8, eps_BB 0.5, sigma_BB 0.88), rho 1.2, T* 0.8."""
    R, L = fcc(N, 1.2, 0.05, SEED + k)
    types = np.where(np.random.default_rng(SEED + k).random(N) < 0.8, 1, 2)
    md = lib.system(1, 1, 2.5, 0.3, N, types, [1.0, 1.0])
    if precision is not None:
        lib.EmDee_set_precision(md, precision)
    lib.EmDee_set_pair_model(md, 1, 1, lib.EmDee_pair_lj_cut(1.0, 1.0), 0.0)
    lib.EmDee_set_pair_model(md, 2, 2, lib.EmDee_pair_lj_cut(0.5, 0.88), 0.0)
    lib.EmDee_set_pair_model(md, 1, 2, lib.EmDee_pair_lj_cut(1.5, 0.8), 0.0)
    lib.upload(md, "box", np.array([L]))
    lib.upload(md, "coordinates", R)
    lib.EmDee_random_momenta(C.byref(md), 0.8, True, SEED + k)
    return md


def test_replicas_binary_mixture(gpu, oracle):
    sizes = [864, 500, 1372]
    mds = [make_binary(gpu, N, k, MIXED) for k, N in enumerate(sizes)]
    b, keep = batch(gpu, mds)
    gpu.lib.EmDee_replicas_run(b, STEPS, 0.004, NPROP)
    for k, N in enumerate(sizes):
        got = state(gpu, mds[k], N)
        ref_md = make_binary(oracle, N, k)
        velocity_verlet(oracle, ref_md, 0.004, STEPS, NPROP)
        ref = state(oracle, ref_md, N)
        rel = np.abs(got[0] - ref[0]) / np.abs(ref[0])
        print(N, "binary batch vs oracle", rel, np.abs(got[2] - ref[2]).max(), got[1], ref[1])
        assert rel.max() < 1e-4 and np.abs(got[2] - ref[2]).max() < 1e-4 and got[1] == ref[1]
    gpu.lib.EmDee_replicas_destroy(b)
