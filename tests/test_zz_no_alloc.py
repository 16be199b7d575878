"""EmDee_boost_noalloc against EmDee_boost, through the C ABI.

EmDee_boost_noalloc serves callers that must not allocate device memory when
they call it: a process whose device memory belongs to another allocator (a
framework's caching allocator, a pool reserved at start-up), or a loop that
cannot afford the synchronization cudaMalloc/cudaFree may imply.  It runs the
same boost + kinetic-energy kernel as EmDee_boost on caller-owned device
arrays, with its reduction scratch in a fixed device array.  The sizes cover
one block, the full grid of 1184 blocks with its grid-stride loop (400,000
atoms: more than 1184 x 256 threads, so every per-block partial slot of the
scratch is written), and two calls in a row each.  This file is collected last
so that a run stopping at the first failure has already run every other test;
it passes both alone in a fresh process and after the rest of the suite.
"""
import ctypes as C
import math

import numpy as np
import pytest

from mdrun import fcc_lattice

pytestmark = pytest.mark.gpu

REL_TOL = 1e-13   # FP64 arithmetic, same kernel: results agree to rounding


def phi(x):
    """src/math.f90:230-237, as EmDee_boost evaluates it."""
    if abs(x) > 1e-4:
        return (1.0 - math.exp(-x)) / x
    return 1.0 + 0.5 * x * ((1.0 / 3.0) * x * (1.0 - 0.25 * x) - 1.0)


@pytest.fixture(scope="module")
def gpu():
    import emdee_gb300
    from emdee_gb300.build import build
    build()
    lib = emdee_gb300.load()
    lib.lib.EmDee_boost_noalloc.restype = C.c_int
    lib.lib.EmDee_boost_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_double,
                                            C.c_void_p, C.c_void_p]
    return lib


def _system(lib, N, masses):
    types = (np.arange(N) % 2) + 1
    L = (N / 0.8) ** (1.0 / 3.0)
    md = lib.system(1, 1, 2.5, 0.3, N, types, masses)
    for t in (1, 2):
        lib.EmDee_set_pair_model(md, t, t, lib.EmDee_pair_lj_cut(1.0, 1.0), 0.0)
    lib.upload(md, "box", np.array([L]))
    lib.upload(md, "coordinates", fcc_lattice(N, L, 0.05, 11))
    return md, types


@pytest.mark.parametrize("N,alpha,masses", [(200, 0.0, [1.0, 1.0]), (5000, 0.0, [1.0, 1.0]),
                                            (5000, 0.3, [1.0, 2.5]), (400000, 0.3, [1.0, 2.5])])
def test_noalloc_matches_boost_twice(gpu, N, alpha, masses):
    import torch
    dt = 0.005
    md, types = _system(gpu, N, masses)
    rng = np.random.default_rng(5)
    P0 = rng.normal(size=(N, 3))
    F0 = rng.normal(size=(N, 3)) * 10.0
    gpu.upload(md, "momenta", P0)
    gpu.upload(md, "forces", F0)
    CF = phi(alpha * dt) * dt
    CP = 1.0 - alpha * CF
    md.Options.Compute = True

    # existing entry point, twice
    ref_P, ref_K = [], []
    for _ in range(2):
        gpu.EmDee_boost(C.byref(md), 1.0, alpha, dt)
        ref_P.append(gpu.download(md, "momenta", (N, 3)))
        ref_K.append(2.0 * np.array(md.Kinetic.TransPart[:]))

    # allocation-free entry point on caller-owned device arrays, twice
    dev = torch.device("cuda")
    P = torch.tensor(P0, dtype=torch.float64, device=dev).contiguous()
    F = torch.tensor(F0, dtype=torch.float64, device=dev).contiguous()
    inv = None if masses == [1.0, 1.0] else torch.tensor(1.0 / np.array(masses)[types - 1], dtype=torch.float64,
                                                         device=dev)
    K = torch.zeros(3, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        rc = gpu.lib.EmDee_boost_noalloc(P.data_ptr(), F.data_ptr(), None if inv is None else inv.data_ptr(), N,
                                         CP, 1.0 * CF, K.data_ptr(), stream)
        assert rc == 0
        torch.cuda.synchronize()
        got_P, got_K = P.cpu().numpy(), K.cpu().numpy()
        assert np.max(np.abs(got_P - ref_P[call])) <= REL_TOL * np.max(np.abs(ref_P[call]))
        assert np.all(np.abs(got_K - ref_K[call]) <= REL_TOL * np.abs(ref_K[call]))
    gpu.EmDee_destroy(C.byref(md))


def test_noalloc_rejects_bad_arguments(gpu):
    assert gpu.lib.EmDee_boost_noalloc(None, None, None, 0, 1.0, 0.1, None, None) == 1
    assert gpu.lib.EmDee_boost_noalloc(None, None, None, -5, 1.0, 0.1, None, None) == 1
    # NULL arrays are refused before any CUDA call
    assert gpu.lib.EmDee_boost_noalloc(None, None, None, 100, 1.0, 0.1, None, None) == 1
