"""The two neighbor-list builds of the plain case (one atom type, no exclusions,
M > 5) against each other and against the oracle: the cell-parallel build (one
warp per cell, the default) and the thread-per-atom build (EMDEE_BUILD=thread)
must write the same entries in the same order, so the mixed-precision forces,
whose FP32 sums follow the list order, are bit-identical; and the pair sets are
the oracle's.  The thread-per-atom build runs in a child process (the choice is
read once per process)."""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

from emdee_gb300.emdee import EmDee, MIXED
from mdrun import fcc_lattice

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CASES = [(4000, 0.85, 3), (32000, 0.8442, 5), (6912, 0.7, 9), (864, 0.8, 2)]


def run_case(lib, N, rho, seed, steps=30):
    """Forces after the initial build and after `steps` velocity-Verlet steps
    (several rebuilds), energies every step."""
    L = (N / rho) ** (1.0 / 3.0)
    md = lib.system(1, 1, 2.5, 0.3, N)
    lib.EmDee_set_precision(md, MIXED)
    lib.EmDee_set_pair_model(md, 1, 1, lib.EmDee_pair_lj_cut(1.0, 1.0), 0.0)
    lib.upload(md, "box", np.array([L]))
    lib.upload(md, "coordinates", fcc_lattice(N, L, 0.05, seed))
    lib.EmDee_random_momenta(C.byref(md), 1.5, True, seed)
    F0 = lib.download(md, "forces", (N, 3))
    pairs0 = lib.neighbor_pairs(md)
    for _ in range(steps):
        md.Options.Compute = True
        lib.EmDee_boost(C.byref(md), 1.0, 0.0, 0.0025)
        lib.EmDee_displace(C.byref(md), 1.0, 0.0, 0.005)
        lib.EmDee_boost(C.byref(md), 1.0, 0.0, 0.0025)
    F1 = lib.download(md, "forces", (N, 3))
    R1 = lib.download(md, "coordinates", (N, 3))
    return dict(F0=F0, F1=F1, R1=R1, pairs0=pairs0, pairs1=lib.neighbor_pairs(md), builds=md.Builds,
                U=md.Energy.Potential, W=md.Virial.Total)


def _child(out):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import emdee_gb300
    lib = emdee_gb300.load()
    res = {}
    for N, rho, seed in CASES:
        r = run_case(lib, N, rho, seed)
        for k, v in r.items():
            res["%d_%s" % (N, k)] = v
    np.savez(out, **res)


@pytest.fixture(scope="module")
def gpu():
    import emdee_gb300
    from emdee_gb300.build import build
    build()
    return emdee_gb300.load()


@pytest.fixture(scope="module")
def thread_build(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("build") / "thread.npz")
    env = dict(os.environ, EMDEE_BUILD="thread")
    code = "import sys; sys.path.insert(0, %r); import test_gpu_build as t; t._child(%r)" % (
        os.path.join(ROOT, "tests"), out)
    subprocess.run([sys.executable, "-c", code], env=env, check=True, cwd=ROOT)
    return np.load(out)


@pytest.mark.parametrize("N,rho,seed", CASES)
def test_cell_build_matches_thread_build(gpu, thread_build, N, rho, seed):
    r = run_case(gpu, N, rho, seed)
    for k in ("F0", "F1", "R1", "pairs0", "pairs1"):
        assert np.array_equal(r[k], thread_build["%d_%s" % (N, k)]), k
    assert r["builds"] == thread_build["%d_builds" % N] and r["builds"] > 1
    assert r["U"] == thread_build["%d_U" % N] and r["W"] == thread_build["%d_W" % N]


def test_cell_build_pairs_vs_oracle(gpu, oracle_path):
    oracle = EmDee(oracle_path)
    for N, rho, seed in CASES:
        L = (N / rho) ** (1.0 / 3.0)
        R = fcc_lattice(N, L, 0.05, seed)
        sets = []
        for lib in (gpu, oracle):
            md = lib.system(1, 1, 2.5, 0.3, N)
            lib.EmDee_set_pair_model(md, 1, 1, lib.EmDee_pair_lj_cut(1.0, 1.0), 0.0)
            lib.upload(md, "box", np.array([L]))
            lib.upload(md, "coordinates", R)
            sets.append(lib.neighbor_pairs(md))
        assert np.array_equal(sets[0], sets[1]), N
