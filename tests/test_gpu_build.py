"""Neighbor-list builds of the plain case (one atom type, no exclusions, M > 5)
over several box sizes and densities: sorted pair sets equal the oracle's, and
two identical runs give bit-identical forces, coordinates, energies and rebuild
counts (the build's list order, hence every FP32 sum that follows it, is a
deterministic function of the coordinates)."""
import ctypes as C

import numpy as np
import pytest

from emdee_gb300.emdee import EmDee, MIXED
from mdrun import fcc_lattice

pytestmark = pytest.mark.gpu

CASES = [(4000, 0.85, 3), (32000, 0.8442, 5), (6912, 0.7, 9), (864, 0.8, 2)]


@pytest.fixture(scope="module")
def gpu():
    import emdee_gb300
    from emdee_gb300.build import build
    build()
    return emdee_gb300.load()


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
    out = dict(F0=F0, F1=lib.download(md, "forces", (N, 3)), R1=lib.download(md, "coordinates", (N, 3)),
               pairs0=pairs0, pairs1=lib.neighbor_pairs(md), builds=md.Builds, U=md.Energy.Potential,
               W=md.Virial.Total)
    lib.EmDee_destroy(C.byref(md))
    return out


@pytest.mark.parametrize("N,rho,seed", CASES)
def test_build_deterministic(gpu, N, rho, seed):
    a, b = run_case(gpu, N, rho, seed), run_case(gpu, N, rho, seed)
    for k in ("F0", "F1", "R1", "pairs0", "pairs1"):
        assert np.array_equal(a[k], b[k]), k
    assert a["builds"] == b["builds"] and a["builds"] > 1
    assert a["U"] == b["U"] and a["W"] == b["W"]


def test_build_pairs_vs_oracle(gpu, oracle_path):
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
