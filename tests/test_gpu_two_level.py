"""Two-level neighbor lists (EmDee_set_outer_skin, emdee_gb300/csrc/neighbor.cu):
outer lists of radius rc + skin + delta are built only when the two largest
displacements since the last outer build reach delta; every other rebuild is the
pair kernel filtering them into the lists the reference builds
(src/neighbor_lists.f90:199-300).  After every rebuild of a mixed-precision
Lennard-Jones run the pair set must equal the FP64 oracle's pair set for the same
coordinates, bit for bit, and the forces must match the oracle's within the
mixed-precision bound; the rebuild schedule must equal that of the same run with
single-level lists.  Cases: an outer skin that covers several rebuilds, one too
small to cover any (every rebuild is an outer build), and a box of 37,044 atoms."""
import ctypes as C

import numpy as np
import pytest

from emdee_gb300.emdee import EmDee, MIXED
from mdrun import fcc_lattice

pytestmark = pytest.mark.gpu

FORCE_RMS_MIXED = 1.0e-5


@pytest.fixture(scope="module")
def gpu():
    import emdee_gb300
    from emdee_gb300.build import build
    build()
    return emdee_gb300.load()


@pytest.fixture(scope="module")
def oracle(oracle_path):
    return EmDee(oracle_path)


def fcc_box(N, rho, seed):
    L = (N / rho) ** (1.0 / 3.0)
    return fcc_lattice(N, L, 0.05, seed), L


def system(lib, R, L, outer=None, precision=None, momenta=True):
    md = lib.system(1, 1, 2.5, 0.3, len(R))
    if precision is not None:
        lib.EmDee_set_precision(md, precision)
    if outer is not None:
        lib.EmDee_set_outer_skin(md, outer)
    lib.EmDee_set_pair_model(md, 1, 1, lib.EmDee_pair_lj_cut(1.0, 1.0), 0.0)
    lib.upload(md, "box", np.array([L]))
    lib.upload(md, "coordinates", R)
    if momenta:
        lib.EmDee_random_momenta(C.byref(md), 1.5, True, 86245)
    return md


def step(lib, md, dt=0.005):
    md.Options.Compute = True
    lib.EmDee_boost(C.byref(md), 1.0, 0.0, 0.5 * dt)
    lib.EmDee_displace(C.byref(md), 1.0, 0.0, dt)
    lib.EmDee_boost(C.byref(md), 1.0, 0.0, 0.5 * dt)


def rel_rms(a, b):
    return float(np.sqrt(np.sum((a - b) ** 2) / np.sum(b ** 2)))


def run(gpu, oracle, N, rho, outer, steps, seed=11):
    """Steps a two-level system and a single-level one side by side; after every
    rebuild compares the two-level pair set and forces with a fresh oracle build
    at the same coordinates.  Returns (builds, outer builds, rebuilds checked)."""
    R, L = fcc_box(N, rho, seed)
    two = system(gpu, R, L, outer, MIXED)
    one = system(gpu, R, L, None, MIXED)   # default: single-level lists
    builds, checked = two.Builds, 0
    for _ in range(steps):
        step(gpu, two)
        step(gpu, one)
        assert two.Builds == one.Builds
        if two.Builds != builds:
            builds = two.Builds
            X = gpu.download(two, "coordinates", (N, 3))
            ref = system(oracle, X, L, momenta=False)
            assert np.array_equal(gpu.neighbor_pairs(two), oracle.neighbor_pairs(ref))
            F = gpu.download(two, "forces", (N, 3))
            assert rel_rms(F, oracle.download(ref, "forces", (N, 3))) < FORCE_RMS_MIXED
            assert abs(two.Energy.Potential - ref.Energy.Potential) < 1e-5 * abs(ref.Energy.Potential)
            checked += 1
    assert abs(two.Energy.Potential - one.Energy.Potential) < 1e-5 * abs(one.Energy.Potential)
    assert gpu.EmDee_outer_builds(one) == 0
    return two.Builds, gpu.EmDee_outer_builds(two), checked


def test_outer_lists_cover_several_rebuilds(gpu, oracle):
    builds, outer, checked = run(gpu, oracle, 4000, 0.85, 0.6, 160)
    print("builds", builds, "outer builds", outer, "rebuilds checked", checked)
    assert checked >= 10
    assert 1 <= outer <= builds // 2 + 1   # most rebuilds filtered the outer lists


def test_outer_skin_too_small_to_cover(gpu, oracle):
    builds, outer, checked = run(gpu, oracle, 4000, 0.85, 0.01, 60)
    print("builds", builds, "outer builds", outer, "rebuilds checked", checked)
    assert checked >= 3
    assert outer == builds   # every rebuild (and the first build) is an outer build


def test_larger_box(gpu, oracle):
    builds, outer, checked = run(gpu, oracle, 37044, 0.8442, 0.45, 40)
    print("builds", builds, "outer builds", outer, "rebuilds checked", checked)
    assert checked >= 3
    assert 1 <= outer < builds
