"""Edge cases of the GPU path against the oracle: a single atom, two atoms within
the cut-off (checked against the analytic Lennard-Jones force too), a dilute
gas whose neighbor lists are empty, and a dense cluster in a large box (many
atoms per cell, most tiles empty), in FP64 and mixed precision, through a few
velocity-Verlet steps."""
import ctypes as C

import numpy as np
import pytest

from emdee_gb300.emdee import EmDee, FP64, MIXED
from mdrun import velocity_verlet

pytestmark = pytest.mark.gpu

TOL = {FP64: 1e-12, MIXED: 1e-4}   # mixed: FP32 pair arithmetic, forces with cancellation


@pytest.fixture(scope="module")
def gpu():
    import emdee_gb300
    from emdee_gb300.build import build
    build()
    return emdee_gb300.load()


@pytest.fixture(scope="module")
def oracle(oracle_path):
    return EmDee(oracle_path)


def system(lib, R, L, precision):
    md = lib.system(1, 1, 2.5, 0.3, len(R))
    if precision is not None:
        lib.EmDee_set_precision(md, precision)
    lib.EmDee_set_pair_model(md, 1, 1, lib.EmDee_pair_lj_cut(1.0, 1.0), 0.0)
    lib.upload(md, "box", np.array([L]))
    lib.upload(md, "coordinates", np.asarray(R, dtype=np.float64))
    return md


def run(lib, R, L, precision, steps=10):
    N = len(R)
    md = system(lib, R, L, precision)
    F0 = lib.download(md, "forces", (N, 3))
    lib.EmDee_random_momenta(C.byref(md), 0.5, True, 7)
    velocity_verlet(lib, md, 0.002, steps, 1)
    return F0, np.array([md.Energy.Potential, md.Virial.Total, md.Kinetic.Total]), \
        lib.download(md, "coordinates", (N, 3)), md.Builds


def compare(got, ref, precision, label):
    (F, E, R, b), (Fr, Er, Rr, br) = got, ref
    scale = max(np.abs(Fr).max(), 1e-30)
    print(label, "max |dF|/max|F| %.2e" % (np.abs(F - Fr).max() / scale), "E", E, Er, "builds", b, br)
    assert np.abs(F - Fr).max() <= TOL[precision] * scale + 1e-300
    # a single atom has no degrees of freedom left after the centre-of-mass
    # correction of EmDee_random_momenta: both libraries give NaN momenta there
    assert np.allclose(E, Er, rtol=TOL[precision], atol=1e-12, equal_nan=True)
    assert np.array_equal(np.isnan(R), np.isnan(Rr))
    assert np.nan_to_num(np.abs(R - Rr)).max() < 1e3 * TOL[precision]
    assert b == br


@pytest.mark.parametrize("precision", [FP64, MIXED])
def test_single_atom(gpu, oracle, precision):
    R = [[1.0, 2.0, 3.0]]
    got, ref = run(gpu, R, 10.0, precision), run(oracle, R, 10.0, None)
    assert np.all(got[0] == 0.0) and got[1][0] == 0.0 and got[1][1] == 0.0
    compare(got, ref, precision, "single atom")


@pytest.mark.parametrize("precision", [FP64, MIXED])
def test_two_atoms(gpu, oracle, precision):
    r = 1.12
    R = [[2.0, 2.0, 2.0], [2.0 + r, 2.0, 2.0]]
    md = system(gpu, R, 12.0, precision)
    F = gpu.download(md, "forces", (2, 3))
    f = 24.0 * (2.0 / r ** 13 - 1.0 / r ** 7)   # -dU/dr of 4 (r^-12 - r^-6)
    # near the minimum the force is a small difference of two large terms: bound the
    # error by the size of the terms (FP32 pair arithmetic in mixed precision)
    tol = (1e-12 if precision == FP64 else 2e-5) * 24.0 * (2.0 / r ** 13 + 1.0 / r ** 7)
    assert abs(F[1, 0] - f) <= tol and abs(F[0, 0] + f) <= tol
    got, ref = run(gpu, R, 12.0, precision), run(oracle, R, 12.0, None)
    compare(got, ref, precision, "two atoms")


@pytest.mark.parametrize("precision", [FP64, MIXED])
def test_dilute_gas_empty_lists(gpu, oracle, precision):
    g = np.stack(np.meshgrid(np.arange(4), np.arange(4), np.arange(4), indexing="ij"), -1).reshape(-1, 3)
    R = g * 6.0 + 1.0                            # 64 atoms 6 sigma apart: nothing within rc + skin
    got, ref = run(gpu, R, 24.0, precision), run(oracle, R, 24.0, None)
    assert got[1][0] == 0.0
    assert gpu.neighbor_pairs(system(gpu, R, 24.0, precision)).shape[0] == 0
    compare(got, ref, precision, "dilute gas")


@pytest.mark.parametrize("precision", [FP64, MIXED])
def test_dense_cluster_in_large_box(gpu, oracle, precision):
    rng = np.random.default_rng(5)
    g = np.stack(np.meshgrid(np.arange(5), np.arange(5), np.arange(5), indexing="ij"), -1).reshape(-1, 3)
    R = 10.0 + 1.05 * g + rng.uniform(-0.05, 0.05, g.shape)   # 125 atoms in one corner of a 40 sigma box
    got, ref = run(gpu, R, 40.0, precision), run(oracle, R, 40.0, None)
    pairs = gpu.neighbor_pairs(system(gpu, R, 40.0, precision))
    ref_pairs = oracle.neighbor_pairs(system(oracle, R, 40.0, None))
    assert np.array_equal(pairs, ref_pairs)
    compare(got, ref, precision, "dense cluster")


@pytest.mark.parametrize("precision", [FP64, MIXED])
@pytest.mark.parametrize("N", [2, 8, 32, 33, 100])
def test_small_random_systems(gpu, oracle, precision, N):
    """Few atoms per tile (blocks narrower than the halo's cell count)."""
    rng = np.random.default_rng(N)
    R = rng.uniform(0.0, 12.0, (N, 3))
    g, o = system(gpu, R, 12.0, precision), system(oracle, R, 12.0, None)
    assert np.array_equal(gpu.neighbor_pairs(g), oracle.neighbor_pairs(o))
    F, Fo = gpu.download(g, "forces", (N, 3)), oracle.download(o, "forces", (N, 3))
    scale = max(np.abs(Fo).max(), 1e-30)
    assert np.abs(F - Fo).max() <= (1e-12 if precision == FP64 else 1e-4) * scale
