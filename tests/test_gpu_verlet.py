"""GPU parity of EmDee_verlet_step (src/EmDeeCode.f90:1107-1211) with the CPU
oracle, for free atoms (NIST LJ sample) and rigid bodies (SPC/E water, exact
and NO_SQUISH rotation), including the shadow-Hamiltonian terms; and the GPU
step against the GPU's own boost/displace/boost loop (the same arithmetic, so
the same trajectory bit for bit)."""
import ctypes as C

import numpy as np
import pytest

from emdee_gb300.emdee import EmDee, FP64, MIXED
from mdrun import initialize, load_golden, setup_lj_sample, setup_water, velocity_verlet

pytestmark = pytest.mark.gpu

FP64_REL = 1e-10


@pytest.fixture(scope="module")
def gpu():
    import emdee_gb300
    from emdee_gb300.build import build
    build()
    return emdee_gb300.load()


@pytest.fixture(scope="module")
def oracle(oracle_path):
    return EmDee(oracle_path)


def fields(md):
    return np.array([md.Energy.Potential, md.Energy.ShadowPotential, md.Kinetic.Total, md.Kinetic.ShadowKinetic,
                     md.Kinetic.ShadowRotational, md.Virial.Total])


def close(a, b, tol):
    return np.all(np.abs(a - b) <= tol * np.maximum(np.abs(b), 1e-300)), (a, b)


def test_verlet_lj_fp64(gpu, oracle):
    lj = load_golden("nist_lj_sample.json")
    N, dt = len(lj["coordinates"]), lj["run"]["dt"]
    out = []
    for lib, prec in ((oracle, None), (gpu, FP64)):
        md = setup_lj_sample(lib, lj, "shifted_force", precision=prec)
        initialize(lib, md, lj)
        for _ in range(30):
            lib.EmDee_verlet_step(C.byref(md), dt)
        out.append((fields(md), lib.download(md, "coordinates", (N, 3)), md.Builds))
    ok, info = close(out[1][0], out[0][0], FP64_REL)
    assert ok, info
    assert np.abs(out[1][1] - out[0][1]).max() < 1e-10
    assert out[1][2] == out[0][2]


@pytest.mark.parametrize("precision", [FP64, MIXED])
def test_verlet_matches_boost_displace_boost_on_gpu(gpu, precision):
    lj = load_golden("nist_lj_sample.json")
    N, dt = len(lj["coordinates"]), lj["run"]["dt"]
    a = setup_lj_sample(gpu, lj, "shifted_force", precision=precision)
    initialize(gpu, a, lj)
    b = setup_lj_sample(gpu, lj, "shifted_force", precision=precision)
    initialize(gpu, b, lj)
    for _ in range(20):
        gpu.EmDee_verlet_step(C.byref(a), dt)
    velocity_verlet(gpu, b, dt, 20)
    assert np.array_equal(gpu.download(a, "coordinates", (N, 3)), gpu.download(b, "coordinates", (N, 3)))
    assert np.array_equal(gpu.download(a, "momenta", (N, 3)), gpu.download(b, "momenta", (N, 3)))


@pytest.mark.parametrize("mode", [0, 3])
def test_verlet_rigid_fp64(gpu, oracle, mode):
    w = load_golden("nist_spce_sample.json")
    run, N = w["run"], len(w["coordinates"])
    out = []
    for lib, prec in ((oracle, None), (gpu, FP64)):
        md = setup_water(lib, w, "shifted_force(coul_damped)", precision=prec, rigid=True, coords_first=True)
        lib.EmDee_random_momenta(C.byref(md), run["kB"] * run["temp"], True, run["seed"])
        md.Options.RotationMode = mode
        for _ in range(6):
            lib.EmDee_verlet_step(C.byref(md), 1.0)
        out.append((fields(md), lib.download(md, "coordinates", (N, 3)), lib.download(md, "quaternions", (N // 3, 4))))
    ok, info = close(out[1][0], out[0][0], 1e-9)
    assert ok, info
    assert np.abs(out[1][1] - out[0][1]).max() < 1e-9
    assert np.abs(out[1][2] - out[0][2]).max() < 1e-10


def test_verlet_without_energies(gpu):
    lj = load_golden("nist_lj_sample.json")
    md = setup_lj_sample(gpu, lj, "shifted_force", precision=FP64)
    initialize(gpu, md, lj)
    md.Options.Compute = False
    gpu.EmDee_verlet_step(C.byref(md), lj["run"]["dt"])
    assert not md.Kinetic.UpToDate and not md.Energy.UpToDate
