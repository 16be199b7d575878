"""GPU parity of the CUDA library against the CPU oracle and the reference's
golden vectors, called through the C ABI."""
import ctypes as C

import numpy as np
import pytest

from emdee_gb300.emdee import EmDee, FP64, MIXED
from mdrun import fcc_lattice, initialize, load_golden, observables, setup_lj_sample, velocity_verlet

pytestmark = pytest.mark.gpu

TOL = 1.0e-8               # golden tolerance, test/common/declarations.f90:16
FORCE_RMS_MIXED = 1.0e-5   # FP32 pair math vs FP64 oracle, relative RMS of the force field
ENERGY_REL_MIXED = 1.0e-5  # relative error of the total potential energy
VIRIAL_REL_MIXED = 5.0e-5  # relative error of the total virial (a sum with strong cancellation)


@pytest.fixture(scope="module")
def gpu():
    import emdee_gb300
    from emdee_gb300.build import build
    build()
    return emdee_gb300.load()


@pytest.fixture(scope="module")
def oracle(oracle_path):
    return EmDee(oracle_path)


@pytest.fixture(scope="module")
def nist():
    return load_golden("nist_lj_sample.json")


def rel_rms(a, b):
    return float(np.sqrt(np.sum((a - b) ** 2) / np.sum(b ** 2)))


@pytest.mark.parametrize("modifier,skin_width,key", [
    ("none", None, "pair_lj_cut"),
    ("shifted_force", None, "pair_lj_sf"),
    ("square_smoothed", 1.0, "pair_lj_smoothed"),
])
def test_golden_fp64(gpu, nist, modifier, skin_width, key):
    md = setup_lj_sample(gpu, nist, modifier, skin_width, precision=FP64)
    initialize(gpu, md, nist)
    run = nist["run"]
    velocity_verlet(gpu, md, run["dt"], run["nsteps"], run["nprop"])
    obs = observables(md)
    assert np.all(np.abs(obs - nist["expected"][key]) < TOL), obs - nist["expected"][key]
    assert md.Builds == 5


def _init_pair(lib, cfg, precision, modifier="none", skin_width=None):
    md = setup_lj_sample(lib, cfg, modifier, skin_width, precision=precision)
    initialize(lib, md, cfg)
    return md


def test_neighbor_pairs_identical_nist(gpu, oracle, nist):
    a = _init_pair(gpu, nist, MIXED)
    b = _init_pair(oracle, nist, None)
    pa, pb = gpu.neighbor_pairs(a), oracle.neighbor_pairs(b)
    assert len(pa) > 0
    assert np.array_equal(pa, pb)


@pytest.mark.parametrize("modifier,skin_width", [("none", None), ("shifted", None), ("shifted_force", None),
                                                 ("square_smoothed", 1.0), ("shifted_square_smoothed", 1.0)])
def test_forces_energy_virial_nist(gpu, oracle, nist, modifier, skin_width):
    N = len(nist["coordinates"])
    ref = _init_pair(oracle, nist, None, modifier, skin_width)
    Fo = oracle.download(ref, "forces", (N, 3))
    d64 = _init_pair(gpu, nist, FP64, modifier, skin_width)
    F64 = gpu.download(d64, "forces", (N, 3))
    assert rel_rms(F64, Fo) < 1e-13
    assert abs(d64.Energy.Potential - ref.Energy.Potential) < 1e-9 * abs(ref.Energy.Potential)
    assert abs(d64.Virial.Total - ref.Virial.Total) < 1e-9 * max(1.0, abs(ref.Virial.Total))
    d32 = _init_pair(gpu, nist, MIXED, modifier, skin_width)
    F32 = gpu.download(d32, "forces", (N, 3))
    errs = (rel_rms(F32, Fo), abs(d32.Energy.Potential / ref.Energy.Potential - 1),
            abs(d32.Virial.Total - ref.Virial.Total) / abs(ref.Virial.Total))
    print("mixed precision errors (force rel. RMS, energy, virial):", errs)
    assert errs[0] < FORCE_RMS_MIXED
    assert errs[1] < ENERGY_REL_MIXED
    assert errs[2] < VIRIAL_REL_MIXED


def _fcc_system(lib, N, rho, seed, precision, rc=2.5, skin=0.3):
    L = (N / rho) ** (1.0 / 3.0)
    R = fcc_lattice(N, L, 0.05, seed)
    md = lib.system(1, 1, rc, skin, N)
    if precision is not None:
        lib.EmDee_set_precision(md, precision)
    lib.EmDee_set_pair_model(md, 1, 1, lib.EmDee_pair_lj_cut(1.0, 1.0), 0.0)
    lib.upload(md, "box", np.array([L]))
    lib.upload(md, "coordinates", R)
    lib.EmDee_random_momenta(C.byref(md), 1.5, True, 86245)
    return md


@pytest.mark.parametrize("N,rho", [(4000, 0.85), (256, 0.9), (2048, 0.7)])
def test_fcc_pairs_and_forces(gpu, oracle, N, rho):
    ref = _fcc_system(oracle, N, rho, 7, None)
    dev = _fcc_system(gpu, N, rho, 7, MIXED)
    assert np.array_equal(gpu.neighbor_pairs(dev), oracle.neighbor_pairs(ref))
    Fo = oracle.download(ref, "forces", (N, 3))
    F32 = gpu.download(dev, "forces", (N, 3))
    assert rel_rms(F32, Fo) < FORCE_RMS_MIXED


def test_trajectory_fp64_tracks_oracle(gpu, oracle):
    """Config-0 shape (N=4000, rho=0.85, T*=1.5, dt=0.005): 200 FP64 steps."""
    N = 4000
    ref = _fcc_system(oracle, N, 0.85, 3, None)
    dev = _fcc_system(gpu, N, 0.85, 3, FP64)
    for md, lib in ((ref, oracle), (dev, gpu)):
        velocity_verlet(lib, md, 0.005, 200, 1)
    assert dev.Builds == ref.Builds
    assert abs(dev.Energy.Potential - ref.Energy.Potential) < 1e-8 * abs(ref.Energy.Potential)
    assert abs(dev.Kinetic.Total - ref.Kinetic.Total) < 1e-8 * abs(ref.Kinetic.Total)
    Ro = oracle.download(ref, "coordinates", (N, 3))
    Rd = gpu.download(dev, "coordinates", (N, 3))
    assert np.max(np.abs(Ro - Rd)) < 1e-9


def test_destroy_and_recreate(gpu, oracle):
    """A system created after another was destroyed starts from clean state."""
    ref = _fcc_system(oracle, 2048, 0.8, 9, None)
    Fo = oracle.download(ref, "forces", (2048, 3))
    for _ in range(3):
        md = _fcc_system(gpu, 2048, 0.8, 9, MIXED)
        F = gpu.download(md, "forces", (2048, 3))
        assert rel_rms(F, Fo) < FORCE_RMS_MIXED
        gpu.EmDee_destroy(C.byref(md))
