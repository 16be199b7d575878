"""GPU parity of coul_long with the Ewald k-space solver (src/coul_long.f90,
src/kspace_ewald.f90, src/modelClass_kspace.f90) against the CPU oracle:
SPC/E water as rigid bodies and as free atoms with exclusions, and the rock-salt
lattice whose total Coulomb energy gives the Madelung constant.  The k-space
kernels run in FP64 in both precision modes; mixed mode differs from the oracle
only through the FP32 real-space pair terms."""
import ctypes as C

import numpy as np
import pytest

from emdee_gb300.emdee import EmDee, FP64, MIXED
from mdrun import load_golden, observables, velocity_verlet
from test_oracle_ewald import MADELUNG_NACL, ewald_water, rock_salt

pytestmark = pytest.mark.gpu

FP64_REL = 1e-11
MIXED_FORCE_RMS = 1e-5
MIXED_ENERGY = 2e-5


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
def water():
    return load_golden("nist_spce_sample.json")


def rel_rms(a, b):
    return float(np.sqrt(np.sum((a - b) ** 2) / np.sum(b ** 2)))


@pytest.mark.parametrize("rigid", [True, False])
def test_ewald_water_fp64(gpu, oracle, water, rigid):
    N = len(water["coordinates"])
    ref = ewald_water(oracle, water, 1e-6, rigid=rigid)
    dev = ewald_water(gpu, water, 1e-6, rigid=rigid, precision=FP64)
    Fo, Fg = oracle.download(ref, "forces", (N, 3)), gpu.download(dev, "forces", (N, 3))
    assert rel_rms(Fg, Fo) < FP64_REL
    for a, b in ((dev.Energy.Potential, ref.Energy.Potential), (dev.Energy.Coulomb, ref.Energy.Coulomb),
                 (dev.Virial.Total, ref.Virial.Total)):
        assert abs(a - b) <= FP64_REL * abs(b), (a, b)


def test_ewald_water_mixed(gpu, oracle, water):
    N = len(water["coordinates"])
    ref = ewald_water(oracle, water, 1e-6, rigid=True)
    dev = ewald_water(gpu, water, 1e-6, rigid=True, precision=MIXED)
    Fo, Fg = oracle.download(ref, "forces", (N, 3)), gpu.download(dev, "forces", (N, 3))
    assert rel_rms(Fg, Fo) < MIXED_FORCE_RMS
    assert abs(dev.Energy.Potential - ref.Energy.Potential) <= MIXED_ENERGY * abs(ref.Energy.Potential)
    # the total virial is a small difference of Coulomb terms of the size of the
    # Coulomb energy (real space, k space, rigid bodies): bound it on that scale
    assert abs(dev.Virial.Total - ref.Virial.Total) <= MIXED_ENERGY * abs(ref.Energy.Coulomb)


@pytest.mark.parametrize("precision", [FP64, MIXED])
def test_madelung_constant_gpu(gpu, oracle, precision):
    md, N = rock_salt(gpu, 8, 1e-8, precision)
    ref, _ = rock_salt(oracle, 8, 1e-8)
    assert abs(-md.Energy.Coulomb / (N / 2) - MADELUNG_NACL) < 2e-6
    tol = FP64_REL if precision == FP64 else MIXED_ENERGY
    assert abs(md.Energy.Coulomb - ref.Energy.Coulomb) <= tol * abs(ref.Energy.Coulomb)


def test_ewald_rigid_trajectory(gpu, oracle, water):
    mv = water["run"]["mvv2e"]
    N = len(water["coordinates"])
    run = water["run"]
    out = []
    for lib, prec in ((oracle, None), (gpu, FP64)):
        md = ewald_water(lib, water, 1e-6, rigid=True, precision=prec)
        lib.EmDee_random_momenta(C.byref(md), run["kB"] * run["temp"], True, run["seed"])
        obs = []
        velocity_verlet(lib, md, 1.0, 6, 3, lambda s, m: obs.append(observables(m, mv)))
        out.append((obs[-1], lib.download(md, "coordinates", (N, 3))))
    (o_obs, o_R), (g_obs, g_R) = out
    assert np.all(np.abs(g_obs - o_obs) <= 1e-9 * np.abs(o_obs))
    assert np.abs(g_R - o_R).max() < 1e-9
