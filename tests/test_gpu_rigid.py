"""GPU parity of rigid bodies (src/ArBee.f90, body branches of
src/EmDeeData.f90) against the CPU oracle: the SPC/E sample with each molecule
a rigid body, as test/test_rigid_body_exact.f90 (exact free rotation) and
test/test_rigid_body_miller.f90 (NO_SQUISH) set it up, integrated with
velocity Verlet through the C ABI.  FP64 mode follows the oracle's arithmetic
statement by statement; the transcendental functions of the exact rotation
(sin, cos, atan, sqrt) may differ from the host's by an ulp, so trajectories
are compared with a relative bound of 1e-9.  Mixed mode is compared with the
bounds the free-atom tests state."""
import ctypes as C

import numpy as np
import pytest

from emdee_gb300.emdee import EmDee, FP64, MIXED
from mdrun import load_golden, observables, setup_water, velocity_verlet

pytestmark = pytest.mark.gpu

FP64_TRAJ = 1.0e-9
MIXED_ENERGY = 2.0e-5
MIXED_COORD = 1.0e-5   # in Angstrom, after a few steps


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


def rigid(lib, w, coul, mode, precision=None, miller=False):
    run = w["run"]
    md = setup_water(lib, w, coul, precision=precision, rigid=True, coords_first=not miller)
    lib.EmDee_random_momenta(C.byref(md), run["kB"] * run["temp"], True, run["seed"])
    md.Options.RotationMode = mode
    return md


BODY_ITEMS = [("centersOfMass", 3), ("quaternions", 4), ("quatmom", 4), ("angmom", 3), ("bodymom", 3),
              ("bodyforces", 3), ("torques", 3), ("inertia", 3)]


def snapshot(lib, md, N):
    nb = N // 3
    out = {k: lib.download(md, k, (nb, w)) for k, w in BODY_ITEMS}
    out["coordinates"] = lib.download(md, "coordinates", (N, 3))
    out["momenta"] = lib.download(md, "momenta", (N, 3))
    out["forces"] = lib.download(md, "forces", (N, 3))
    return out


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("coul", ["coul_sf", "shifted_force(coul_damped)"])
@pytest.mark.parametrize("mode,miller", [(0, False), (1, True), (3, False)])
def test_rigid_water_fp64(gpu, oracle, water, coul, mode, miller):
    N = len(water["coordinates"])
    mv = water["run"]["mvv2e"]
    ref = rigid(oracle, water, coul, mode, miller=miller)
    dev = rigid(gpu, water, coul, mode, FP64, miller=miller)
    assert (dev.DoF, dev.RotDoF) == (ref.DoF, ref.RotDoF)
    assert abs(dev.Kinetic.Total - ref.Kinetic.Total) <= 1e-12 * ref.Kinetic.Total
    assert abs(dev.Kinetic.Rotational - ref.Kinetic.Rotational) <= 1e-12 * ref.Kinetic.Rotational
    s0, g0 = snapshot(oracle, ref, N), snapshot(gpu, dev, N)
    for k in s0:
        assert rel(g0[k], s0[k]) < 1e-12, k
    o_obs, g_obs = [], []
    velocity_verlet(oracle, ref, 1.0, 10, 5, lambda s, m: o_obs.append(observables(m, mv)))
    velocity_verlet(gpu, dev, 1.0, 10, 5, lambda s, m: g_obs.append(observables(m, mv)))
    s1, g1 = snapshot(oracle, ref, N), snapshot(gpu, dev, N)
    for k in s1:
        assert rel(g1[k], s1[k]) < FP64_TRAJ, k
    for a, b in zip(g_obs[4::5], o_obs[4::5]):
        assert np.all(np.abs(a - b) <= FP64_TRAJ * np.abs(b)), (a, b)
    assert dev.Builds == ref.Builds


@pytest.mark.parametrize("mode", [0, 3])
def test_rigid_water_mixed(gpu, oracle, water, mode):
    coul = "shifted_force(coul_damped)"
    N = len(water["coordinates"])
    ref = rigid(oracle, water, coul, mode)
    dev = rigid(gpu, water, coul, mode, MIXED)
    velocity_verlet(oracle, ref, 1.0, 10, 5)
    velocity_verlet(gpu, dev, 1.0, 10, 5)
    Ro, Rg = oracle.download(ref, "coordinates", (N, 3)), gpu.download(dev, "coordinates", (N, 3))
    assert np.abs(Rg - Ro).max() < MIXED_COORD
    for a, b in ((dev.Energy.Potential, ref.Energy.Potential), (dev.Kinetic.Total, ref.Kinetic.Total),
                 (dev.Virial.Total, ref.Virial.Total)):
        assert abs(a - b) <= MIXED_ENERGY * abs(b), (a, b)


def test_rigid_uploads(gpu, oracle, water):
    """Momenta uploaded into a rigid system become body momenta (src/EmDeeData.f90:157-189);
    coordinates uploaded into an initialized system rebuild the bodies when AutoBodyUpdate is on."""
    coul = "shifted_force(coul_damped)"
    N = len(water["coordinates"])
    ref = rigid(oracle, water, coul, 0)
    dev = rigid(gpu, water, coul, 0, FP64)
    velocity_verlet(oracle, ref, 1.0, 3)
    velocity_verlet(gpu, dev, 1.0, 3)
    P = oracle.download(ref, "momenta", (N, 3)) * 1.1
    R = oracle.download(ref, "coordinates", (N, 3))
    for lib, md in ((oracle, ref), (gpu, dev)):
        md.Options.AutoBodyUpdate = True
        lib.upload(md, "coordinates", R)
        lib.upload(md, "momenta", P)
    assert abs(dev.Kinetic.Total - ref.Kinetic.Total) <= 1e-12 * ref.Kinetic.Total
    assert abs(dev.Kinetic.Rotational - ref.Kinetic.Rotational) <= 1e-12 * ref.Kinetic.Rotational
    s, g = snapshot(oracle, ref, N), snapshot(gpu, dev, N)
    for k in s:
        assert rel(g[k], s[k]) < 1e-11, k
    velocity_verlet(oracle, ref, 1.0, 3)
    velocity_verlet(gpu, dev, 1.0, 3)
    assert rel(gpu.download(dev, "coordinates", (N, 3)), oracle.download(ref, "coordinates", (N, 3))) < FP64_TRAJ
