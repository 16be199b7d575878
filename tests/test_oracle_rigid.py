"""Physics checks of the oracle's rigid bodies (src/ArBee.f90 and the body
branches of src/EmDeeData.f90), on the SPC/E sample with each molecule a rigid
body: the equipartition of EmDee_random_momenta, the motion and torque
response of single calls, the convergence of the NO_SQUISH splitting to the
exact free rotation, and energy conservation of velocity Verlet with a time
step error that shrinks as dt^2.

The Coulomb model here is shifted_force(coul_damped), whose energy is
continuous at the cutoff; coul_sf is not, because EmDee_set_coul_model zeroes
its shift (src/EmDeeData.f90 modifier_setup after cutoff_setup), so its total
energy jumps whenever a pair crosses rc."""
import ctypes as C

import numpy as np
import pytest

from emdee_gb300.emdee import EmDee
from mdrun import load_golden, setup_water, velocity_verlet

COUL = "shifted_force(coul_damped)"


@pytest.fixture(scope="module")
def oracle(oracle_path):
    return EmDee(oracle_path)


@pytest.fixture(scope="module")
def water():
    return load_golden("nist_spce_sample.json")


def rigid_water(lib, w, mode=0):
    run = w["run"]
    md = setup_water(lib, w, COUL, rigid=True, coords_first=True)
    lib.EmDee_random_momenta(C.byref(md), run["kB"] * run["temp"], True, run["seed"])
    md.Options.RotationMode = mode
    return md


def masses(w):
    return np.array(w["mass"])[np.array(w["type"]) - 1]


def test_degrees_of_freedom_and_temperature(oracle, water):
    md = rigid_water(oracle, water)
    nmol = len(water["coordinates"]) // 3
    assert md.DoF == 6 * nmol - 3 and md.RotDoF == 3 * nmol
    T = 2.0 * md.Kinetic.Total / (md.DoF * water["run"]["kB"])
    assert abs(T - water["run"]["temp"]) < 1e-9 * water["run"]["temp"]
    Pcm = oracle.download(md, "bodymom", (nmol, 3)).sum(0)
    assert np.abs(Pcm).max() < 1e-12   # momenta of order 0.1


def test_body_geometry_is_preserved(oracle, water):
    md = rigid_water(oracle, water)
    N, L = len(water["coordinates"]), water["box"]

    def bonds(R):
        R = R.reshape(-1, 3, 3)
        out = []
        for a, b in ((0, 1), (0, 2), (1, 2)):
            d = R[:, b] - R[:, a]
            d -= L * np.round(d / L)
            out.append(np.linalg.norm(d, axis=1))
        return np.array(out)

    b0 = bonds(np.array(water["coordinates"]))
    velocity_verlet(oracle, md, 2.0, 5)
    assert np.abs(bonds(oracle.download(md, "coordinates", (N, 3))) - b0).max() < 1e-12
    q = oracle.download(md, "quaternions", (N // 3, 4))
    assert np.abs(np.linalg.norm(q, axis=1) - 1.0).max() < 1e-14


def test_motion_and_torque_response(oracle, water):
    """A short displacement moves atoms with the particle momenta; a short boost
    changes each body's momentum by F h and its angular momentum by tau h."""
    N = len(water["coordinates"])
    m = masses(water)
    h = 1e-3
    md = rigid_water(oracle, water)
    R0 = oracle.download(md, "coordinates", (N, 3))
    P0 = oracle.download(md, "momenta", (N, 3))
    oracle.EmDee_displace(C.byref(md), 1.0, 0.0, h)
    V = (oracle.download(md, "coordinates", (N, 3)) - R0) / h
    v0 = P0 / m[:, None]
    assert np.abs(V - v0).max() < 1e-3 * np.abs(v0).max()

    md = rigid_water(oracle, water)
    R = oracle.download(md, "coordinates", (N, 3)).reshape(-1, 3, 3)
    P0 = oracle.download(md, "momenta", (N, 3)).reshape(-1, 3, 3)
    F = oracle.download(md, "forces", (N, 3)).reshape(-1, 3, 3)
    mm = m.reshape(-1, 3)
    rcm = (mm[:, :, None] * R).sum(1) / mm.sum(1)[:, None]
    arm = R - rcm[:, None, :]
    tau = np.cross(arm, F).sum(1)
    oracle.EmDee_boost(C.byref(md), 1.0, 0.0, h)
    P1 = oracle.download(md, "momenta", (N, 3)).reshape(-1, 3, 3)
    dL = (np.cross(arm, P1).sum(1) - np.cross(arm, P0).sum(1)) / h
    assert np.abs(dL - tau).max() < 1e-9 * np.abs(tau).max()
    assert np.abs((P1 - P0).sum(1) / h - F.sum(1)).max() < 1e-9 * np.abs(F.sum(1)).max()


def test_no_squish_converges_to_exact_rotation(oracle, water):
    N = len(water["coordinates"])
    R = {}
    for mode in (0, 1, 10, 100):
        md = rigid_water(oracle, water, mode)
        oracle.EmDee_displace(C.byref(md), 1.0, 0.0, 20.0)
        R[mode] = oracle.download(md, "coordinates", (N, 3))
    e = [np.abs(R[n] - R[0]).max() for n in (1, 10, 100)]
    assert e[0] < 0.05 and e[1] < e[0] / 50 and e[2] < e[1] / 50   # second order in dt/n


@pytest.mark.parametrize("mode", [0, 3])
def test_energy_conservation_is_second_order(oracle, water, mode):
    mv = water["run"]["mvv2e"]
    spread = []
    for dt, steps in ((1.0, 16), (0.5, 32)):
        md = rigid_water(oracle, water, mode)
        E = []
        velocity_verlet(oracle, md, dt, steps, 1,
                        lambda s, m: E.append(mv * (m.Energy.Potential + m.Kinetic.Total)))
        spread.append(np.max(E) - np.min(E))
    assert spread[0] < 1.0                      # kcal/mol over 16 fs, total energy about -4.6e3
    assert 3.0 < spread[0] / spread[1] < 5.0    # dt^2
