"""Oracle checks of EmDee_verlet_step (src/EmDeeCode.f90:1107-1211), which the
reference's tests do not pin: the step moves the system exactly as the
reference's boost/displace/boost loop does, and its shadow Hamiltonian
(ShadowPotential + ShadowKinetic) is conserved much better than the plain
total energy, as a shadow Hamiltonian of velocity Verlet must be."""
import ctypes as C

import numpy as np
import pytest

from emdee_gb300.emdee import EmDee
from mdrun import initialize, load_golden, setup_lj_sample, setup_water, velocity_verlet


@pytest.fixture(scope="module")
def oracle(oracle_path):
    return EmDee(oracle_path)


def test_verlet_step_equals_boost_displace_boost(oracle):
    lj = load_golden("nist_lj_sample.json")
    N, dt = len(lj["coordinates"]), lj["run"]["dt"]
    a = setup_lj_sample(oracle, lj, "shifted_force")
    initialize(oracle, a, lj)
    b = setup_lj_sample(oracle, lj, "shifted_force")
    initialize(oracle, b, lj)
    for _ in range(25):
        oracle.EmDee_verlet_step(C.byref(a), dt)
    velocity_verlet(oracle, b, dt, 25)
    assert np.array_equal(oracle.download(a, "coordinates", (N, 3)), oracle.download(b, "coordinates", (N, 3)))
    assert np.array_equal(oracle.download(a, "momenta", (N, 3)), oracle.download(b, "momenta", (N, 3)))
    assert a.Energy.Potential == b.Energy.Potential and a.Virial.Total == b.Virial.Total


def test_shadow_hamiltonian_lj(oracle):
    lj = load_golden("nist_lj_sample.json")
    md = setup_lj_sample(oracle, lj, "shifted_force")
    initialize(oracle, md, lj)
    E, H = [], []
    for _ in range(150):
        oracle.EmDee_verlet_step(C.byref(md), lj["run"]["dt"])
        E.append(md.Energy.Potential + md.Kinetic.Total)
        H.append(md.Energy.ShadowPotential + md.Kinetic.ShadowKinetic)
    assert np.std(H) < np.std(E) / 10


def test_shadow_hamiltonian_rigid(oracle):
    w = load_golden("nist_spce_sample.json")
    run = w["run"]
    md = setup_water(oracle, w, "shifted_force(coul_damped)", rigid=True, coords_first=True)
    oracle.EmDee_random_momenta(C.byref(md), run["kB"] * run["temp"], True, run["seed"])
    E, H = [], []
    for _ in range(25):
        oracle.EmDee_verlet_step(C.byref(md), 1.0)
        E.append(md.Energy.Potential + md.Kinetic.Total)
        H.append(md.Energy.ShadowPotential + md.Kinetic.ShadowKinetic)
    assert np.std(H) < 0.75 * np.std(E)
    assert md.Kinetic.ShadowRotational != 0.0
