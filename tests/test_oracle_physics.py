"""Physics checks of the CPU oracle for the models the reference's tests leave
unpinned (softcore, every Coulomb model, every modifier): forces are minus the
gradient of the potential (central finite differences) and the virial is
sum_i r_i . F_i for forces from pair terms."""
import numpy as np
import pytest

from emdee_gb300.emdee import EmDee
from mdrun import COUL_MODELS, load_golden, setup_water


@pytest.fixture(scope="module")
def oracle(oracle_path):
    return EmDee(oracle_path)


@pytest.fixture(scope="module")
def water():
    return load_golden("nist_spce_sample.json")


def energy_at(lib, md, R):
    lib.upload(md, "coordinates", R)
    md.Options.Compute = True
    lib.EmDee_compute_forces(__import__("ctypes").byref(md))
    return md.Energy.Potential


MODELS = sorted(COUL_MODELS)


@pytest.mark.parametrize("coul", MODELS)
@pytest.mark.parametrize("pair", ["shifted_force", "softcore"])
def test_force_is_minus_gradient(oracle, water, coul, pair):
    N = 600
    md = setup_water(oracle, water, coul, pair, natoms=N)
    R0 = np.array(water["coordinates"][:N])
    F = oracle.download(md, "forces", (N, 3))
    h = 1e-5
    rng = np.random.default_rng(1)
    for a in rng.choice(N, size=6, replace=False):
        for d in range(3):
            Rp, Rm = R0.copy(), R0.copy()
            Rp[a, d] += h
            Rm[a, d] -= h
            fd = -(energy_at(oracle, md, Rp) - energy_at(oracle, md, Rm)) / (2 * h)
            assert abs(fd - F[a, d]) <= 1e-5 * max(1.0, abs(F[a, d])), (a, d, fd, F[a, d])


@pytest.mark.parametrize("coul", ["coul_damped", "coul_damped_square_smoothed", "coul_shifted_square_smoothed"])
def test_virial_is_sum_r_dot_f(oracle, water, coul):
    """W = sum over pairs of r_ij . F_ij; with the minimum-image pair vectors and
    no intramolecular terms this is sum_i r_i . F_i computed pair by pair."""
    N = 600
    md = setup_water(oracle, water, coul, natoms=N)
    R = np.array(water["coordinates"][:N])
    F = oracle.download(md, "forces", (N, 3))
    # W = -dU/d(ln L) for uniform scaling of all coordinates and the box
    L = water["box"]
    eps = 1e-6
    U = []
    for s in (1 + eps, 1 - eps):
        md2 = setup_water(oracle, water, coul, natoms=N)
        oracle.upload(md2, "box", np.array([L * s]))
        U.append(energy_at(oracle, md2, R * s))
    W_fd = -(U[0] - U[1]) / (2 * eps)
    assert abs(md.Virial.Total - W_fd) <= 1e-5 * max(1.0, abs(md.Virial.Total))
    assert np.isfinite(F).all()
