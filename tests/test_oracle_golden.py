"""Pins the CPU oracle to the reference's own golden vectors:
the [U, W, U+K] triples of test/test_pair_lj_*.f90 (step 100, tolerance 1e-8,
test/common/contained.f90:81-87) on test/NIST_lj_sample.mol."""
import ctypes as C

import numpy as np
import pytest

from emdee_gb300.emdee import EmDee
from mdrun import initialize, load_golden, observables, setup_lj_sample, velocity_verlet

TOL = 1.0e-8  # test/common/declarations.f90:16


@pytest.fixture(scope="module")
def cfg():
    return load_golden("nist_lj_sample.json")


@pytest.fixture(scope="module")
def oracle(oracle_path):
    return EmDee(oracle_path)


def run_case(oracle, cfg, modifier, skin_width=None, threads=2, eshift=None):
    md = setup_lj_sample(oracle, cfg, modifier, skin_width, threads)
    if eshift is not None:
        oracle.lib.oracle_set_eshift.argtypes = [type(md), C.c_int, C.c_int, C.c_double]
        oracle.lib.oracle_set_eshift(md, 1, 1, eshift)
    initialize(oracle, md, cfg)
    run = cfg["run"]
    velocity_verlet(oracle, md, run["dt"], run["nsteps"], run["nprop"])
    return md


@pytest.mark.parametrize("threads", [1, 2])
def test_lj_cut(oracle, cfg, threads):
    md = run_case(oracle, cfg, "none", threads=threads)
    assert np.all(np.abs(observables(md) - cfg["expected"]["pair_lj_cut"]) < TOL)
    assert md.Builds == 5


@pytest.mark.parametrize("threads", [1, 2])
def test_lj_shifted_force(oracle, cfg, threads):
    md = run_case(oracle, cfg, "shifted_force", threads=threads)
    assert np.all(np.abs(observables(md) - cfg["expected"]["pair_lj_sf"]) < TOL)


def test_lj_square_smoothed(oracle, cfg):
    # The golden run switched over [Rc-1, Rc]: in the current interface the
    # modifier argument is the switching width (src/modelClass_nonbonded.f90:257),
    # so the same switch is EmDee_square_smoothed(model, 1.0).
    md = run_case(oracle, cfg, "square_smoothed", skin_width=1.0)
    assert np.all(np.abs(observables(md) - cfg["expected"]["pair_lj_smoothed"]) < TOL)


def test_lj_shifted_square_smoothed(oracle, cfg):
    # The golden run used the [Rc-1, Rc] switch with a shift of -E(Rc) that was
    # added inside the switching region only.  The forces depend on the shift
    # only inside that region, so the oracle's current arithmetic with
    # eshift = -E(Rc) must give the golden virial and kinetic energy exactly,
    # and the golden potential after the constant E(Rc) * n(r < Rm) that the
    # current convention adds outside the region.
    Rc, Rm = cfg["run"]["Rc"], cfg["run"]["Rc"] - 1.0
    Ec = 4.0 * (Rc ** -12 - Rc ** -6)
    md = run_case(oracle, cfg, "shifted_square_smoothed", skin_width=1.0, eshift=-Ec)
    R = oracle.download(md, "coordinates", (len(cfg["coordinates"]), 3))
    L = cfg["box"]
    d = R[:, None, :] - R[None, :, :]
    d -= L * np.round(d / L)
    r = np.sqrt((d ** 2).sum(-1))[np.triu_indices(len(R), 1)]
    inner = np.count_nonzero(r < Rm)
    U, W, H = observables(md)
    U_old = U + Ec * inner
    exp = cfg["expected"]["pair_lj_shifted_smoothed"]
    assert abs(W - exp[1]) < TOL
    assert abs(U_old - exp[0]) < TOL
    assert abs(H + Ec * inner - exp[2]) < TOL


def test_random_momenta_deterministic(oracle, cfg):
    a = run_case(oracle, cfg, "none", threads=2)
    b = run_case(oracle, cfg, "none", threads=2)
    N = len(cfg["coordinates"])
    assert np.array_equal(oracle.download(a, "momenta", (N, 3)), oracle.download(b, "momenta", (N, 3)))
