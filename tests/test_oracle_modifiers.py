"""Oracle checks of the linear-r switching modifiers EmDee_smoothed and
EmDee_shifted_smoothed (src/modelClass_nonbonded.f90:133-190, set-up at
:245-296, evaluation in src/apply_modifier.f90), which no reference test
exercises:

* two atoms at distances across the switching range against a numpy
  restatement of the switch (E -> (E + eshift) G(u), W -> W G + E WG with
  u = (r - Rm)/(rc - Rm), G = 1 + u^3 (15u - 6u^2 - 10));
* the energy and the force vanish continuously at the cut-off;
* forces are minus the gradient of the energy (central differences) on the
  800-atom NIST Lennard-Jones sample.
"""
import ctypes as C

import numpy as np
import pytest

from emdee_gb300.emdee import EmDee
from mdrun import load_golden

RC, SKIN_LIST = 2.5, 0.3


@pytest.fixture(scope="module")
def oracle(oracle_path):
    return EmDee(oracle_path)


def lj(r, eps=1.0, sig=1.0):
    sr6 = (sig / r) ** 6
    return 4 * eps * sr6 * (sr6 - 1), 24 * eps * sr6 * (2 * sr6 - 1)


def switched(r, width, shifted):
    """E and W (= -r dE/dr) of lj_cut with the linear-r switch of width `width`."""
    Rm = RC - width
    eshift = -0.5 * (lj(Rm)[0] + lj(RC)[0]) if shifted else 0.0
    E, W = lj(r)
    E = E + eshift
    if r > Rm:
        factor = 1.0 / (RC - Rm)
        u = factor * r - factor * Rm
        G = 1 + u ** 3 * (15 * u - 6 * u * u - 10)
        WG = -30 * u * u * (2 * u - u * u - 1) * factor * r
        W, E = W * G + E * WG, E * G
    return E, W


def modifier(lib, name, width):
    base = lib.EmDee_pair_lj_cut(1.0, 1.0)
    return {"smoothed": lib.EmDee_smoothed, "shifted_smoothed": lib.EmDee_shifted_smoothed}[name](base, width)


def two_atoms(lib, name, width, r):
    md = lib.system(1, 1, RC, SKIN_LIST, 2)
    lib.EmDee_set_pair_model(md, 1, 1, modifier(lib, name, width), 0.0)
    lib.upload(md, "box", np.array([20.0]))
    lib.upload(md, "coordinates", np.array([[5.0, 5.0, 5.0], [5.0 + r, 5.0, 5.0]]))
    md.Options.Compute = True
    lib.EmDee_compute_forces(C.byref(md))
    F = lib.download(md, "forces", (2, 3))
    return md.Energy.Potential, md.Virial.Total, F


@pytest.mark.parametrize("name", ["smoothed", "shifted_smoothed"])
@pytest.mark.parametrize("width", [0.5, 1.0])
def test_two_atom_switch(oracle, name, width):
    for r in (1.0, 1.3, RC - width - 0.05, RC - width + 1e-3, RC - 0.6 * width, RC - 0.1 * width, RC - 1e-4):
        E, W, F = two_atoms(oracle, name, width, r)
        Ee, We = switched(r, width, name == "shifted_smoothed")
        assert abs(E - Ee) <= 1e-12 * max(1.0, abs(Ee)), (r, E, Ee)
        assert abs(W - We) <= 1e-11 * max(1.0, abs(We)), (r, W, We)
        # F on atom 1 along -x: W/r^2 * (x1 - x2)
        assert abs(F[0, 0] + We / r) <= 1e-11 * max(1.0, abs(We / r)), (r, F[0, 0])
        assert abs(F[0, 0] + F[1, 0]) <= 1e-13 * max(1.0, abs(F[0, 0]))


@pytest.mark.parametrize("name", ["smoothed", "shifted_smoothed"])
def test_continuous_at_cutoff(oracle, name):
    E_in, W_in, _ = two_atoms(oracle, name, 1.0, RC - 1e-6)
    E_out, W_out, _ = two_atoms(oracle, name, 1.0, RC + 1e-6)
    assert E_out == 0.0 and W_out == 0.0
    assert abs(E_in) < 1e-15 and abs(W_in) < 1e-9


def energy_at(lib, md, R):
    lib.upload(md, "coordinates", R)
    md.Options.Compute = True
    lib.EmDee_compute_forces(C.byref(md))
    return md.Energy.Potential


@pytest.mark.parametrize("name", ["smoothed", "shifted_smoothed"])
def test_force_is_minus_gradient_nist(oracle, name):
    cfg = load_golden("nist_lj_sample.json")
    run, N = cfg["run"], len(cfg["coordinates"])
    md = oracle.system(2, 1, run["Rc"], run["skin"], N, cfg["type"], cfg["mass"])
    oracle.EmDee_set_pair_model(md, 1, 1, modifier(oracle, name, 1.0), 0.0)
    R0 = np.array(cfg["coordinates"])
    oracle.upload(md, "box", np.array([cfg["box"]]))
    oracle.upload(md, "coordinates", R0)
    F = oracle.download(md, "forces", (N, 3))
    h = 1e-5   # the energy (~-4e3) carries 1e-12 rounding: h balances it against O(h^2)
    for a in np.random.default_rng(5).choice(N, size=8, replace=False):
        for d in range(3):
            Rp, Rm = R0.copy(), R0.copy()
            Rp[a, d] += h
            Rm[a, d] -= h
            fd = -(energy_at(oracle, md, Rp) - energy_at(oracle, md, Rm)) / (2 * h)
            assert abs(fd - F[a, d]) <= 2e-6 * max(1.0, abs(F[a, d])), (a, d, fd, F[a, d])
