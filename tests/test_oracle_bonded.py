"""Checks of the oracle's bonded terms (EmDee_add_bond / EmDee_add_angle with
bond_harmonic and angle_harmonic, src/EmDeeData.f90:443-550), which the
reference's tests leave unpinned:

- with only bonds and angles, the forces are minus the gradient of the energy
  (central differences) and the virial is minus the derivative of the energy
  under a uniform scaling of the box and the coordinates;
- the harmonic energies equal k/2 (r - r0)^2 and k/2 (theta - theta0)^2 summed
  over the molecules (numpy);
- with coul_long, the k-space discounts of bonds (O-H) and angles (H...H) make the
  Coulomb energy of flexible SPC/E water equal to that of the same molecules as
  rigid bodies, whose intramolecular pairs are discounted at set-up
  (src/modelClass_kspace.f90:180-230);
- dihedrals only exclude their atom pairs (the reference never evaluates them);
- the errors of the reference for wrong arguments."""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

from emdee_gb300.emdee import EmDee
from mdrun import SPCFW, load_golden, setup_water

from test_oracle_ewald import ewald_water


@pytest.fixture(scope="module")
def oracle(oracle_path):
    return EmDee(oracle_path)


@pytest.fixture(scope="module")
def water():
    return load_golden("nist_spce_sample.json")


def perturbed(w, n, seed, amp=0.05):
    rng = np.random.default_rng(seed)
    return np.array(w["coordinates"][:n]) + rng.uniform(-amp, amp, (n, 3))


def energy(lib, md, R=None, L=None):
    if L is not None:
        lib.upload(md, "box", [L])
    if R is not None:
        lib.upload(md, "coordinates", R)
    md.Options.Compute = True
    lib.EmDee_compute_forces(C.byref(md))
    return md.Energy.Potential


def bonded_only(lib, w, n, seed):
    md = setup_water(lib, w, "none", pair="none", natoms=n, flexible=True)
    R = perturbed(w, n, seed)
    energy(lib, md, R)
    return md, R


def test_bonded_forces_are_minus_gradient(oracle, water):
    n = 90
    md, R0 = bonded_only(oracle, water, n, 1)
    F = oracle.download(md, "forces", (n, 3))
    assert np.abs(F).max() > 1e-3
    h = 1e-6
    for a in range(0, n, 7):
        for d in range(3):
            Rp, Rm = R0.copy(), R0.copy()
            Rp[a, d] += h
            Rm[a, d] -= h
            fd = -(energy(oracle, md, Rp) - energy(oracle, md, Rm)) / (2 * h)
            assert abs(fd - F[a, d]) < 1e-6 * np.abs(F).max() + 1e-9


def test_bonded_energies_and_virial(oracle, water):
    n = 90
    md, R = bonded_only(oracle, water, n, 2)
    run, L = water["run"], water["box"]
    Eb = Ea = 0.0
    for m in range(n // 3):
        o, h1, h2 = R[3 * m], R[3 * m + 1], R[3 * m + 2]
        a, b = h1 - o, h2 - o
        a -= L * np.round(a / L)
        b -= L * np.round(b / L)
        for v in (a, b):
            Eb += 0.5 * SPCFW["kb"] / run["mvv2e"] * (np.linalg.norm(v) - SPCFW["r0"]) ** 2
        th = np.arccos(a @ b / np.linalg.norm(a) / np.linalg.norm(b))
        Ea += 0.5 * SPCFW["ka"] / run["mvv2e"] * (th - SPCFW["theta0"]) ** 2
    assert abs(md.Energy.Bond - Eb) < 1e-12 * Eb
    assert abs(md.Energy.Angle - Ea) < 1e-12 * Ea
    assert md.Energy.Potential == pytest.approx(Eb + Ea, rel=1e-13)
    W = md.Virial.Total
    s = 1e-6   # W = -dU/ds for R -> s R, L -> s L
    Up = energy(oracle, md, R * (1 + s), L * (1 + s))
    Um = energy(oracle, md, R * (1 - s), L * (1 - s))
    assert abs(W + (Up - Um) / (2 * s)) < 1e-6 * abs(W)


def test_kspace_discounts_match_rigid_molecules(oracle, water):
    n = 600
    flex = ewald_water(oracle, water, 1e-6, natoms=n, flexible=True)
    rigid = ewald_water(oracle, water, 1e-6, natoms=n, rigid=True)
    assert flex.Energy.Coulomb == pytest.approx(rigid.Energy.Coulomb, rel=1e-11)
    # the bonded energies are those of the SPC/E geometry under SPC/Fw parameters
    assert flex.Energy.Bond > 0 and flex.Energy.Angle > 0


def test_dihedrals_only_exclude(oracle, water):
    n = 12
    pairs = ((1, 2), (1, 4), (1, 5), (2, 4), (2, 5), (4, 5))

    def dihedral(lib, md):
        lib.EmDee_add_dihedral(md, 1, 2, 4, 5, lib.EmDee_dihedral_none())

    def ignore(lib, md):
        for i, j in pairs:
            lib.EmDee_ignore_pair(md, i, j)

    plain, dih, ref = [setup_water(oracle, water, "coul_damped_smoothed", natoms=n, exclusions=False, hook=h)
                       for h in (None, dihedral, ignore)]
    for md in (plain, dih, ref):
        energy(oracle, md)
    assert dih.Energy.Potential == ref.Energy.Potential
    assert dih.Energy.Potential != plain.Energy.Potential
    assert dih.Energy.Bond == 0.0 and dih.Energy.Angle == 0.0


@pytest.mark.parametrize("call,message", [
    ("lib.EmDee_add_bond(md, 1, 99, lib.EmDee_bond_harmonic(1.0, 1.0))", "atom index out of range"),
    ("lib.EmDee_add_bond(md, 1, 2, lib.EmDee_angle_harmonic(1.0, 1.0))", "must be a bond model"),
    ("lib.EmDee_add_angle(md, 1, 2, 3, lib.EmDee_bond_harmonic(1.0, 1.0))", "must be an angle model"),
    ("lib.EmDee_add_bond(md, 1, 2, None)", "a valid model must be provided"),
])
def test_bonded_errors(oracle_path, call, message):
    code = "\n".join([
        "import sys; sys.path.insert(0, %r)" % os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
        "from emdee_gb300.emdee import EmDee",
        "lib = EmDee(%r)" % oracle_path,
        "md = lib.system(1, 1, 2.5, 0.3, 4)",
        call,
    ])
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True)
    assert r.returncode == 1 and message in r.stderr
