"""Physics checks of the oracle's Ewald solver (coul_long + kspace_ewald,
src/coul_long.f90, src/kspace_ewald.f90, src/modelClass_kspace.f90), which
the reference's tests leave unpinned:

- the Madelung constant of rock salt from the total Coulomb energy (real
  space + reciprocal space + self energy), to the accuracy the A&S 7.1.26
  erfc polynomial allows (src/math.f90:685-691, |error| <= 1.5e-7);
- forces equal minus the gradient of the total energy (central differences),
  on SPC/E water as free atoms with intramolecular exclusions (exclusions are
  not discounted in k-space, as in the reference, and the test holds anyway);
- the total Coulomb energy of rigid SPC/E water does not depend on the
  accuracy setting beyond the erfc polynomial's error."""
import ctypes as C

import numpy as np
import pytest

from emdee_gb300.emdee import EmDee
from mdrun import add_flexible_water, load_golden

MADELUNG_NACL = 1.747564594633182   # nearest-neighbour convention


@pytest.fixture(scope="module")
def oracle(oracle_path):
    return EmDee(oracle_path)


@pytest.fixture(scope="module")
def water():
    return load_golden("nist_spce_sample.json")


def rock_salt(lib, n, acc, precision=None):
    g = np.stack(np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij"), -1).reshape(-1, 3)
    types = 1 + (g.sum(1) % 2)
    md = lib.system(1, 1, 3.5, 0.4, len(g), types, [1.0, 1.0])
    if precision is not None:
        lib.EmDee_set_precision(md, precision)
    for t in (1, 2):
        lib.EmDee_set_pair_model(md, t, t, lib.EmDee_pair_none(), 1.0)
    lib.EmDee_set_coul_model(md, lib.EmDee_coul_long())
    lib.EmDee_set_kspace_model(md, lib.EmDee_kspace_ewald(acc))
    lib.upload(md, "charges", np.where(types == 1, 1.0, -1.0))
    lib.upload(md, "box", [float(n)])
    lib.upload(md, "coordinates", g.astype(np.float64))
    return md, len(g)


def ewald_water(lib, w, acc, natoms=None, rigid=False, precision=None, rc=10.0, flexible=False):
    run = w["run"]
    N = natoms or len(w["coordinates"])
    md = lib.system(1, 1, rc, 2.0, N, w["type"][:N], w["mass"], w["molecule"][:N] if rigid else None)
    if precision is not None:
        lib.EmDee_set_precision(md, precision)
    for i, (eps, sig) in enumerate(zip(w["epsilon"], w["sigma"])):
        p = lib.EmDee_pair_none() if eps == 0.0 else lib.EmDee_shifted_force(
            lib.EmDee_pair_lj_cut(eps / run["mvv2e"], sig))
        lib.EmDee_set_pair_model(md, i + 1, i + 1, p, run["kCoul"])
    lib.EmDee_set_coul_model(md, lib.EmDee_coul_long())
    lib.EmDee_set_kspace_model(md, lib.EmDee_kspace_ewald(acc))
    if flexible:
        add_flexible_water(lib, md, N, run["mvv2e"])
    elif not rigid:
        first = {}
        for a, m in enumerate(w["molecule"][:N]):
            first.setdefault(m, []).append(a + 1)
        for atoms in first.values():
            for x in range(len(atoms)):
                for y in range(x + 1, len(atoms)):
                    lib.EmDee_ignore_pair(md, atoms[x], atoms[y])
    lib.upload(md, "charges", w["charge"][:N])
    lib.upload(md, "box", [w["box"]])
    lib.upload(md, "coordinates", np.array(w["coordinates"][:N]))
    return md


@pytest.mark.parametrize("acc", [1e-6, 1e-8])
def test_madelung_constant(oracle, acc):
    md, N = rock_salt(oracle, 8, acc)
    M = -md.Energy.Coulomb / (N / 2)
    assert abs(M - MADELUNG_NACL) < 2e-6
    # pure 1/r interactions: the Coulomb virial equals the Coulomb energy
    assert abs(md.Virial.Total - md.Energy.Coulomb) < 1e-9 * abs(md.Energy.Coulomb)


def test_ewald_force_is_minus_gradient(oracle, water):
    n = 300
    md = ewald_water(oracle, water, 1e-6, natoms=n)
    R0 = np.array(water["coordinates"][:n])
    F = oracle.download(md, "forces", (n, 3))

    def U(R):
        oracle.upload(md, "coordinates", R)
        md.Options.Compute = True
        oracle.EmDee_compute_forces(C.byref(md))
        return md.Energy.Potential

    h = 1e-5
    rng = np.random.default_rng(3)
    for a in rng.choice(n, 5, replace=False):
        for d in range(3):
            Rp, Rm = R0.copy(), R0.copy()
            Rp[a, d] += h
            Rm[a, d] -= h
            fd = -(U(Rp) - U(Rm)) / (2 * h)
            assert abs(fd - F[a, d]) < 1e-4 * np.abs(F).max()


def test_energy_does_not_depend_on_accuracy(oracle, water):
    E = [ewald_water(oracle, water, acc, rigid=True).Energy.Coulomb for acc in (1e-7, 1e-9)]
    assert abs(E[0] - E[1]) < 1e-5 * abs(E[1])
