"""Bonds and angles on the GPU (emdee_gb300/csrc/bonded.cu) against the FP64
CPU oracle, on the SPC/E water sample (2250 atoms) made flexible with SPC/Fw
harmonic O-H bonds and H-O-H angles (src/EmDeeData.f90:443-550):

- bonded terms alone: forces, bond and angle energies and the virial agree with
  the oracle to FP64 round-off (the same statements, compiled without FMA
  contraction; per-atom sums in the reference's item order);
- with Lennard-Jones and coul_damped_smoothed, and with coul_long + Ewald
  (whose k-space discounts for bonds and angles enter the Coulomb energy, the
  virial through W(long) and the forces), in FP64 and mixed precision, within
  the tolerances of the water tests (mixed: FP32 pair arithmetic);
- 40 velocity-Verlet steps of flexible water (dt 0.5 fs): FP64 trajectories
  follow the oracle to round-off, with the same neighbor-list rebuilds."""
import ctypes as C
import os

import numpy as np
import pytest

from emdee_gb300.emdee import EmDee, FP64, MIXED
from mdrun import load_golden, setup_water, velocity_verlet

from test_oracle_ewald import ewald_water

pytestmark = pytest.mark.gpu

TOL_F = {FP64: 1e-11, MIXED: 3e-5}    # relative RMS force error
TOL_E = {FP64: 1e-11, MIXED: 4e-5}    # relative energy / virial error


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


def perturbed(w, seed, amp=0.05):
    rng = np.random.default_rng(seed)
    R = np.array(w["coordinates"])
    return R + rng.uniform(-amp, amp, R.shape)


def evaluate(lib, md, R):
    lib.upload(md, "coordinates", R)
    md.Options.Compute = True
    lib.EmDee_compute_forces(C.byref(md))
    N = len(R)
    e = md.Energy
    return lib.download(md, "forces", (N, 3)), np.array(
        [e.Potential, e.Dispersion, e.Coulomb, e.Bond, e.Angle, md.Virial.Total])


def compare(got, ref, tolF, tolE, label):
    (F, E), (Fr, Er) = got, ref
    rms = np.sqrt(((F - Fr) ** 2).mean() / (Fr ** 2).mean())
    rel = np.abs(E - Er) / np.maximum(np.abs(Er), 1e-300)
    print(label, "force rel RMS %.2e" % rms, "energies/virial rel", np.array2string(rel, precision=2))
    assert rms < tolF
    nz = np.abs(Er) > 0
    assert (rel[nz] < tolE).all() and (E[~nz] == 0).all()


@pytest.mark.parametrize("precision", [FP64, MIXED])
def test_bonded_only(gpu, oracle, water, precision):
    R = perturbed(water, 1)
    out = []
    for lib, prec in ((oracle, None), (gpu, precision)):
        md = setup_water(lib, water, "none", pair="none", precision=prec, flexible=True)
        out.append(evaluate(lib, md, R))
    compare(out[1], out[0], 1e-13, 1e-12, "bonded only")
    assert out[0][1][3] > 0 and out[0][1][4] > 0


@pytest.mark.parametrize("precision", [FP64, MIXED])
def test_flexible_water_damped(gpu, oracle, water, precision):
    R = perturbed(water, 2)
    out = []
    for lib, prec in ((oracle, None), (gpu, precision)):
        md = setup_water(lib, water, "coul_damped_smoothed", precision=prec, flexible=True)
        out.append(evaluate(lib, md, R))
    compare(out[1], out[0], TOL_F[precision], TOL_E[precision], "damped")


@pytest.mark.parametrize("precision", [FP64, MIXED])
def test_flexible_water_ewald(gpu, oracle, water, precision):
    R = perturbed(water, 3)
    out = []
    for lib, prec in ((oracle, None), (gpu, precision)):
        md = ewald_water(lib, water, 1e-6, precision=prec, flexible=True)
        out.append(evaluate(lib, md, R))
    compare(out[1], out[0], TOL_F[precision], TOL_E[precision], "ewald")


def test_flexible_water_md_fp64(gpu, oracle, water):
    N = len(water["coordinates"])
    run = water["run"]
    out = []
    for lib, prec in ((oracle, None), (gpu, FP64)):
        md = setup_water(lib, water, "coul_damped_smoothed", precision=prec, flexible=True)
        lib.EmDee_random_momenta(C.byref(md), run["kB"] * run["temp"], True, run["seed"])
        obs = []
        velocity_verlet(lib, md, 0.5, 40, 10, lambda s, m: s % 10 == 0 and obs.append(
            [m.Energy.Potential, m.Energy.Bond, m.Energy.Angle, m.Virial.Total, m.Kinetic.Total]))
        out.append((np.array(obs), lib.download(md, "coordinates", (N, 3)), md.Builds))
    (o0, R0, b0), (o1, R1, b1) = out
    rel = np.abs(o1 - o0) / np.abs(o0)
    print("flexible water MD: max rel obs error %.2e, max |dR| %.2e, builds %d %d" % (
        rel.max(), np.abs(R1 - R0).max(), b0, b1))
    assert rel.max() < 1e-9
    assert np.abs(R1 - R0).max() < 1e-9
    assert b0 == b1
