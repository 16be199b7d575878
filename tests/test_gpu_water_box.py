"""The 4096-molecule rigid-water workload (12288 atoms, coul_damped_smoothed
with damping 0.2/A and skin width 1 A, rc 10 A, neighbor skin 1 A, SPC/E
geometry and charges on a simple-cubic lattice with random orientations,
1 g/cm3, 300 K, dt 1 fs, exact rigid-body rotation) on the GPU against the
FP64 CPU oracle.  Each result's error against the oracle is printed and
bounded: FP64 mode follows the oracle to round-off; mixed mode (FP32 pair
arithmetic) stays within the stated tolerances over 100 steps, where the
trajectories have started to separate chaotically.  The mixed-mode force bound
is 3e-5 relative RMS here (1e-5 for Lennard-Jones): each Coulomb pair term
carries FP32 rounding of a few 1e-7, and the net force on an atom is a small
difference of such terms."""
import ctypes as C
import os

import numpy as np
import pytest

from emdee_gb300.emdee import EmDee, FP64, MIXED
from emdee_gb300.workloads import KB, MVV2E, setup_water_box
from mdrun import velocity_verlet

pytestmark = pytest.mark.gpu

NMOL, SEED, STEPS, EVERY = 4096, 86245, 100, 25


@pytest.fixture(scope="module")
def gpu():
    import emdee_gb300
    from emdee_gb300.build import build
    build()
    return emdee_gb300.load()


@pytest.fixture(scope="module")
def reference(oracle_path):
    lib = EmDee(oracle_path)
    md = setup_water_box(lib, NMOL, SEED, threads=os.cpu_count() or 1)
    N = 3 * NMOL
    out = {"F0": lib.download(md, "forces", (N, 3)), "pairs": lib.neighbor_pairs(md),
           "E0": np.array([md.Energy.Potential, md.Virial.Total])}
    lib.EmDee_random_momenta(C.byref(md), KB * 300.0, True, SEED)
    obs = []
    velocity_verlet(lib, md, 1.0, STEPS, EVERY, lambda s, m: s % EVERY == 0 and obs.append(
        [m.Energy.Potential, m.Virial.Total, m.Kinetic.Total]))
    out["obs"] = np.array(obs)
    out["R"] = lib.download(md, "coordinates", (N, 3))
    out["builds"] = md.Builds
    return out


def run_gpu(gpu, precision):
    N = 3 * NMOL
    md = setup_water_box(gpu, NMOL, SEED, precision=precision)
    out = {"F0": gpu.download(md, "forces", (N, 3)), "pairs": gpu.neighbor_pairs(md),
           "E0": np.array([md.Energy.Potential, md.Virial.Total])}
    gpu.EmDee_random_momenta(C.byref(md), KB * 300.0, True, SEED)
    obs = []
    velocity_verlet(gpu, md, 1.0, STEPS, EVERY, lambda s, m: s % EVERY == 0 and obs.append(
        [m.Energy.Potential, m.Virial.Total, m.Kinetic.Total]))
    out["obs"] = np.array(obs)
    out["R"] = gpu.download(md, "coordinates", (N, 3))
    out["builds"] = md.Builds
    return out


def errors(dev, ref):
    f = float(np.sqrt(np.sum((dev["F0"] - ref["F0"]) ** 2) / np.sum(ref["F0"] ** 2)))
    e0 = np.abs(dev["E0"] - ref["E0"]) / np.abs(ref["E0"])
    traj = np.abs(dev["obs"] - ref["obs"]) / np.abs(ref["obs"])
    dR = float(np.abs(dev["R"] - ref["R"]).max())
    print("force rel RMS %.2e | U0, W0 rel %.2e %.2e | U, W, K rel at steps %s: %s | max |dR| %.2e A" %
          (f, e0[0], e0[1], list(range(EVERY, STEPS + 1, EVERY)), np.array2string(traj.max(1), precision=2), dR))
    return f, e0, traj, dR


def test_water_box_fp64(gpu, reference):
    dev = run_gpu(gpu, FP64)
    f, e0, traj, dR = errors(dev, reference)
    assert np.array_equal(dev["pairs"], reference["pairs"])
    assert f < 1e-11 and e0.max() < 1e-11
    assert traj.max() < 1e-8 and dR < 1e-7
    assert dev["builds"] == reference["builds"]


def test_water_box_mixed(gpu, reference):
    dev = run_gpu(gpu, MIXED)
    f, e0, traj, dR = errors(dev, reference)
    assert np.array_equal(dev["pairs"], reference["pairs"])
    assert f < 3e-5 and e0.max() < 2e-5
    assert traj[:, 0].max() < 1e-4 and traj[:, 2].max() < 1e-4   # U and K after 25-100 fs
