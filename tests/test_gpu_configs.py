"""GPU parity on the Lennard-Jones workloads the benchmark is built on, through
the C ABI, against the FP64 oracle:

* the 4000-atom fcc fluid (rho 0.85, T* 1.5, rc 2.5, skin 0.3, dt 0.005) over
  1000 velocity-Verlet steps with per-step energy, virial and rebuild count
  (the loop of test/common/contained.f90:63-72);
* the 1,048,576-atom fcc box (rho 0.8442) on which the throughput is quoted:
  sorted neighbor pair sets after the first build and after the first
  skin-triggered rebuild, forces, energy and virial.

Two FP64 trajectories that differ only in the order of their force sums drift
apart chaotically: the oracle against itself with 1 and 2 threads differs by
2e-9 in the energy and 9e-8 in the virial after 1000 steps (1e-14 before step
400), so the FP64 tolerances below grow with the step.  Mixed precision rounds
pair terms to FP32, which puts its trajectory on a different chaotic orbit
within a few hundred steps; it is therefore checked by shadowing: at every
step the oracle evaluates the configuration the GPU reached (coordinates
uploaded bit for bit), and forces, energy, virial and the rebuild count are
compared there.
"""
import ctypes as C
import os

import numpy as np
import pytest

from emdee_gb300.emdee import EmDee, FP64, MIXED
from mdrun import fcc_lattice

pytestmark = pytest.mark.gpu

FORCE_RMS_MIXED = 1.0e-5    # relative RMS of the force field, FP32 pair math vs FP64
ENERGY_REL_MIXED = 1.0e-5   # relative error of the potential energy
VIRIAL_REL_MIXED = 5.0e-5   # relative error of the virial (a sum with strong cancellation)


@pytest.fixture(scope="module")
def gpu():
    import emdee_gb300
    from emdee_gb300.build import build
    build()
    return emdee_gb300.load()


@pytest.fixture(scope="module")
def oracle(oracle_path):
    return EmDee(oracle_path)


def rel_rms(a, b):
    return float(np.sqrt(np.sum((a - b) ** 2) / np.sum(b ** 2)))


def lj_fcc(lib, N, rho, seed, precision=None, threads=1, kT=1.5):
    L = (N / rho) ** (1.0 / 3.0)
    md = lib.system(threads, 1, 2.5, 0.3, N)
    if precision is not None:
        lib.EmDee_set_precision(md, precision)
    lib.EmDee_set_pair_model(md, 1, 1, lib.EmDee_pair_lj_cut(1.0, 1.0), 0.0)
    lib.upload(md, "box", np.array([L]))
    lib.upload(md, "coordinates", fcc_lattice(N, L, 0.05, seed))
    lib.EmDee_random_momenta(C.byref(md), kT, True, 86245)
    return md


def vv_step(lib, md, dt):
    lib.EmDee_boost(C.byref(md), 1.0, 0.0, 0.5 * dt)
    lib.EmDee_displace(C.byref(md), 1.0, 0.0, dt)
    lib.EmDee_boost(C.byref(md), 1.0, 0.0, 0.5 * dt)


def fp64_tolerance(step):
    """Energy and virial bounds of independent FP64 trajectories at a step: ten
    times the measured oracle-vs-oracle separation envelope."""
    grow = 10.0 ** max(0.0, (step - 400) / 100.0)   # x10 per 100 steps after step 400
    return min(1e-12 * grow, 1e-6), min(1e-11 * grow, 1e-5)


def test_config0_fp64_1000_steps(gpu, oracle):
    N, dt = 4000, 0.005
    ref = lj_fcc(oracle, N, 0.85, 3)
    dev = lj_fcc(gpu, N, 0.85, 3, FP64)
    worst = [0.0, 0.0]
    for step in range(1, 1001):
        for lib, md in ((oracle, ref), (gpu, dev)):
            md.Options.Compute = True
            vv_step(lib, md, dt)
        eu = abs(dev.Energy.Potential - ref.Energy.Potential) / abs(ref.Energy.Potential)
        ew = abs(dev.Virial.Total - ref.Virial.Total) / abs(ref.Virial.Total)
        tu, tw = fp64_tolerance(step)
        assert dev.Builds == ref.Builds, step
        assert eu < tu and ew < tw, (step, eu, ew)
        worst = [max(worst[0], eu), max(worst[1], ew)]
    ek = abs(dev.Kinetic.Total - ref.Kinetic.Total) / abs(ref.Kinetic.Total)
    print("FP64, 1000 steps: worst energy / virial error %.2e / %.2e, kinetic %.2e, builds %d"
          % (worst[0], worst[1], ek, dev.Builds))


def test_config0_mixed_1000_steps_shadowed(gpu, oracle):
    """Mixed precision (the benchmark's mode): the oracle evaluates every step's
    configuration of the GPU trajectory; its own skin check, run on the same
    coordinates, must rebuild at the same steps."""
    N, dt = 4000, 0.005
    dev = lj_fcc(gpu, N, 0.85, 3, MIXED)
    shadow = lj_fcc(oracle, N, 0.85, 3)
    worst = np.zeros(3)
    for step in range(1, 1001):
        dev.Options.Compute = True
        vv_step(gpu, dev, dt)
        R = gpu.download(dev, "coordinates", (N, 3))
        oracle.upload(shadow, "coordinates", R)
        shadow.Options.Compute = True
        oracle.EmDee_compute_forces(C.byref(shadow))
        Fo = oracle.download(shadow, "forces", (N, 3))
        Fd = gpu.download(dev, "forces", (N, 3))
        e = np.array([rel_rms(Fd, Fo),
                      abs(dev.Energy.Potential - shadow.Energy.Potential) / abs(shadow.Energy.Potential),
                      abs(dev.Virial.Total - shadow.Virial.Total) / abs(shadow.Virial.Total)])
        assert dev.Builds == shadow.Builds, step
        assert e[0] < FORCE_RMS_MIXED and e[1] < ENERGY_REL_MIXED and e[2] < VIRIAL_REL_MIXED, (step, e)
        worst = np.maximum(worst, e)
    print("mixed, 1000 steps: worst force RMS %.2e, energy %.2e, virial %.2e; builds %d"
          % (worst[0], worst[1], worst[2], dev.Builds))


def test_config2_full_size(gpu, oracle):
    """N = 1,048,576 (fcc 4 x 64^3, rho 0.8442, M = 76 cells per edge), mixed
    precision: pair sets bit-identical after the first build and after the first
    rebuild the skin check triggers; forces, energy and virial at both."""
    N, dt = 1048576, 0.005
    dev = lj_fcc(gpu, N, 0.8442, 86245, MIXED)
    ref = lj_fcc(oracle, N, 0.8442, 86245, threads=os.cpu_count() or 1)

    def compare(tag):
        pd, po = gpu.neighbor_pairs(dev), oracle.neighbor_pairs(ref)
        assert pd.shape == po.shape and np.array_equal(pd, po), tag
        Fd = gpu.download(dev, "forces", (N, 3))
        Fo = oracle.download(ref, "forces", (N, 3))
        e = (rel_rms(Fd, Fo), abs(dev.Energy.Potential / ref.Energy.Potential - 1),
             abs(dev.Virial.Total / ref.Virial.Total - 1))
        print(tag, "pairs", len(pd), "force RMS %.2e energy %.2e virial %.2e" % e)
        assert e[0] < FORCE_RMS_MIXED and e[1] < ENERGY_REL_MIXED and e[2] < VIRIAL_REL_MIXED, (tag, e)

    compare("first build")
    b0 = dev.Builds
    for step in range(1, 60):
        dev.Options.Compute = True
        vv_step(gpu, dev, dt)
        if dev.Builds > b0:
            break
    assert dev.Builds == b0 + 1
    # the oracle evaluates the GPU's configuration; its skin check, on the same
    # coordinates, must have rebuilt at this step as well (it builds here once)
    oracle.upload(ref, "coordinates", gpu.download(dev, "coordinates", (N, 3)))
    ref.Options.Compute = True
    oracle.EmDee_compute_forces(C.byref(ref))
    assert ref.Builds == dev.Builds
    compare("rebuild at step %d" % step)
