"""Kinetic energies of EmDee_boost with energies requested (src/EmDeeCode.f90:
1024-1065: each boost reports 2KE per dimension of the kicked momenta), in mixed
precision, where the kick itself is deferred into the next kernel that touches
the momenta and only its kinetic energy is computed when the boost returns:

* after a displacement, once the new forces are computed, by a pass over P and
  F that writes nothing and also sums the kinetic energy of a second identical
  kick, used by the next half-kick of a velocity-Verlet step when nothing
  changed in between (float-float arithmetic for unit masses, FP64 otherwise);
* otherwise by a pass over P, F and the pending kicks that writes nothing.

After every boost the reported energy must equal 1/2 sum P^2/m of the momenta
downloaded at that point (which applies the pending kicks), and a step sequence
must give the oracle's kinetic energies.
"""
import ctypes as C

import numpy as np
import pytest

from emdee_gb300.emdee import EmDee, MIXED
from mdrun import fcc_lattice

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    import emdee_gb300
    from emdee_gb300.build import build
    build()
    return emdee_gb300.load()


@pytest.fixture(scope="module")
def oracle(oracle_path):
    return EmDee(oracle_path)


def system(lib, N, masses, precision=None):
    L = (N / 0.8) ** (1.0 / 3.0)
    types = (np.arange(N) % len(masses)) + 1
    md = lib.system(1, 1, 2.5, 0.3, N, types, masses)
    if precision is not None:
        lib.EmDee_set_precision(md, precision)
    for t in range(1, len(masses) + 1):
        lib.EmDee_set_pair_model(md, t, t, lib.EmDee_pair_lj_cut(1.0, 1.0), 0.0)
    lib.upload(md, "box", np.array([L]))
    lib.upload(md, "coordinates", fcc_lattice(N, L, 0.05, 21))
    lib.EmDee_random_momenta(C.byref(md), 1.4, True, 4321)
    return md, np.array(masses)[types - 1]


def ke_of(lib, md, N, m):
    P = lib.download(md, "momenta", (N, 3))
    return 0.5 * (P * P / m[:, None]).sum(0)


@pytest.mark.parametrize("masses", [[1.0], [1.0, 2.5]])
def test_boost_energies_match_momenta(gpu, masses):
    N, dt = 2048, 0.005
    md, m = system(gpu, N, masses, MIXED)
    md.Options.Compute = True
    for step in range(12):
        for call in range(3):
            if call == 1:
                gpu.EmDee_displace(C.byref(md), 1.0, 0.0, dt)
                continue
            gpu.EmDee_boost(C.byref(md), 1.0, 0.0, 0.5 * dt)
            if step % 3 == 2:   # some steps leave the kicks pending (no download)
                continue
            ke = ke_of(gpu, md, N, m)
            got = np.array(md.Kinetic.TransPart[:])
            assert np.all(np.abs(got - ke) <= 1e-13 * np.abs(ke)), (step, call, got, ke)
            assert abs(md.Kinetic.Total - ke.sum()) <= 1e-13 * ke.sum()


def test_boost_energies_varying_kicks(gpu):
    """Kicks of different sizes and a boost with up-to-date forces (no speculative
    value applies): the kinetic-energy pass path."""
    N = 1500
    md, m = system(gpu, N, [1.0], MIXED)
    md.Options.Compute = True
    for cf in (0.001, 0.002, 0.002, 0.0005, -0.001):
        gpu.EmDee_boost(C.byref(md), 1.0, 0.0, cf)
        ke = ke_of(gpu, md, N, m)
        assert abs(md.Kinetic.Total - ke.sum()) <= 1e-13 * ke.sum()
    gpu.EmDee_displace(C.byref(md), 1.0, 0.0, 0.004)
    gpu.EmDee_boost(C.byref(md), 1.0, 0.0, 0.003)   # forces recomputed: the two-kick pass
    k1 = md.Kinetic.Total
    gpu.EmDee_boost(C.byref(md), 1.0, 0.0, 0.002)   # a different kick: no speculative value
    k2 = md.Kinetic.Total
    ke = ke_of(gpu, md, N, m)
    assert abs(k2 - ke.sum()) <= 1e-13 * ke.sum() and k1 != k2


def test_kinetic_trajectory_vs_oracle(gpu, oracle):
    """30 velocity-Verlet steps with energies every step: kinetic energy after
    each boost against the oracle (the trajectories separate only at the level of
    FP32 pair rounding over these few steps)."""
    N, dt = 2048, 0.005
    a, _ = system(oracle, N, [1.0, 2.5])
    b, _ = system(gpu, N, [1.0, 2.5], MIXED)
    worst = 0.0
    for step in range(30):
        for md, lib in ((a, oracle), (b, gpu)):
            md.Options.Compute = True
            lib.EmDee_boost(C.byref(md), 1.0, 0.0, 0.5 * dt)
        worst = max(worst, abs(b.Kinetic.Total / a.Kinetic.Total - 1))
        for md, lib in ((a, oracle), (b, gpu)):
            lib.EmDee_displace(C.byref(md), 1.0, 0.0, dt)
            lib.EmDee_boost(C.byref(md), 1.0, 0.0, 0.5 * dt)
        worst = max(worst, abs(b.Kinetic.Total / a.Kinetic.Total - 1))
    print("kinetic energy, worst relative difference over 30 steps: %.2e" % worst)
    assert worst < 1e-6


@pytest.mark.parametrize("pinned", [False, True])
def test_boost_energies_after_momenta_upload(gpu, pinned):
    """A velocity-Verlet loop that uploads new momenta at the start of every step
    (the upload also sums the kinetic energy of the next half-kick): each boost's
    energy equals 1/2 sum P^2 of the momenta downloaded right after it."""
    N, dt = 2048, 0.005
    md, m = system(gpu, N, [1.0], MIXED)
    md.Options.Compute = True
    rng = np.random.default_rng(5)
    if pinned:
        torch = pytest.importorskip("torch")
        buf = torch.empty((N, 3), dtype=torch.float64, pin_memory=True).numpy()
    for step in range(8):
        P = rng.normal(0.0, 1.2, (N, 3))
        if pinned:
            buf[:] = P
            gpu.upload(md, "momenta", buf)
        else:
            gpu.upload(md, "momenta", np.ascontiguousarray(P))
        for call in range(3):
            if call == 1:
                gpu.EmDee_displace(C.byref(md), 1.0, 0.0, dt)
                continue
            gpu.EmDee_boost(C.byref(md), 1.0, 0.0, 0.5 * dt)
            ke = ke_of(gpu, md, N, m)
            assert abs(md.Kinetic.Total - ke.sum()) <= 1e-13 * ke.sum(), (step, call)
