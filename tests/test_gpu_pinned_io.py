"""Uploads and downloads through page-locked caller buffers take fused kernel paths
(emdee_gb300/csrc/motion.cu, api.cpp): the kinetic-energy kernel reads uploaded
momenta straight from the caller's buffer and stores them, and a momenta download
with pending kicks applies them and writes the caller's buffer in one pass
(coordinate downloads leave the kicks pending).  Every result must be bit-identical
to the copy paths that pageable buffers take, in mixed and FP64 precision, with one
and with two pending kicks."""
import ctypes as C

import numpy as np
import pytest

from emdee_gb300.emdee import FP64, MIXED, _ptr
from mdrun import fcc_lattice

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    import emdee_gb300
    from emdee_gb300.build import build
    build()
    return emdee_gb300.load()


def system(lib, R, L, precision):
    md = lib.system(1, 1, 2.5, 0.3, len(R))
    lib.EmDee_set_precision(md, precision)
    lib.EmDee_set_pair_model(md, 1, 1, lib.EmDee_pair_lj_cut(1.0, 1.0), 0.0)
    lib.upload(md, "box", np.array([L]))
    lib.upload(md, "coordinates", R)
    return md


def pinned(shape):
    torch = pytest.importorskip("torch")
    return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()


@pytest.mark.parametrize("precision", [MIXED, FP64])
def test_pinned_paths_match_copies(gpu, precision):
    N, rho, dt = 4000, 0.85, 0.005
    L = (N / rho) ** (1.0 / 3.0)
    R0 = fcc_lattice(N, L, 0.05, 5)
    a, b = system(gpu, R0, L, precision), system(gpu, R0, L, precision)
    P = np.random.default_rng(3).normal(0.0, 1.2, (N, 3))
    Pb, Rb_out, Pb_out = pinned((N, 3)), pinned((N, 3)), pinned((N, 3))
    for step in range(12):
        Pb[:] = P
        gpu.upload(a, "momenta", P)      # pageable: copy, then the kinetic sum
        gpu.upload(b, "momenta", Pb)     # pinned: one kernel reads the caller's buffer
        assert a.Kinetic.Total == b.Kinetic.Total
        for md in (a, b):
            md.Options.Compute = step % 3 == 0   # boosts without energies are deferred kicks
            gpu.EmDee_boost(C.byref(md), 1.0, 0.0, 0.5 * dt)
            gpu.EmDee_displace(C.byref(md), 1.0, 0.0, dt)
            gpu.EmDee_boost(C.byref(md), 1.0, 0.0, 0.5 * dt)
            if step % 4 == 3:   # a second pending kick before the downloads
                gpu.EmDee_boost(C.byref(md), 1.0, 0.0, 0.25 * dt)
        Ra = gpu.download(a, "coordinates", (N, 3))
        gpu.lib.EmDee_download(b, b"coordinates", _ptr(Rb_out))
        Pa = gpu.download(a, "momenta", (N, 3))
        gpu.lib.EmDee_download(b, b"momenta", _ptr(Pb_out))   # applies the pending kicks
        assert np.array_equal(Ra, Rb_out) and np.array_equal(Pa, Pb_out)
        assert a.Energy.Potential == b.Energy.Potential and a.Virial.Total == b.Virial.Total
        P = Pa * 0.999   # the next step's upload
    # the state the kernels left on the device is the same too
    assert np.array_equal(gpu.download(a, "momenta", (N, 3)), gpu.download(b, "momenta", (N, 3)))
