"""Boost and displacement with a non-zero alpha (src/EmDeeCode.f90:1024-1103): the
momenta are scaled by CP = 1 - alpha CF and the coordinates and the box by
CR = 1 - alpha CP, so the box length changes every step while the neighbor
lists stay those of the last build (the skin check runs on real coordinates).
GPU against the oracle on the NIST Lennard-Jones sample, FP64 and mixed
precision, plus a box re-upload after initialization."""
import ctypes as C

import numpy as np
import pytest

from emdee_gb300.emdee import EmDee, FP64, MIXED
from mdrun import initialize, load_golden, setup_lj_sample

pytestmark = pytest.mark.gpu

TOL = {FP64: 1e-10, MIXED: 2e-5}


@pytest.fixture(scope="module")
def gpu():
    import emdee_gb300
    from emdee_gb300.build import build
    build()
    return emdee_gb300.load()


@pytest.fixture(scope="module")
def oracle(oracle_path):
    return EmDee(oracle_path)


def run(lib, cfg, precision, steps, alpha_p, alpha_r, rescale_at=None):
    N, dt = len(cfg["coordinates"]), cfg["run"]["dt"]
    md = setup_lj_sample(lib, cfg, "shifted_force", precision=precision)
    initialize(lib, md, cfg)
    obs = []
    for step in range(steps):
        if step == rescale_at:   # a new box with the same coordinates
            L = lib.download(md, "box", (1,))[0]
            lib.upload(md, "box", np.array([L * 1.002]))
        md.Options.Compute = True
        lib.EmDee_boost(C.byref(md), 1.0, alpha_p, 0.5 * dt)
        lib.EmDee_displace(C.byref(md), 1.0, alpha_r, dt)
        lib.EmDee_boost(C.byref(md), 1.0, alpha_p, 0.5 * dt)
        obs.append([md.Energy.Potential, md.Virial.Total, md.Kinetic.Total])
    return np.array(obs), lib.download(md, "coordinates", (N, 3)), lib.download(md, "box", (1,))[0], md.Builds


@pytest.mark.parametrize("precision", [FP64, MIXED])
@pytest.mark.parametrize("rescale_at", [None, 7])
def test_alpha_scaling_matches_oracle(gpu, oracle, precision, rescale_at):
    cfg = load_golden("nist_lj_sample.json")
    ref = run(oracle, cfg, None, 25, 0.3, 0.2, rescale_at)
    got = run(gpu, cfg, precision, 25, 0.3, 0.2, rescale_at)
    rel = np.abs(got[0] - ref[0]) / np.abs(ref[0])
    print("precision %d: max rel obs error %.2e, max |dR| %.2e, box %.15g %.15g, builds %d %d" % (
        precision, rel.max(), np.abs(got[1] - ref[1]).max(), got[2], ref[2], got[3], ref[3]))
    assert got[2] == pytest.approx(ref[2], rel=1e-14)
    assert ref[2] != cfg["box"]
    assert rel.max() < TOL[precision]
    assert np.abs(got[1] - ref[1]).max() < 1e3 * TOL[precision]
    assert got[3] == ref[3]
