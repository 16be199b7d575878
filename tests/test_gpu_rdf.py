"""GPU parity of EmDee_rdf (src/EmDeeCode.f90:1281-1395) with the CPU oracle:
the histograms are integer counts of the same pairs at the same FP64
distances, so the normalised g(r) agree exactly."""
import ctypes as C

import numpy as np
import pytest

from emdee_gb300.emdee import EmDee, FP64, MIXED
from mdrun import initialize, load_golden, setup_lj_sample, setup_water, velocity_verlet
from test_oracle_rdf import rdf

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


@pytest.mark.parametrize("Rc,bins", [(3.0, 40), (3.4, 100), (1.5, 7)])
def test_rdf_lj(gpu, oracle, Rc, bins):
    lj = load_golden("nist_lj_sample.json")
    out = []
    for lib, prec in ((oracle, None), (gpu, FP64)):
        md = setup_lj_sample(lib, lj, "shifted_force", precision=prec)
        initialize(lib, md, lj)
        velocity_verlet(lib, md, lj["run"]["dt"], 8)
        out.append(rdf(lib, md, bins, Rc, [(1, 1)]))
    assert np.array_equal(out[0], out[1])


@pytest.mark.parametrize("precision", [FP64, MIXED])
def test_rdf_water(gpu, oracle, precision):
    w = load_golden("nist_spce_sample.json")
    pairs = [(1, 1), (1, 2), (2, 1), (2, 2)]
    ref = rdf(oracle, setup_water(oracle, w, "coul_sf"), 50, 9.5, pairs)
    dev = rdf(gpu, setup_water(gpu, w, "coul_sf", precision=precision), 50, 9.5, pairs)
    assert np.array_equal(ref, dev)
    assert np.array_equal(dev[1], dev[2])
