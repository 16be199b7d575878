"""GPU parity of every pair model, Coulomb model and modifier against the CPU
oracle (FP64 and mixed precision), on the NIST SPC/E configuration treated as
free atoms with intramolecular exclusions (2 atom types, charges)."""
import numpy as np
import pytest

from emdee_gb300.emdee import EmDee, FP64, MIXED
from mdrun import COUL_MODELS, load_golden, setup_water

pytestmark = pytest.mark.gpu

FORCE_RMS_MIXED = 1.0e-5
ENERGY_REL_MIXED = 2.0e-5   # Coulomb sums cancel strongly; stated relative to the total
FP64_REL = 1.0e-12


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


def rel_rms(a, b):
    return float(np.sqrt(np.sum((a - b) ** 2) / np.sum(b ** 2)))


@pytest.mark.parametrize("pair", ["shifted_force", "softcore"])
@pytest.mark.parametrize("coul", sorted(COUL_MODELS))
def test_water_models(gpu, oracle, water, coul, pair):
    N = len(water["coordinates"])
    ref = setup_water(oracle, water, coul, pair)
    Fo = oracle.download(ref, "forces", (N, 3))
    assert np.array_equal(gpu.neighbor_pairs(setup_water(gpu, water, coul, pair, MIXED)),
                          oracle.neighbor_pairs(ref))
    d64 = setup_water(gpu, water, coul, pair, FP64)
    F64 = gpu.download(d64, "forces", (N, 3))
    assert rel_rms(F64, Fo) < FP64_REL
    for a, b in ((d64.Energy.Potential, ref.Energy.Potential), (d64.Energy.Coulomb, ref.Energy.Coulomb),
                 (d64.Virial.Total, ref.Virial.Total)):
        assert abs(a - b) <= FP64_REL * max(1.0, abs(b))
    d32 = setup_water(gpu, water, coul, pair, MIXED)
    F32 = gpu.download(d32, "forces", (N, 3))
    errs = (rel_rms(F32, Fo), abs(d32.Energy.Potential - ref.Energy.Potential) / abs(ref.Energy.Potential),
            abs(d32.Virial.Total - ref.Virial.Total) / abs(ref.Virial.Total))
    print(coul, pair, "mixed errors (force RMS, energy, virial):", errs)
    assert errs[0] < FORCE_RMS_MIXED
    assert errs[1] < ENERGY_REL_MIXED
    assert errs[2] < ENERGY_REL_MIXED
