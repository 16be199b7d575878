"""GPU parity, through the C ABI, of reference entry points that no reference
test drives, against the oracle on the same inputs:

* the linear-r switches EmDee_smoothed / EmDee_shifted_smoothed
  (src/modelClass_nonbonded.f90:133-190);
* model layers: EmDee_set_pair_multimodel, EmDee_set_coul_multimodel,
  EmDee_layer_based_parameters (an inner cut-off served by the inner part of
  the neighbor lists, src/neighbor_lists.f90:256,265) and
  EmDee_switch_model_layer (src/EmDeeCode.f90:273-305,363-412,486-520,929-946);
* EmDee_share_phase_space (src/EmDeeCode.f90:239-269), following
  test/test_phase_space_sharing.f90 (rigid SPC/E water, a second system at half
  the cut-off that reads the first one's phase space);
* writes through EmDee_memory_address (src/EmDeeCode.f90:212-235) taking
  effect in the next call.
"""
import ctypes as C

import numpy as np
import pytest

from emdee_gb300.emdee import EmDee, FP64, MIXED
from mdrun import initialize, load_golden, observables, setup_water, velocity_verlet

pytestmark = pytest.mark.gpu

FORCE_RMS_MIXED = 1.0e-5
ENERGY_REL_MIXED = 1.0e-5
VIRIAL_REL_MIXED = 5.0e-5
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
def nist():
    return load_golden("nist_lj_sample.json")


@pytest.fixture(scope="module")
def water():
    return load_golden("nist_spce_sample.json")


def rel_rms(a, b):
    return float(np.sqrt(np.sum((a - b) ** 2) / np.sum(b ** 2)))


def close(a, b, rel):
    return abs(a - b) <= rel * max(1.0, abs(b))


def view(ptr, shape):
    n = int(np.prod(shape))
    return np.ctypeslib.as_array((C.c_double * n).from_address(ptr)).reshape(shape)


# ---- linear-r switching -----------------------------------------------------------


def lj_switched(lib, cfg, name, width, precision=None, layers=1):
    run, N = cfg["run"], len(cfg["coordinates"])
    md = lib.system(2, layers, run["Rc"], run["skin"], N, cfg["type"], cfg["mass"])
    if precision is not None:
        lib.EmDee_set_precision(md, precision)
    base = lib.EmDee_pair_lj_cut(cfg["epsilon"][0], cfg["sigma"][0])
    p = {"smoothed": lib.EmDee_smoothed, "shifted_smoothed": lib.EmDee_shifted_smoothed}[name](base, width)
    lib.EmDee_set_pair_model(md, 1, 1, p, run["kCoul"])
    return md


@pytest.mark.parametrize("name", ["smoothed", "shifted_smoothed"])
def test_linear_switch_nist(gpu, oracle, nist, name):
    N = len(nist["coordinates"])
    ref = lj_switched(oracle, nist, name, 1.0)
    initialize(oracle, ref, nist)
    Fo = oracle.download(ref, "forces", (N, 3))
    d64 = lj_switched(gpu, nist, name, 1.0, FP64)
    initialize(gpu, d64, nist)
    assert np.array_equal(gpu.neighbor_pairs(d64), oracle.neighbor_pairs(ref))
    assert rel_rms(gpu.download(d64, "forces", (N, 3)), Fo) < 1e-13
    assert close(d64.Energy.Potential, ref.Energy.Potential, FP64_REL)
    assert close(d64.Virial.Total, ref.Virial.Total, FP64_REL)
    d32 = lj_switched(gpu, nist, name, 1.0, MIXED)
    initialize(gpu, d32, nist)
    e = (rel_rms(gpu.download(d32, "forces", (N, 3)), Fo),
         abs(d32.Energy.Potential / ref.Energy.Potential - 1), abs(d32.Virial.Total / ref.Virial.Total - 1))
    print(name, "mixed errors (force RMS, energy, virial):", e)
    assert e[0] < FORCE_RMS_MIXED and e[1] < ENERGY_REL_MIXED and e[2] < VIRIAL_REL_MIXED
    # the golden-test protocol (100 steps, energies every 20) in FP64
    run = nist["run"]
    for lib, md in ((oracle, ref), (gpu, d64)):
        velocity_verlet(lib, md, run["dt"], run["nsteps"], run["nprop"])
    assert d64.Builds == ref.Builds
    assert np.all(np.abs(observables(d64) - observables(ref)) < 1e-8), observables(d64) - observables(ref)


# ---- model layers -----------------------------------------------------------------


def layered_lj(lib, cfg, precision=None):
    """Two layers on the NIST sample: lj_cut, and a shifted-force Lennard-Jones
    of smaller epsilon restricted to an inner cut-off of rc - 1."""
    run, N = cfg["run"], len(cfg["coordinates"])
    md = lib.system(2, 2, run["Rc"], run["skin"], N, cfg["type"], cfg["mass"])
    if precision is not None:
        lib.EmDee_set_precision(md, precision)
    eps, sig = cfg["epsilon"][0], cfg["sigma"][0]
    models = (C.c_void_p * 2)(lib.EmDee_pair_lj_cut(eps, sig),
                              lib.EmDee_shifted_force(lib.EmDee_pair_lj_cut(0.7 * eps, sig)))
    kc = np.array([run["kCoul"], run["kCoul"]])
    lib.EmDee_set_pair_multimodel(md, 1, 1, models, kc.ctypes.data_as(C.c_void_p))
    apply_, bonded = np.array([0, 1], dtype=np.int32), np.array([0, 0], dtype=np.int32)
    lib.EmDee_layer_based_parameters(md, run["Rc"] - 1.0, apply_.ctypes.data_as(C.c_void_p),
                                     bonded.ctypes.data_as(C.c_void_p))
    initialize(lib, md, cfg)
    return md


def layer_state(lib, md, N, layer):
    lib.EmDee_switch_model_layer(C.byref(md), layer)
    md.Options.Compute = True
    lib.EmDee_compute_forces(C.byref(md))
    return md.Energy.Potential, md.Virial.Total, lib.download(md, "forces", (N, 3))


@pytest.mark.parametrize("precision", [FP64, MIXED])
def test_pair_multimodel_layers(gpu, oracle, nist, precision):
    N = len(nist["coordinates"])
    ref, dev = layered_lj(oracle, nist), layered_lj(gpu, nist, precision)
    tolF = 1e-13 if precision == FP64 else FORCE_RMS_MIXED
    tolE = FP64_REL if precision == FP64 else ENERGY_REL_MIXED
    tolW = FP64_REL if precision == FP64 else VIRIAL_REL_MIXED
    seen = {}
    for layer in (1, 2):
        Uo, Wo, Fo = layer_state(oracle, ref, N, layer)
        Ud, Wd, Fd = layer_state(gpu, dev, N, layer)
        assert rel_rms(Fd, Fo) < tolF, layer
        assert close(Ud, Uo, tolE) and close(Wd, Wo, tolW), (layer, Ud, Uo, Wd, Wo)
        seen[layer] = (Ud, Wd)
    assert abs(seen[1][0] - seen[2][0]) > 1.0   # the layers differ
    # switching back restores the stored results of layer 1 without a new computation
    gpu.EmDee_switch_model_layer(C.byref(dev), 1)
    assert dev.Energy.Potential == seen[1][0] and dev.Virial.Total == seen[1][1]
    # every layer's forces through the library's own buffer
    Ld = view(gpu.EmDee_memory_address(dev, b"layerForces"), (2, N, 3)).copy()
    Lo = view(oracle.EmDee_memory_address(ref, b"layerForces"), (2, N, 3)).copy()
    for k in range(2):
        assert rel_rms(Ld[k], Lo[k]) < tolF, k
    # 40 steps kicked by the forces of both layers (each recomputed on its own
    # layer after the displacement), energies of both layers at the end
    dt = nist["run"]["dt"]
    for lib, md in ((oracle, ref), (gpu, dev)):
        for _ in range(40):
            lib.EmDee_switch_model_layer(C.byref(md), 2)
            lib.EmDee_boost(C.byref(md), 1.0, 0.0, 0.5 * dt)
            lib.EmDee_switch_model_layer(C.byref(md), 1)
            lib.EmDee_boost(C.byref(md), 1.0, 0.0, 0.5 * dt)
            lib.EmDee_displace(C.byref(md), 1.0, 0.0, dt)
            lib.EmDee_boost(C.byref(md), 1.0, 0.0, 0.5 * dt)
            lib.EmDee_switch_model_layer(C.byref(md), 2)
            lib.EmDee_boost(C.byref(md), 1.0, 0.0, 0.5 * dt)
    assert dev.Builds == ref.Builds
    tolR = 1e-9 if precision == FP64 else 1e-4
    assert np.max(np.abs(gpu.download(dev, "coordinates", (N, 3)) -
                         oracle.download(ref, "coordinates", (N, 3)))) < tolR
    for layer in (1, 2):
        Uo, Wo, Fo = layer_state(oracle, ref, N, layer)
        if precision == MIXED:   # the trajectories separated slightly: the oracle on the GPU's configuration
            R = gpu.download(dev, "coordinates", (N, 3))
            oracle.upload(ref, "coordinates", R)
            Uo, Wo, Fo = layer_state(oracle, ref, N, layer)
        Ud, Wd, Fd = layer_state(gpu, dev, N, layer)
        assert rel_rms(Fd, Fo) < (1e-9 if precision == FP64 else FORCE_RMS_MIXED), layer
        assert close(Ud, Uo, 1e-9 if precision == FP64 else ENERGY_REL_MIXED), (layer, Ud, Uo)


def test_coul_multimodel_layers(gpu, oracle, water):
    """SPC/E as free atoms with intramolecular exclusions: layer 1 damped Coulomb
    over the full cut-off, layer 2 shifted-force Coulomb over an inner 6 A."""
    N = len(water["coordinates"])

    def hook(lib, md):
        models = (C.c_void_p * 2)(lib.EmDee_coul_damped(0.2), lib.EmDee_coul_sf())
        lib.EmDee_set_coul_multimodel(md, models)

    def make(lib, precision=None):
        run = water["run"]
        md = lib.system(1, 2, run["Rc"], run["skin"], N, water["type"], water["mass"])
        if precision is not None:
            lib.EmDee_set_precision(md, precision)
        apply_, bonded = np.array([0, 1], dtype=np.int32), np.array([0, 0], dtype=np.int32)
        lib.EmDee_layer_based_parameters(md, 6.0, apply_.ctypes.data_as(C.c_void_p),
                                         bonded.ctypes.data_as(C.c_void_p))
        for i, (eps, sig) in enumerate(zip(water["epsilon"], water["sigma"])):
            p = lib.EmDee_pair_none() if eps == 0.0 else \
                lib.EmDee_shifted_force(lib.EmDee_pair_lj_cut(eps / run["mvv2e"], sig))
            lib.EmDee_set_pair_model(md, i + 1, i + 1, p, run["kCoul"])
        hook(lib, md)
        mol = water["molecule"]
        for a in range(0, N, 3):
            assert mol[a] == mol[a + 1] == mol[a + 2]
            for x, y in ((a + 1, a + 2), (a + 1, a + 3), (a + 2, a + 3)):
                lib.EmDee_ignore_pair(md, x, y)
        lib.upload(md, "charges", water["charge"])
        lib.upload(md, "box", np.array([water["box"]]))
        lib.upload(md, "coordinates", np.array(water["coordinates"]))
        return md

    ref = make(oracle)
    for precision, tolF, tolE in ((FP64, 1e-12, FP64_REL), (MIXED, FORCE_RMS_MIXED, 2e-5)):
        dev = make(gpu, precision)
        for layer in (1, 2):
            Uo, Wo, Fo = layer_state(oracle, ref, N, layer)
            Ud, Wd, Fd = layer_state(gpu, dev, N, layer)
            assert rel_rms(Fd, Fo) < tolF, (precision, layer)
            assert abs(Ud - Uo) <= tolE * abs(Uo) and abs(Wd - Wo) <= tolE * abs(Wo), (precision, layer)
            assert abs(dev.Energy.Coulomb - ref.Energy.Coulomb) <= tolE * abs(Uo), (precision, layer)
        oracle.EmDee_switch_model_layer(C.byref(ref), 1)


# ---- phase-space sharing and memory addresses ------------------------------------


def test_share_phase_space(gpu, oracle, water):
    """test/test_phase_space_sharing.f90: `other` (half the cut-off) reads the
    phase space of `md` after the share, through md's later moves as well."""
    N = len(water["coordinates"])
    run = water["run"]

    def make(lib, rc):
        md = lib.system(1, 1, rc, run["skin"], N, water["type"], water["mass"], water["molecule"])
        for i, (eps, sig) in enumerate(zip(water["epsilon"], water["sigma"])):
            p = lib.EmDee_pair_none() if eps == 0.0 else \
                lib.EmDee_shifted_force(lib.EmDee_pair_lj_cut(eps / run["mvv2e"], sig))
            lib.EmDee_set_pair_model(md, i + 1, i + 1, p, run["kCoul"])
        lib.EmDee_set_coul_model(md, lib.EmDee_coul_sf())
        lib.upload(md, "charges", water["charge"])
        lib.upload(md, "coordinates", np.array(water["coordinates"]))
        lib.upload(md, "box", np.array([water["box"]]))
        return md

    pairs = {}
    for name, lib in (("oracle", oracle), ("gpu", gpu)):
        md, other = make(lib, run["Rc"]), make(lib, 0.5 * run["Rc"])
        if lib is gpu:
            lib.EmDee_set_precision(md, FP64)
            lib.EmDee_set_precision(other, FP64)
        lib.EmDee_random_momenta(C.byref(md), run["kB"] * run["temp"], True, run["seed"])
        velocity_verlet(lib, md, run["dt"], 20, 1)
        lib.EmDee_share_phase_space(md, C.byref(other))
        kin = other.Kinetic.Total
        other.Options.Compute = True
        lib.EmDee_compute_forces(C.byref(other))
        first = (other.Energy.Potential, other.Virial.Total, kin, md.Kinetic.Total)
        velocity_verlet(lib, md, run["dt"], 10, 1)
        other.Options.Compute = True
        lib.EmDee_compute_forces(C.byref(other))
        second = (other.Energy.Potential, other.Virial.Total,
                  np.max(np.abs(lib.download(other, "coordinates", (N, 3)) - lib.download(md, "coordinates", (N, 3)))))
        pairs[name] = (first, second)
    (fo, so), (fd, sd) = pairs["oracle"], pairs["gpu"]
    # the two FP64 trajectories of md separate by ~1e-9 over 30 rigid-body steps
    # (summation order), so the comparisons carry 1e-7
    assert fd[2] == fd[3]                      # kinetic energy copied at the share
    assert close(fd[0], fo[0], 1e-7) and close(fd[1], fo[1], 1e-7), (fd, fo)
    assert sd[2] == 0.0 and so[2] == 0.0       # other sees md's coordinates
    assert close(sd[0], so[0], 1e-7) and close(sd[1], so[1], 1e-7), (sd, so)
    assert abs(sd[0] - fd[0]) > 1e-6 * abs(fd[0])   # md's moves reached other


@pytest.mark.parametrize("precision", [FP64, MIXED])
def test_memory_address_writes(gpu, oracle, nist, precision):
    """A write into EmDee_memory_address("coordinates") changes the forces of
    the next call, as the same write does in the oracle; after a displacement
    the buffer holds the new coordinates."""
    from mdrun import setup_lj_sample
    N = len(nist["coordinates"])
    mds = {}
    for name, lib in (("oracle", oracle), ("gpu", gpu)):
        md = setup_lj_sample(lib, nist, precision=precision if lib is gpu else None)
        initialize(lib, md, nist)
        lib.download(md, "forces", (N, 3))
        R = view(lib.EmDee_memory_address(md, b"coordinates"), (N, 3))
        R[17] += np.array([0.05, -0.03, 0.02])
        R[400, 1] -= 0.04
        md.Options.Compute = True
        lib.EmDee_compute_forces(C.byref(md))
        mds[name] = (lib, md, lib.download(md, "forces", (N, 3)), md.Energy.Potential, R)
    _, ref, Fo, Uo, _ = mds["oracle"]
    _, dev, Fd, Ud, Rd = mds["gpu"]
    tol = 1e-13 if precision == FP64 else FORCE_RMS_MIXED
    assert rel_rms(Fd, Fo) < tol
    assert close(Ud, Uo, 1e-12 if precision == FP64 else ENERGY_REL_MIXED)
    moved = setup_lj_sample(oracle, nist)
    initialize(oracle, moved, nist)
    R = np.array(nist["coordinates"])
    R[17] += np.array([0.05, -0.03, 0.02])
    R[400, 1] -= 0.04
    oracle.upload(moved, "coordinates", R)
    assert rel_rms(oracle.download(moved, "forces", (N, 3)), Fo) < 1e-14   # the write took effect
    gpu.EmDee_displace(C.byref(dev), 1.0, 0.0, nist["run"]["dt"])
    assert np.array_equal(Rd, gpu.download(dev, "coordinates", (N, 3)))
