"""Shared drivers that call an EmDee-ABI library the way the reference's
test programs do (test/common/contained.f90:58-87)."""
import ctypes as C
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_golden(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def setup_lj_sample(lib, cfg, modifier="none", skin_width=None, threads=2, precision=None):
    """test/test_pair_lj_*.f90:33-44 on the NIST LJ sample."""
    run = cfg["run"]
    N = len(cfg["coordinates"])
    md = lib.system(threads, 1, run["Rc"], run["skin"], N, cfg["type"], cfg["mass"])
    if precision is not None:
        lib.EmDee_set_precision(md, precision)
    for i, (eps, sig) in enumerate(zip(cfg["epsilon"], cfg["sigma"])):
        p = lib.EmDee_pair_lj_cut(eps / run["mvv2e"], sig)
        if modifier == "shifted_force":
            p = lib.EmDee_shifted_force(p)
        elif modifier == "square_smoothed":
            p = lib.EmDee_square_smoothed(p, skin_width)
        elif modifier == "shifted_square_smoothed":
            p = lib.EmDee_shifted_square_smoothed(p, skin_width)
        lib.EmDee_set_pair_model(md, i + 1, i + 1, p, run["kCoul"])
    return md


def initialize(lib, md, cfg, seed=None, kT=None):
    run = cfg["run"]
    lib.upload(md, "charges", cfg["charge"])
    lib.upload(md, "box", np.array([cfg["box"]]))
    lib.upload(md, "coordinates", np.array(cfg["coordinates"]))
    lib.EmDee_random_momenta(C.byref(md), run["kB"] * run["temp"] if kT is None else kT, True,
                             run["seed"] if seed is None else seed)


def velocity_verlet(lib, md, dt, nsteps, nprop=1, on_step=None):
    """test/common/contained.f90:63-72"""
    for step in range(1, nsteps + 1):
        md.Options.Compute = (step % nprop == 0)
        lib.EmDee_boost(C.byref(md), 1.0, 0.0, 0.5 * dt)
        lib.EmDee_displace(C.byref(md), 1.0, 0.0, dt)
        lib.EmDee_boost(C.byref(md), 1.0, 0.0, 0.5 * dt)
        if on_step is not None:
            on_step(step, md)


def observables(md, mvv2e=1.0):
    return np.array([mvv2e * md.Energy.Potential, mvv2e * md.Virial.Total,
                     mvv2e * (md.Energy.Potential + md.Kinetic.Total)])


def fcc_lattice(N, L, jitter, seed):
    """fcc sites filling the smallest 4 n^3 lattice >= N (first N sites), jittered
    uniformly by +-jitter; the box-filling idea of src/testc.c:77-89."""
    n = 1
    while 4 * n ** 3 < N:
        n += 1
    a = L / n
    base = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    g = np.stack(np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij"), -1).reshape(-1, 3)
    sites = (g[:, None, :] + base[None, :, :]).reshape(-1, 3)[:N] * a
    rng = np.random.default_rng(seed)
    return sites + rng.uniform(-jitter, jitter, size=sites.shape)


COUL_MODELS = {
    # name -> factory(lib) as the reference's test_coul_*.f90 build them (test/test_coul_*.f90:45)
    "coul_cut": lambda lib: lib.EmDee_coul_cut(),
    "coul_sf": lambda lib: lib.EmDee_coul_sf(),
    "coul_damped": lambda lib: lib.EmDee_coul_damped(0.2),
    "coul_damped_smoothed": lambda lib: lib.EmDee_coul_damped_smoothed(0.2, 1.0),
    "coul_damped_square_smoothed": lambda lib: lib.EmDee_coul_damped_square_smoothed(0.2, 1.0),
    "coul_square_smoothed": lambda lib: lib.EmDee_coul_square_smoothed(1.0),
    "coul_shifted_square_smoothed": lambda lib: lib.EmDee_coul_shifted_square_smoothed(1.0),
    "shifted_force(coul_damped)": lambda lib: lib.EmDee_shifted_force(lib.EmDee_coul_damped(0.2)),
    "square_smoothed(coul_cut)": lambda lib: lib.EmDee_square_smoothed(lib.EmDee_coul_cut(), 1.0),
    "none": lambda lib: lib.EmDee_coul_none(),
}


# SPC/Fw flexible water (Wu, Tepper and Voth, J. Chem. Phys. 124, 024503 (2006)):
# O-H bonds and the H-O-H angle, force constants in kcal/mol per A^2 and per rad^2
SPCFW = dict(kb=1059.162, r0=1.012, ka=75.90, theta0=np.radians(113.24))


def add_flexible_water(lib, md, natoms, mvv2e, kb=None, ka=None):
    """Harmonic O-H bonds and H-O-H angles for molecules laid out as O, H, H
    (EmDee_add_bond / EmDee_add_angle, src/EmDeeCode.f90:574-624); these also
    exclude the intramolecular pairs from the neighbor lists."""
    bond = lib.EmDee_bond_harmonic((kb or SPCFW["kb"]) / mvv2e, SPCFW["r0"])
    angle = lib.EmDee_angle_harmonic((ka or SPCFW["ka"]) / mvv2e, SPCFW["theta0"])
    for m in range(natoms // 3):
        o, h1, h2 = 3 * m + 1, 3 * m + 2, 3 * m + 3
        lib.EmDee_add_bond(md, o, h1, bond)
        lib.EmDee_add_bond(md, o, h2, bond)
        lib.EmDee_add_angle(md, h1, o, h2, angle)


def setup_water(lib, cfg, coul, pair="shifted_force", precision=None, natoms=None, exclusions=True,
                rigid=False, coords_first=False, flexible=False, hook=None):
    """SPC/E sample (test/test_coul_*.f90:33-48): O-O Lennard-Jones (H:
    pair_none) and the Coulomb model `coul`.  With rigid=False the molecules are
    free atoms whose intramolecular pairs are excluded with EmDee_ignore_pair
    (flexible=True: with SPC/Fw bonds and angles, which exclude them instead;
    hook(lib, md), if given, runs after the models are set, before initialization);
    with rigid=True each molecule is a rigid body (EmDee_system's `bodies`
    argument, test/test_rigid_body_exact.f90:35), which drops its internal pairs
    from the neighbor lists.  coords_first uploads the coordinates before the box
    (test/test_rigid_body_exact.f90:46-48), so the bodies are set up when the box
    arrives."""
    run = cfg["run"]
    N = natoms or len(cfg["coordinates"])
    bodies = cfg["molecule"][:N] if rigid else None
    md = lib.system(1, 1, run["Rc"], run["skin"], N, cfg["type"][:N], cfg["mass"], bodies)
    if precision is not None:
        lib.EmDee_set_precision(md, precision)
    for i, (eps, sig) in enumerate(zip(cfg["epsilon"], cfg["sigma"])):
        if eps == 0.0 or pair == "none":
            p = lib.EmDee_pair_none()
        elif pair == "softcore":
            p = lib.EmDee_pair_softcore_cut(eps / run["mvv2e"], sig, 0.7)
        else:
            p = lib.EmDee_shifted_force(lib.EmDee_pair_lj_cut(eps / run["mvv2e"], sig))
        lib.EmDee_set_pair_model(md, i + 1, i + 1, p, run["kCoul"])
    lib.EmDee_set_coul_model(md, COUL_MODELS[coul](lib))
    if flexible:
        add_flexible_water(lib, md, N, run["mvv2e"])
    elif exclusions and not rigid:
        mol = cfg["molecule"][:N]
        first = {}
        for a, m in enumerate(mol):
            first.setdefault(m, []).append(a + 1)
        for atoms in first.values():
            for x in range(len(atoms)):
                for y in range(x + 1, len(atoms)):
                    lib.EmDee_ignore_pair(md, atoms[x], atoms[y])
    if hook is not None:
        hook(lib, md)
    lib.upload(md, "charges", cfg["charge"][:N])
    if coords_first:
        lib.upload(md, "coordinates", np.array(cfg["coordinates"][:N]))
        lib.upload(md, "box", np.array([cfg["box"]]))
    else:
        lib.upload(md, "box", np.array([cfg["box"]]))
        lib.upload(md, "coordinates", np.array(cfg["coordinates"][:N]))
    return md
