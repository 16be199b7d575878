"""Synthetic systems of the shapes the benchmarks and parity tests use (there is
no dataset: every input is generated from a seed).

- ``fcc``: Lennard-Jones fcc lattice jittered by U(+-jitter sigma), the first N
  sites of the smallest 4 n^3 lattice that holds N atoms.
- ``water_box``: rigid 3-site water (SPC/E geometry and charges), molecule
  centres on a simple-cubic lattice, uniformly random orientations, cubic box
  at a given mass density (units: Da, Angstrom, fs, e).
"""
import numpy as np

# units of the reference's water tests (test/spce_sample.inp)
MVV2E = 2390.057364            # (kcal/mol) / (Da A^2 / fs^2)
KB = 8.3144621455e-07          # Da A^2 / (fs^2 K)
KCOUL = 0.13893545755135628    # Da A^3 / (fs e)^2
DA_PER_G = 6.02214076e23        # Da per gram


def fcc(N, rho, jitter, seed):
    n = 1
    while 4 * n ** 3 < N:
        n += 1
    L = (N / rho) ** (1.0 / 3.0)
    a = L / n
    base = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    g = np.stack(np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij"), -1).reshape(-1, 3)
    R = (g[:, None, :] + base[None, :, :]).reshape(-1, 3)[:N] * a
    R += np.random.default_rng(seed).uniform(-jitter, jitter, size=R.shape)
    return np.ascontiguousarray(R), L


def _random_rotations(n, rng):
    """Uniform random rotation matrices from uniform unit quaternions (Shoemake's method)."""
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    q = np.stack([np.sqrt(1 - u1) * np.sin(2 * np.pi * u2), np.sqrt(1 - u1) * np.cos(2 * np.pi * u2),
                  np.sqrt(u1) * np.sin(2 * np.pi * u3), np.sqrt(u1) * np.cos(2 * np.pi * u3)], -1)
    w, x, y, z = q.T
    return np.stack([np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1),
                     np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1),
                     np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1)], -2)


WATER = dict(mass=[15.9994, 1.008], epsilon=[0.1553, 0.0], sigma=[3.166, 0.0], charge=[-0.8476, 0.4238],
             roh=1.0, angle_deg=109.47)


def water_box(nmol, seed, density=1.0):
    """Returns (R [3 nmol, 3], types, molecule ids (1-based), charges, L)."""
    n = int(round(nmol ** (1.0 / 3.0)))
    if n ** 3 != nmol:
        raise ValueError("nmol must be a cube")
    mO, mH = WATER["mass"]
    M = mO + 2 * mH
    L = (nmol * M / DA_PER_G / density * 1e24) ** (1.0 / 3.0)   # A^3 per cm^3 = 1e24
    half = np.radians(WATER["angle_deg"]) / 2
    roh = WATER["roh"]
    site = np.array([[0.0, 0.0, 0.0], [roh * np.sin(half), roh * np.cos(half), 0.0],
                     [-roh * np.sin(half), roh * np.cos(half), 0.0]])
    com = (mO * site[0] + mH * site[1] + mH * site[2]) / M
    site -= com
    rng = np.random.default_rng(seed)
    rot = _random_rotations(nmol, rng)
    g = np.stack(np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij"), -1).reshape(-1, 3)
    centres = (g + 0.5) * (L / n)
    R = (centres[:, None, :] + np.einsum("mij,sj->msi", rot, site)).reshape(-1, 3)
    types = np.tile([1, 2, 2], nmol)
    mol = np.repeat(np.arange(1, nmol + 1), 3)
    charges = np.tile([WATER["charge"][0], WATER["charge"][1], WATER["charge"][1]], nmol)
    return np.ascontiguousarray(R), types, mol, charges, L


def setup_water_box(lib, nmol, seed, precision=None, threads=1, rc=10.0, skin=1.0, damp=0.2, skin_width=1.0):
    """The 4096-molecule rigid-water workload: O-O Lennard-Jones (H: pair_none),
    coul_damped_smoothed(damp, skin_width), every molecule a rigid body."""
    R, types, mol, q, L = water_box(nmol, seed)
    md = lib.system(threads, 1, rc, skin, len(R), types, WATER["mass"], mol)
    if precision is not None:
        lib.EmDee_set_precision(md, precision)
    lib.EmDee_set_pair_model(md, 1, 1, lib.EmDee_pair_lj_cut(WATER["epsilon"][0] / MVV2E, WATER["sigma"][0]), KCOUL)
    lib.EmDee_set_pair_model(md, 2, 2, lib.EmDee_pair_none(), KCOUL)
    lib.EmDee_set_coul_model(md, lib.EmDee_coul_damped_smoothed(damp, skin_width))
    lib.upload(md, "charges", q)
    lib.upload(md, "coordinates", R)
    lib.upload(md, "box", np.array([L]))
    return md
