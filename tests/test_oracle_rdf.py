"""Oracle check of EmDee_rdf (src/EmDeeCode.f90:1281-1395): the histogram it
normalises equals a brute-force minimum-image pair count over all atom pairs
(for Rc within the list range, every pair closer than Rc is in the lists)."""
import ctypes as C

import numpy as np
import pytest

from emdee_gb300.emdee import EmDee
from mdrun import initialize, load_golden, setup_lj_sample, velocity_verlet, setup_water

PI4_3 = 4.188790204786391


@pytest.fixture(scope="module")
def oracle(oracle_path):
    return EmDee(oracle_path)


def rdf(lib, md, bins, Rc, pairs):
    it = (C.c_int * len(pairs))(*[p[0] for p in pairs])
    jt = (C.c_int * len(pairs))(*[p[1] for p in pairs])
    g = np.zeros((len(pairs), bins))
    lib.lib.EmDee_rdf(md, bins, Rc, len(pairs), it, jt, g.ctypes.data_as(C.POINTER(C.c_double)))
    return g


def counts_from_rdf(g, bins, Rc, L, Ni, Nj, same):
    b = np.arange(1, bins + 1)
    shell = PI4_3 * (Rc / L / bins) ** 3 * (3 * b * (b - 1) + 1)
    c = g * shell * Ni * Nj
    return np.rint(c / 2.0 if same else c).astype(np.int64)


def brute_counts(R, L, A, B, bins, Rc, same):
    Rs = R / L
    d = Rs[A][:, None, :] - Rs[B][None, :, :]
    d -= np.round(d)
    r = np.sqrt((d ** 2).sum(-1)) * L
    if same:
        r = r[np.triu_indices(len(A), 1)]
    r = r[r < Rc]
    return np.bincount(np.minimum((r / Rc * bins).astype(int), bins - 1), minlength=bins)


def test_rdf_lj_counts(oracle):
    lj = load_golden("nist_lj_sample.json")
    md = setup_lj_sample(oracle, lj, "shifted_force")
    initialize(oracle, md, lj)
    velocity_verlet(oracle, md, lj["run"]["dt"], 5)
    N, L, bins, Rc = len(lj["coordinates"]), lj["box"], 40, 3.0
    g = rdf(oracle, md, bins, Rc, [(1, 1)])
    R = oracle.download(md, "coordinates", (N, 3))
    idx = np.arange(N)
    assert np.array_equal(counts_from_rdf(g[0], bins, Rc, L, N, N, True), brute_counts(R, L, idx, idx, bins, Rc, True))


def test_rdf_water_type_pairs(oracle):
    w = load_golden("nist_spce_sample.json")
    md = setup_water(oracle, w, "coul_sf")
    N, L, bins, Rc = len(w["coordinates"]), w["box"], 30, 8.0
    g = rdf(oracle, md, bins, Rc, [(1, 1), (1, 2), (2, 2)])
    R = np.array(w["coordinates"])
    t = np.array(w["type"])
    O, H = np.where(t == 1)[0], np.where(t == 2)[0]
    # intramolecular pairs are excluded from the lists, so the brute force drops them
    mol = np.array(w["molecule"])
    for k, (A, B, same) in enumerate(((O, O, True), (O, H, False), (H, H, True))):
        c = counts_from_rdf(g[k], bins, Rc, L, len(A), len(B), same)
        ref = brute_counts(R, L, A, B, bins, Rc, same)
        Rs = R / L
        intra = []
        for a in A:
            for b in B:
                if mol[a] == mol[b] and a != b and (not same or a < b):
                    dd = Rs[a] - Rs[b]
                    dd -= np.round(dd)
                    intra.append(np.sqrt((dd ** 2).sum()) * L)
        intra = np.array(intra)
        ref = ref - np.bincount(np.minimum((intra[intra < Rc] / Rc * bins).astype(int), bins - 1), minlength=bins)
        assert np.array_equal(c, ref), k
