"""Regenerates tests/golden/*.json from the reference tree's own test fixtures.

Run once in a container that holds the reference checkout:

    python tests/golden/make_golden.py /path/to/EmDee

It reads, as data, the reference's test configurations (test/NIST_lj_sample.mol,
test/NIST_spce_sample.mol), its run parameters (test/lj_sample.inp,
test/spce_sample.inp) and the expected [U, W, U+K] triples hard-coded in
test/test_pair_lj_*.f90, and writes them as JSON so the tests run where the
reference tree is absent.  Floats are written with repr(), which round-trips
exactly.
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def read_mol(path):
    """Reads the .mol layout parsed by test/common/mConfig.f90:33-58."""
    lines = [ln for ln in open(path).read().splitlines()]
    it = iter(lines)

    def data_line():
        # each block is a '#' comment line followed by data
        while True:
            ln = next(it)
            if ln.strip() and not ln.lstrip().startswith("#"):
                return ln

    description = data_line().strip()
    ntypes = int(data_line().split()[0])
    types = {}
    for _ in range(ntypes):
        f = data_line().split()
        types[int(f[0])] = dict(mass=float(f[1]), epsilon=float(f[2]), sigma=float(f[3]))
    box = float(data_line().split()[0])  # read(inp,*) L takes the first length
    n = int(data_line().split()[0])
    atoms = [None] * n
    for _ in range(n):
        f = data_line().split()
        idx = int(f[0])
        atoms[idx - 1] = dict(mol=int(f[1]), type=int(f[2]), charge=float(f[3]),
                              r=[float(f[4]), float(f[5]), float(f[6])])
    return dict(description=description,
                mass=[types[t]["mass"] for t in range(1, ntypes + 1)],
                epsilon=[types[t]["epsilon"] for t in range(1, ntypes + 1)],
                sigma=[types[t]["sigma"] for t in range(1, ntypes + 1)],
                box=box,
                type=[a["type"] for a in atoms],
                molecule=[a["mol"] for a in atoms],
                charge=[a["charge"] for a in atoms],
                coordinates=[a["r"] for a in atoms])


def read_inp(path):
    """Reads the 12 '[...]' blocks of test/common/contained.f90:24-45."""
    keys = ["config", "Rc", "skin", "seed", "dt", "nsteps", "nprop", "temp",
            "mvv2e", "pconv", "kB", "kCoul"]
    vals = []
    lines = open(path).read().splitlines()
    for i, ln in enumerate(lines):
        if ln.startswith("["):
            vals.append(lines[i + 1].split()[0])
    out = dict(zip(keys, vals))
    for k in keys[1:]:
        out[k] = int(out[k]) if k in ("seed", "nsteps", "nprop") else float(out[k])
    return out


def expected(path):
    txt = open(path).read()
    m = re.search(r"expected\s*=\s*\[([^\]]*)\]", txt)
    return [float(v.replace("_rb", "")) for v in m.group(1).split(",")]


def main(ref):
    t = os.path.join(ref, "test")
    lj = read_mol(os.path.join(t, "NIST_lj_sample.mol"))
    lj["run"] = read_inp(os.path.join(t, "lj_sample.inp"))
    lj["expected"] = {
        name: expected(os.path.join(t, "test_%s.f90" % name))
        for name in ("pair_lj_cut", "pair_lj_sf", "pair_lj_smoothed", "pair_lj_shifted_smoothed")
    }
    lj["source"] = {"configuration": "test/NIST_lj_sample.mol", "run": "test/lj_sample.inp",
                    "expected": "test/test_pair_lj_*.f90 (the 'expected = [...]' line)"}
    with open(os.path.join(HERE, "nist_lj_sample.json"), "w") as f:
        json.dump(lj, f)
    spce = read_mol(os.path.join(t, "NIST_spce_sample.mol"))
    spce["run"] = read_inp(os.path.join(t, "spce_sample.inp"))
    spce["source"] = {"configuration": "test/NIST_spce_sample.mol", "run": "test/spce_sample.inp"}
    with open(os.path.join(HERE, "nist_spce_sample.json"), "w") as f:
        json.dump(spce, f)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <path of the EmDee source tree>")
    main(sys.argv[1])
