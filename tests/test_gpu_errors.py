"""Error behaviour of the GPU library at the C ABI, as the reference's error()
(src/global.f90:51-56): "Error in <task>: <message>." on stderr and exit(1).
Each case runs in a child process."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PRELUDE = "\n".join([
    "import sys; sys.path.insert(0, %r)" % ROOT,
    "import numpy as np, ctypes as C",
    "import emdee_gb300",
    "lib = emdee_gb300.load()",
    "md = lib.system(1, 1, 2.5, 0.3, 4)",
    "lib.EmDee_set_pair_model(md, 1, 1, lib.EmDee_pair_lj_cut(1.0, 1.0), 0.0)",
])

CASES = [
    ("lib.EmDee_add_bond(md, 1, 9, lib.EmDee_bond_harmonic(1.0, 1.0))", "atom index out of range"),
    ("lib.EmDee_add_bond(md, 1, 2, lib.EmDee_angle_harmonic(1.0, 1.0))", "must be a bond model"),
    ("lib.EmDee_add_angle(md, 1, 2, 3, lib.EmDee_bond_harmonic(1.0, 1.0))", "must be an angle model"),
    ("lib.EmDee_add_dihedral(md, 1, 2, 3, 4, lib.EmDee_bond_harmonic(1.0, 1.0))", "must be a dihedral model"),
    ("lib.upload(md, 'momenta', np.zeros((4, 3)))", "box and coordinates have not been defined"),
    ("lib.EmDee_set_pair_model(md, 1, 3, lib.EmDee_pair_lj_cut(1.0, 1.0), 0.0)", "type index is out of range"),
    ("lib.upload(md, 'box', np.array([10.0])); lib.upload(md, 'coordinates', np.random.rand(4, 3) * 10);"
     " lib.download(md, 'nonsense', (4, 3))", "invalid option"),
    ("lib.upload(md, 'box', np.array([10.0])); lib.upload(md, 'coordinates', np.random.rand(4, 3) * 10);"
     " lib.upload(md, 'charges', np.zeros(4))", "cannot set charges after"),
]


@pytest.fixture(scope="module", autouse=True)
def built():
    from emdee_gb300.build import build
    build()


@pytest.mark.parametrize("call,message", CASES)
def test_fatal_errors(call, message):
    r = subprocess.run([sys.executable, "-c", PRELUDE + "\n" + call], capture_output=True, text=True, timeout=300)
    print(r.stderr.strip().splitlines()[-1] if r.stderr.strip() else "(no stderr)")
    assert r.returncode == 1 and message in r.stderr and "Error in" in r.stderr
