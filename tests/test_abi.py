"""CPU checks of the C ABI: the library builds, loads without a GPU and exports
every entry point declared in include/emdee.h; the ctypes structure layout
matches the header's static asserts."""
import ctypes as C
import os
import re
import subprocess

import pytest

from conftest import ROOT
from emdee_gb300.emdee import EXTENSIONS, SIGNATURES, tEmDee, tOpts

HEADER = os.path.join(ROOT, "include", "emdee.h")


def declared_symbols():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"\b(EmDee_\w+)\s*\(", txt)))


@pytest.fixture(scope="module")
def libpath():
    from emdee_gb300.build import build
    return build()


def test_header_declares_reference_api():
    names = declared_symbols()
    for core in ["EmDee_system", "EmDee_set_pair_model", "EmDee_set_coul_model", "EmDee_upload",
                 "EmDee_download", "EmDee_compute_forces", "EmDee_boost", "EmDee_displace", "EmDee_move",
                 "EmDee_pair_lj_cut", "EmDee_pair_softcore_cut", "EmDee_coul_damped_smoothed", "EmDee_coul_long",
                 "EmDee_shifted_force", "EmDee_square_smoothed", "EmDee_random_momenta"]:
        assert core in names


def test_library_exports_every_declared_symbol(libpath):
    out = subprocess.run(["nm", "-D", "--defined-only", libpath], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (EmDee_\w+)", out))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing


def test_library_loads_without_gpu(libpath):
    lib = C.CDLL(libpath)
    for name in declared_symbols():
        assert hasattr(lib, name)
    assert set(SIGNATURES) >= set(declared_symbols())


def test_struct_layout():
    assert C.sizeof(tEmDee) == 240
    assert C.sizeof(tOpts) == 12
    assert tEmDee.Time.offset == 8 and tEmDee.Energy.offset == 40 and tEmDee.Kinetic.offset == 104
    assert tEmDee.Virial.offset == 192 and tEmDee.DoF.offset == 208 and tEmDee.Data.offset == 216


def test_oracle_exports_same_abi(oracle_path):
    out = subprocess.run(["nm", "-D", "--defined-only", oracle_path], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\bT (EmDee_\w+)", out))
    assert set(declared_symbols()) - EXTENSIONS - {"EmDee_set_precision", "EmDee_neighbor_pairs",
                                                   "EmDee_destroy"} <= exported


def test_fortran_module_matches_c_header():
    """include/emdee.f03 binds every reference entry point of include/emdee.h (the
    C-only extensions for batches, the surrogate and profiling aside), and nothing
    the C header does not declare."""
    f03 = open(os.path.join(ROOT, "include", "emdee.f03")).read()
    bound = set(re.findall(r'bind\(C,\s*name="(EmDee_\w+)"\)', f03))
    c_only = {"EmDee_boost_noalloc", "EmDee_cuda_stream", "EmDee_device_pointer", "EmDee_kernel_times",
              "EmDee_launch_count", "EmDee_neighbor_pairs", "EmDee_pair_statistics", "EmDee_profile"}
    c_only |= {n for n in EXTENSIONS if n.startswith(("EmDee_replicas_", "EmDee_surrogate_"))}
    declared = set(declared_symbols())
    assert bound <= declared, sorted(bound - declared)
    assert declared - c_only <= bound, sorted(declared - c_only - bound)
