"""ctypes mirror of the EmDee C ABI (include/emdee.h).

`EmDee` binds every entry point of a library that exports the reference's
bind(C) interface (src/EmDeeCode.f90, src/modelClass_nonbonded.f90 and the
generated model factories of src/make_models_module.sh).  The structure
layouts follow src/emdee_header.f03:28-84.  Host programs in Python call the
library exactly as the reference's C and Fortran drivers do
(src/testc.c:116-157, test/common/contained.f90:58-72).
"""
import ctypes as C
import os

import numpy as np


class tTime(C.Structure):
    _fields_ = [("Pair", C.c_double), ("Motion", C.c_double), ("Neighbor", C.c_double), ("Total", C.c_double)]


class tEnergy(C.Structure):
    _fields_ = [("Potential", C.c_double), ("Dispersion", C.c_double), ("Coulomb", C.c_double),
                ("Bond", C.c_double), ("Angle", C.c_double), ("Dihedral", C.c_double),
                ("ShadowPotential", C.c_double), ("UpToDate", C.c_bool)]


class tKinetic(C.Structure):
    _fields_ = [("Total", C.c_double), ("TransPart", C.c_double * 3), ("Rotational", C.c_double),
                ("RotPart", C.c_double * 3), ("ShadowKinetic", C.c_double), ("ShadowRotational", C.c_double),
                ("UpToDate", C.c_bool)]


class tVirial(C.Structure):
    _fields_ = [("Total", C.c_double), ("Body", C.c_double)]


class tOpts(C.Structure):
    _fields_ = [("Translate", C.c_bool), ("Rotate", C.c_bool), ("RotationMode", C.c_int),
                ("AutoForceCompute", C.c_bool), ("AutoBodyUpdate", C.c_bool), ("Compute", C.c_bool)]


class tEmDee(C.Structure):
    _fields_ = [("Builds", C.c_int), ("Time", tTime), ("Energy", tEnergy), ("Kinetic", tKinetic),
                ("Virial", tVirial), ("DoF", C.c_int), ("RotDoF", C.c_int), ("Data", C.c_void_p),
                ("Options", tOpts)]


assert C.sizeof(tEmDee) == 240 and tEmDee.Options.offset == 224 and tEmDee.Kinetic.offset == 104

_P = C.c_void_p
_D = C.c_double
_I = C.c_int
_PT = C.POINTER(tEmDee)

# name -> (restype, argtypes)
SIGNATURES = {
    "EmDee_system": (tEmDee, [_I, _I, _D, _D, _I, _P, _P, _P]),
    "EmDee_memory_address": (_P, [tEmDee, C.c_char_p]),
    "EmDee_share_phase_space": (None, [tEmDee, _PT]),
    "EmDee_layer_based_parameters": (None, [tEmDee, _D, _P, _P]),
    "EmDee_set_pair_model": (None, [tEmDee, _I, _I, _P, _D]),
    "EmDee_set_pair_multimodel": (None, [tEmDee, _I, _I, _P, _P]),
    "EmDee_set_kspace_model": (None, [tEmDee, _P]),
    "EmDee_set_coul_model": (None, [tEmDee, _P]),
    "EmDee_set_coul_multimodel": (None, [tEmDee, _P]),
    "EmDee_ignore_pair": (None, [tEmDee, _I, _I]),
    "EmDee_add_bond": (None, [tEmDee, _I, _I, _P]),
    "EmDee_add_angle": (None, [tEmDee, _I, _I, _I, _P]),
    "EmDee_add_dihedral": (None, [tEmDee, _I, _I, _I, _I, _P]),
    "EmDee_download": (None, [tEmDee, C.c_char_p, _P]),
    "EmDee_upload": (None, [_PT, C.c_char_p, _P]),
    "EmDee_switch_model_layer": (None, [_PT, _I]),
    "EmDee_random_momenta": (None, [_PT, _D, C.c_bool, _I]),
    "EmDee_boost": (None, [_PT, _D, _D, _D]),
    "EmDee_displace": (None, [_PT, _D, _D, _D]),
    "EmDee_move": (None, [_PT, _D, _D, _D]),
    "EmDee_verlet_step": (None, [_PT, _D]),
    "EmDee_compute_forces": (None, [_PT]),
    "EmDee_rdf": (None, [tEmDee, _I, _D, _I, _P, _P, _P]),
    "EmDee_shifted": (_P, [_P]),
    "EmDee_shifted_force": (_P, [_P]),
    "EmDee_smoothed": (_P, [_P, _D]),
    "EmDee_shifted_smoothed": (_P, [_P, _D]),
    "EmDee_square_smoothed": (_P, [_P, _D]),
    "EmDee_shifted_square_smoothed": (_P, [_P, _D]),
    "EmDee_pair_none": (_P, []),
    "EmDee_coul_none": (_P, []),
    "EmDee_bond_none": (_P, []),
    "EmDee_angle_none": (_P, []),
    "EmDee_dihedral_none": (_P, []),
    "EmDee_pair_lj_cut": (_P, [_D, _D]),
    "EmDee_pair_softcore_cut": (_P, [_D, _D, _D]),
    "EmDee_coul_cut": (_P, []),
    "EmDee_coul_sf": (_P, []),
    "EmDee_coul_damped": (_P, [_D]),
    "EmDee_coul_damped_smoothed": (_P, [_D, _D]),
    "EmDee_coul_damped_square_smoothed": (_P, [_D, _D]),
    "EmDee_coul_square_smoothed": (_P, [_D]),
    "EmDee_coul_shifted_square_smoothed": (_P, [_D]),
    "EmDee_coul_long": (_P, []),
    "EmDee_kspace_ewald": (_P, [_D]),
    "EmDee_bond_harmonic": (_P, [_D, _D]),
    "EmDee_angle_harmonic": (_P, [_D, _D]),
    "EmDee_set_precision": (None, [tEmDee, _I]),
    "EmDee_set_outer_skin": (None, [tEmDee, _D]),
    "EmDee_outer_builds": (C.c_long, [tEmDee]),
    "EmDee_neighbor_pairs": (C.c_long, [tEmDee, _P, C.c_long]),
    "EmDee_destroy": (None, [_PT]),
    "EmDee_cuda_stream": (_P, [tEmDee]),
    "EmDee_profile": (None, [tEmDee, _I]),
    "EmDee_kernel_times": (_I, [tEmDee, _P, _P, _I]),
    "EmDee_pair_statistics": (None, [tEmDee, _P, _P]),
    "EmDee_launch_count": (C.c_long, [tEmDee]),
    "EmDee_tile_edge": (C.c_int, [tEmDee]),
    "EmDee_tile_threads": (C.c_int, [tEmDee, C.c_int]),
    "EmDee_boost_noalloc": (C.c_int, [_P, _P, _P, _I, _D, _D, _P, _P]),
    "EmDee_replicas_create": (C.c_void_p, [_I, _P]),
    "EmDee_replicas_run": (None, [C.c_void_p, _I, _D, _I]),
    "EmDee_replicas_block_size": (C.c_int, [C.c_void_p]),
    "EmDee_replicas_pair_threads": (C.c_int, [C.c_void_p]),
    "EmDee_replicas_destroy": (None, [C.c_void_p]),
    "EmDee_replicas_evaluate": (None, [C.c_void_p]),
    "EmDee_replicas_checkpoint": (None, [C.c_void_p]),
    "EmDee_replicas_restore": (None, [C.c_void_p, _P]),
    "EmDee_replicas_gather": (None, [C.c_void_p, C.c_char_p, _P]),
    "EmDee_replicas_scatter": (None, [C.c_void_p, C.c_char_p, _P]),
    "EmDee_device_pointer": (C.c_void_p, [tEmDee, C.c_char_p]),
    "EmDee_surrogate_param_count": (_I, []),
    "EmDee_surrogate_create": (C.c_void_p, [_I, _I, _D, _P, _D, _D, _D, _D, _D]),
    "EmDee_surrogate_set_params": (None, [C.c_void_p, _P]),
    "EmDee_surrogate_get_params": (None, [C.c_void_p, _P]),
    "EmDee_surrogate_descriptors": (None, [C.c_void_p, _P, _P, _I, _P]),
    "EmDee_surrogate_forces": (_I, [C.c_void_p, _P, _P, _P, _I, _P]),
    "EmDee_surrogate_atom_outputs": (None, [C.c_void_p, _P, _P, _P]),
    "EmDee_surrogate_gradient": (None, [C.c_void_p, _P, _P, _P, _D, _D, _P, _P, _P]),
    "EmDee_surrogate_adam": (None, [C.c_void_p, _P, _D, _I, _P]),
    "EmDee_surrogate_trajectory": (None, [C.c_void_p, _P, _P, _P, _P, _I, _D, _P]),
    "EmDee_surrogate_destroy": (None, [C.c_void_p]),
}

# entry points of the GB300 library with no counterpart in the reference
EXTENSIONS = {"EmDee_set_precision", "EmDee_set_outer_skin", "EmDee_outer_builds", "EmDee_neighbor_pairs", "EmDee_destroy", "EmDee_cuda_stream",
              "EmDee_profile", "EmDee_kernel_times", "EmDee_pair_statistics",
              "EmDee_launch_count", "EmDee_tile_edge", "EmDee_tile_threads", "EmDee_boost_noalloc", "EmDee_replicas_create", "EmDee_replicas_run",
              "EmDee_replicas_block_size", "EmDee_replicas_pair_threads", "EmDee_replicas_destroy", "EmDee_replicas_evaluate",
              "EmDee_replicas_checkpoint", "EmDee_replicas_restore", "EmDee_device_pointer",
              "EmDee_replicas_gather", "EmDee_replicas_scatter",
              "EmDee_surrogate_param_count", "EmDee_surrogate_create", "EmDee_surrogate_set_params",
              "EmDee_surrogate_get_params", "EmDee_surrogate_descriptors", "EmDee_surrogate_forces",
              "EmDee_surrogate_atom_outputs", "EmDee_surrogate_gradient", "EmDee_surrogate_adam",
              "EmDee_surrogate_trajectory", "EmDee_surrogate_destroy"}

MIXED, FP64 = 0, 1


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


class EmDee:
    """Binds one EmDee-ABI shared library and exposes it with the reference's
    names; `lib.EmDee_*` are the raw C entry points."""

    def __init__(self, path):
        if not os.path.exists(path):
            raise FileNotFoundError("EmDee library not found: %s" % path)
        self.path = path
        self.lib = C.CDLL(path, mode=C.RTLD_LOCAL)
        for name, (res, args) in SIGNATURES.items():
            if name in EXTENSIONS and not hasattr(self.lib, name):
                continue
            fn = getattr(self.lib, name)
            fn.restype = res
            fn.argtypes = args
        self._keep = []

    def __getattr__(self, name):
        if name.startswith("EmDee_"):
            return getattr(self.lib, name)
        raise AttributeError(name)

    # ---- convenience wrappers (arrays are numpy, coordinates are (N,3) float64) ----

    def system(self, threads, layers, rc, skin, N, types=None, masses=None, bodies=None):
        t = None if types is None else np.ascontiguousarray(types, dtype=np.int32)
        m = None if masses is None else np.ascontiguousarray(masses, dtype=np.float64)
        b = None if bodies is None else np.ascontiguousarray(bodies, dtype=np.int32)
        self._keep += [t, m, b]
        return self.lib.EmDee_system(threads, layers, rc, skin, N, _ptr(t), _ptr(m), _ptr(b))

    def upload(self, md, option, array):
        a = np.ascontiguousarray(array, dtype=np.float64)
        self.lib.EmDee_upload(C.byref(md), option.encode(), _ptr(a))

    def download(self, md, option, shape):
        a = np.zeros(shape, dtype=np.float64)
        self.lib.EmDee_download(md, option.encode(), _ptr(a))
        return a

    def neighbor_pairs(self, md):
        n = self.lib.EmDee_neighbor_pairs(md, None, 0)
        n = -n if n < 0 else n
        buf = np.zeros((max(n, 1), 2), dtype=np.int32)
        k = self.lib.EmDee_neighbor_pairs(md, _ptr(buf), n)
        assert k == n, (k, n)
        return buf[:n]
