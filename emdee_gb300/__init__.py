"""GB300-native EmDee hot path: pair forces, Verlet neighbor lists and
boost/displace behind the reference's C ABI (include/emdee.h).

`load()` returns the ctypes binding of the in-tree CUDA library
(emdee_gb300/lib/libemdee.so).  There is no CPU fallback: if the library has
not been built, `load()` raises.
"""
import os

from .emdee import EmDee, FP64, MIXED  # noqa: F401

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib", "libemdee.so")
_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libemdee.so is not built; run `python -m emdee_gb300.build` "
                               "(the GB300 library has no CPU fallback)")
        _lib = EmDee(LIB_PATH)
    return _lib
