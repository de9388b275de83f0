"""ctypes handle on the compiled, unmodified reference (test infrastructure ONLY).

oracle/Makefile builds oracle/_ref/liboracle.so from the reference sources
(zquatev.cc, blocked.cc, unblocked.cc, transpose.cc) against scipy's OpenBLAS.
It exists only where those sources were present at build time; callers must
treat ``available()`` False as "pinned fixtures only".
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_ref", "liboracle.so")
# C++ linkage of ts::zquatev(int, std::complex<double>*, int, double*) (zquatev.h:54)
SYMBOL = "_ZN2ts7zquatevEiPSt7complexIdEiPd"
_lib = None


def available() -> bool:
    return os.path.exists(LIB_PATH)


def _load():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(LIB_PATH)
        fn = getattr(lib, SYMBOL)
        fn.restype = ctypes.c_int
        fn.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        _lib = fn
    return _lib


def zquatev(n2: int, d: np.ndarray, ld2: int, eig: np.ndarray) -> int:
    """Call the reference on a Fortran-ordered complex128 (ld2, n2) array in place."""
    assert d.dtype == np.complex128 and d.flags.f_contiguous
    assert eig.dtype == np.float64 and eig.flags.c_contiguous
    return _load()(n2, d.ctypes.data, ld2, eig.ctypes.data)
