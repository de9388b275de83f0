"""GB300-native quaternion eigensolver: a drop-in for ts::zquatev.

The compute path is libzquatev_gb300.so (hand-written sm_103a CUDA kernels
behind the C ABI in include/zquatev_gb300.h); this package holds its build
script, the ctypes binding and thin host-side helpers.
"""
from .solver import eigvals, solve, zquatev  # noqa: F401

__all__ = ["zquatev", "eigvals", "solve"]
