"""ctypes binding of libzquatev_gb300.so (the C ABI in include/zquatev_gb300.h).

The library is built in-tree by zquatev_gb300.build. Loading fails loudly if it
is missing: there is no CPU fallback anywhere in this package.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libzquatev_gb300.so")

_c_int, _c_ll, _vp = ctypes.c_int, ctypes.c_longlong, ctypes.c_void_p

# name -> (restype, argtypes); every entry point declared in include/zquatev_gb300.h
SIGNATURES = {
    "zquatev_c": (_c_int, [_c_int, _vp, _c_int, _vp]),
    "zquatev_values": (_c_int, [_c_int, _vp, _c_int, _vp]),
    "zquatev_device": (_c_int, [_c_int, _vp, _c_int, _vp, _vp]),
    "zquatev_values_device": (_c_int, [_c_int, _vp, _c_int, _vp, _vp]),
    "zq_stedc_device": (_c_int, [_c_int, _vp, _vp, _vp, _vp, _c_int, _vp]),
    "zquatev_batched_device": (_c_int, [_c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "zquatev_device_noalloc": (_c_int, [_c_int, _vp, _c_int, _vp, _vp]),
    "zquatev_refined_device": (_c_int, [_c_int, _vp, _c_int, _vp, _vp, _c_int]),
    "zq_refine_stats": (_c_int, [ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)]),
    "zquatev_fp64_c": (_c_int, [_c_int, _vp, _c_int, _vp]),
    "zquatev_refined_c": (_c_int, [_c_int, _vp, _c_int, _vp]),
    "zquatev_fp64_device": (_c_int, [_c_int, _vp, _c_int, _vp, _vp]),
    "zq_set_path": (_c_int, [_c_int]),
    "zq_zgemm_accurate": (_c_int, [_c_int, _c_int, _c_int, _c_int, _c_int, _vp, _c_int, _vp, _c_int, _vp, _c_int, _vp]),
    "zq_profile_enable": (_c_int, [_c_int]),
    "zq_profile_read": (_c_int, [_c_int, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_longlong)]),
    "zq_profile_reset": (_c_int, []),
    "zq_profile_flops": (_c_int, [_c_int, ctypes.POINTER(ctypes.c_double)]),
    "zq_set_block_size": (_c_int, [_c_int]),
    "zq_get_block_size": (_c_int, []),
    "zq_release_workspace": (_c_int, []),
    "zq_last_error": (ctypes.c_char_p, []),
    "zq_version": (_c_int, []),
    "zq_launch_count": (_c_ll, []),
    "zq_solve_footprint": (_c_ll, [_c_int, _c_int]),
    "zq_autotune_nb": (_c_int, [_c_int, _c_int, _vp, _vp]),
    "zq_set_ozaki_kernel": (_c_int, [_c_int]),
    "zq_get_ozaki_kernel": (_c_int, []),
    "zq_set_pipeline_wait": (_c_int, [_c_ll]),
    "zq_gemm_tf32x3": (_c_int, [_c_int, _c_int, _c_int, _c_int, _c_int, _c_int, _vp, _c_int, _vp, _c_int, _vp, _c_int,
                                _c_int, _vp]),
    "zq_tuned_nb": (_c_int, [_c_int, _c_int]),
    "zq_set_tuned_nb": (_c_int, [_c_int, _c_int, _c_int]),
    "zq_batch_plan_create": (_vp, [_c_int, _vp, _vp, _vp, _vp, _c_int]),
    "zq_batch_plan_run": (_c_int, [_vp, _vp, _vp, _vp]),
    "zq_batch_plan_info": (_c_int, [_vp, _vp]),
    "zq_batch_plan_shape": (_c_int, [_vp, _vp, _vp, _vp]),
    "zq_batch_plan_destroy": (_c_int, [_vp]),
    "zq_batch_plan_variant": (_c_int, [_vp, _vp, _vp]),
    "zq_set_batch_warp_max": (_c_int, [_c_int]),
    "zq_server_create": (_vp, [_c_ll, _c_int, _c_int, _c_int]),
    "zq_server_submit": (_c_ll, [_vp, _c_int, _vp, _c_int, _vp]),
    "zq_server_test": (_c_int, [_vp, _c_ll]),
    "zq_server_wait": (_c_int, [_vp, _c_ll, _vp, _vp]),
    "zq_server_stats_read": (_c_int, [_vp, _vp]),
    "zq_server_destroy": (_c_int, [_vp]),
}


class ServerStats(ctypes.Structure):
    """zq_server_stats (include/zquatev_gb300.h)."""
    _fields_ = [(name, ctypes.c_longlong) for name in (
        "submitted", "completed", "batches", "batched_solves", "lane_solves", "refined_solves", "fp64_solves",
        "fallbacks", "queued", "in_flight")] + [("lanes", ctypes.c_int)] + [(name, ctypes.c_double) for name in (
            "budget_bytes", "reserved_bytes", "peak_reserved_bytes", "mean_reserved_bytes", "device_used_bytes")]
# the reference's C++ symbol ts::zquatev(int, std::complex<double>*, int, double*)
REFERENCE_SYMBOL = "_ZN2ts7zquatevEiPSt7complexIdEiPd"

_lib = None


class ZquatevError(RuntimeError):
    pass


def load() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ZquatevError(f"{LIB_PATH} is not built; run zquatev_gb300.build.build() first")
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        ref = getattr(lib, REFERENCE_SYMBOL)
        ref.restype = _c_int
        ref.argtypes = [_c_int, _vp, _c_int, _vp]
        _lib = lib
    return _lib


def last_error() -> str:
    msg = load().zq_last_error()
    return msg.decode() if msg else ""


def check(rc: int, what: str) -> int:
    if rc < 0:
        raise ZquatevError(f"{what} returned {rc}: {last_error()}")
    return rc


PROFILE_CLASSES = {"hemv": 0, "trail": 1, "panel": 2, "formq_gemm": 3, "apply_z": 4, "stedc": 5,
                   "tridiag": 6, "formq": 7, "batched": 8, "ozaki": 9, "refine": 10}


def profile_flops(name: str) -> float:
    f = ctypes.c_double()
    check(load().zq_profile_flops(PROFILE_CLASSES[name], ctypes.byref(f)), "zq_profile_flops")
    return f.value


def profile_read(name: str) -> tuple[float, int]:
    ms = ctypes.c_double()
    cnt = ctypes.c_longlong()
    check(load().zq_profile_read(PROFILE_CLASSES[name], ctypes.byref(ms), ctypes.byref(cnt)), "zq_profile_read")
    return ms.value, cnt.value
