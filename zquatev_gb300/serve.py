"""Python handle on the request server (zq_server_* in include/zquatev_gb300.h).

Each request is one ts::zquatev call (zquatev.h:54) on host arrays with the
reference's argument meaning: D is a Fortran-ordered (ld2, n2) complex128 array
whose left half holds [A; B] and is overwritten with the eigenvectors; eig[:n]
receives the eigenvalues; wait() returns the solver's info. The server admits
requests by HBM footprint, batches the small ones into persistent-kernel
launches and runs the larger ones on concurrent lanes; all of it happens in the
native library, this class only keeps the arrays alive until their request is
waited for.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

PATHS = {0: "fp64", 1: "refined", 2: "batched", 3: "refined->fp64"}


class Server:
    def __init__(self, hbm_budget_bytes: int = 0, lanes: int = 4, max_batch: int = 4096, batch_max_n2: int = 128):
        self._lib = _lib.load()
        self._h = self._lib.zq_server_create(int(hbm_budget_bytes), int(lanes), int(max_batch), int(batch_max_n2))
        if not self._h:
            raise _lib.ZquatevError(f"zq_server_create failed: {_lib.last_error()}")
        self._live: dict[int, tuple[np.ndarray, np.ndarray]] = {}

    def submit(self, n2: int, d: np.ndarray, ld2: int, eig: np.ndarray) -> int:
        if d.dtype != np.complex128 or not d.flags.f_contiguous:
            raise TypeError("D must be a Fortran-ordered complex128 array (column-major)")
        if eig.dtype != np.float64 or not eig.flags.c_contiguous:
            raise TypeError("eig must be a contiguous float64 array")
        if d.shape[0] != ld2 or (n2 and d.shape[1] < n2) or eig.size < n2 // 2:
            raise ValueError("array shapes do not match n2 / ld2")
        rid = self._lib.zq_server_submit(self._h, n2, d.ctypes.data, ld2, eig.ctypes.data)
        if rid < 0:
            raise _lib.ZquatevError(f"zq_server_submit returned {rid}: {_lib.last_error()}")
        self._live[rid] = (d, eig)
        return rid

    def done(self, rid: int) -> bool:
        return _lib.check(self._lib.zq_server_test(self._h, rid), "zq_server_test") == 1

    def wait(self, rid: int) -> tuple[int, dict]:
        """(info, {"submit", "admit", "start", "done": ms since creation, "path": name})."""
        t = (ctypes.c_double * 4)()
        path = ctypes.c_int()
        info = self._lib.zq_server_wait(self._h, rid, t, ctypes.byref(path))
        self._live.pop(rid, None)
        return info, {"submit": t[0], "admit": t[1], "start": t[2], "done": t[3],
                      "path": PATHS.get(path.value, str(path.value))}

    def stats(self) -> dict:
        st = _lib.ServerStats()
        _lib.check(self._lib.zq_server_stats_read(self._h, ctypes.byref(st)), "zq_server_stats_read")
        return {name: getattr(st, name) for name, _ in st._fields_}

    def close(self) -> None:
        if self._h:
            self._lib.zq_server_destroy(self._h)
            self._h = None
            self._live.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
