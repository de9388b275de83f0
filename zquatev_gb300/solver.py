"""Python mirror of the reference's public call, ts::zquatev (zquatev.h:54).

``zquatev(n2, D, ld2, eig)`` has the reference's argument meaning and error
behaviour: D is a column-major (ld2, n2) complex128 array whose left half holds
[A; B]; it is overwritten with the eigenvectors in the (U -V*; V U*) layout;
eig[:n] receives the ascending eigenvalues; the return value is the solver's
info (0 on success). The work runs on the GPU through libzquatev_gb300.so.
"""
from __future__ import annotations

import numpy as np

from . import _lib


def _check_host(d: np.ndarray, eig: np.ndarray) -> None:
    if d.dtype != np.complex128 or not d.flags.f_contiguous:
        raise TypeError("D must be a Fortran-ordered complex128 array (column-major)")
    if eig.dtype != np.float64 or not eig.flags.c_contiguous:
        raise TypeError("eig must be a contiguous float64 array")


def zquatev(n2: int, d: np.ndarray, ld2: int, eig: np.ndarray) -> int:
    """In-place drop-in for ts::zquatev on host arrays; returns info."""
    _check_host(d, eig)
    if d.shape[0] != ld2 or (n2 and d.shape[1] < n2) or eig.size < n2 // 2:
        raise ValueError("array shapes do not match n2 / ld2")
    return _lib.load().zquatev_c(n2, d.ctypes.data, ld2, eig.ctypes.data)


def zquatev_fp64(n2: int, d: np.ndarray, ld2: int, eig: np.ndarray) -> int:
    """ts::zquatev on the plain FP64 path (no mixed precision)."""
    _check_host(d, eig)
    return _lib.load().zquatev_fp64_c(n2, d.ctypes.data, ld2, eig.ctypes.data)


def zquatev_refined(n2: int, d: np.ndarray, ld2: int, eig: np.ndarray) -> int:
    """ts::zquatev on the refined path (FP32 decomposition + Ogita-Aishima
    refinement with Ozaki tensor-core products; FP64 fallback if it does not
    converge)."""
    _check_host(d, eig)
    return _lib.load().zquatev_refined_c(n2, d.ctypes.data, ld2, eig.ctypes.data)


def refine_stats() -> tuple[int, float, bool]:
    import ctypes

    it, em, fb = ctypes.c_int(), ctypes.c_double(), ctypes.c_int()
    _lib.load().zq_refine_stats(ctypes.byref(it), ctypes.byref(em), ctypes.byref(fb))
    return it.value, em.value, bool(fb.value)


def eigvals(n2: int, d: np.ndarray, ld2: int, eig: np.ndarray) -> int:
    """Eigenvalues only (D is used as scratch)."""
    _check_host(d, eig)
    return _lib.load().zquatev_values(n2, d.ctypes.data, ld2, eig.ctypes.data)


def solve(d: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Convenience: returns (eigenvalues (n,), eigenvectors (n2, n2)) for a (ld2, n2) input."""
    out = np.array(d, dtype=np.complex128, order="F", copy=True)
    n2 = out.shape[1]
    eig = np.zeros(max(n2, 1))
    _lib.check(zquatev(n2, out, out.shape[0], eig), "zquatev_c")
    return eig[: n2 // 2].copy(), out[:n2]


# --------------------------------------------------------------- device (torch)
def zquatev_device(dmat, deig, stream=None) -> int:
    """Device-pointer variant on torch tensors.

    dmat: complex128 CUDA tensor of shape (n2, ld2) holding D^T row-major, i.e.
    the column-major (ld2, n2) array's memory; deig: float64 CUDA tensor (>= n).
    Runs on ``stream`` (default: torch's current stream) without synchronising.
    """
    import torch

    if dmat.dtype != torch.complex128 or not dmat.is_cuda or not dmat.is_contiguous():
        raise TypeError("dmat must be a contiguous complex128 CUDA tensor")
    n2, ld2 = dmat.shape[0], dmat.shape[1]
    st = stream if stream is not None else torch.cuda.current_stream(dmat.device)
    return _lib.load().zquatev_device(n2, dmat.data_ptr(), ld2, deig.data_ptr(), st.cuda_stream)


def stedc_device(d, e, lam, z, stream=None) -> int:
    """Real symmetric tridiagonal eigensolver on torch float64 CUDA tensors.

    z is an (n, n) tensor receiving Z^T row-major (= Z column-major)."""
    import torch

    n = d.numel()
    st = stream if stream is not None else torch.cuda.current_stream(d.device)
    return _lib.load().zq_stedc_device(n, d.data_ptr(), e.data_ptr() if n > 1 else 0, lam.data_ptr(),
                                       z.data_ptr(), n, st.cuda_stream)


# ------------------------------------------------------------------- tuning
def autotune_nb(n2: int, precision: str = "fp64") -> tuple[int, list[float]]:
    """Times the tridiagonalisation at order n2 for panel widths 16, 32, 64, 128 and
    stores the fastest for n2's size bucket ("fp64": plain path, "fp32": the
    refined path's decomposition). Returns (best nb, [ms per candidate])."""
    import ctypes

    best = ctypes.c_int()
    ms = (ctypes.c_double * 4)()
    prec = {"fp64": 0, "fp32": 1}[precision]
    _lib.check(_lib.load().zq_autotune_nb(n2, prec, ctypes.byref(best), ms), "zq_autotune_nb")
    return best.value, list(ms)


class BatchPlan:
    """Graph-captured batched solve of one layout of small matrices (n2 <= 512).

    Arguments as zquatev_batched_device: per-matrix n2, ld2, complex offset of
    each matrix in the device buffer and offset of its eigenvalues. With
    ctas_per_sm = 0 the first run picks the launch shape by timing each
    candidate on the caller's batch.
    """

    def __init__(self, n2s, ld2s, offs, eoffs, ctas_per_sm: int = 0):
        self._n2s = np.ascontiguousarray(n2s, dtype=np.int32)
        self._ld2s = np.ascontiguousarray(ld2s, dtype=np.int32)
        self._offs = np.ascontiguousarray(offs, dtype=np.int64)
        self._eoffs = np.ascontiguousarray(eoffs, dtype=np.int64)
        lib = _lib.load()
        self._h = lib.zq_batch_plan_create(self._n2s.size, self._n2s.ctypes.data, self._ld2s.ctypes.data,
                                           self._offs.ctypes.data, self._eoffs.ctypes.data, ctas_per_sm)
        if not self._h:
            raise _lib.ZquatevError(f"zq_batch_plan_create failed: {_lib.last_error()}")

    def run(self, dmat, deig, stream=None) -> None:
        """dmat: complex128 CUDA tensor holding the batch; deig: float64 CUDA tensor."""
        import torch

        st = stream if stream is not None else torch.cuda.current_stream(dmat.device)
        _lib.check(_lib.load().zq_batch_plan_run(self._h, dmat.data_ptr(), deig.data_ptr(), st.cuda_stream),
                   "zq_batch_plan_run")

    def info(self, stream=None) -> int:
        import torch

        st = stream if stream is not None else torch.cuda.current_stream()
        return _lib.check(_lib.load().zq_batch_plan_info(self._h, st.cuda_stream), "zq_batch_plan_info")

    def shape(self) -> dict:
        import ctypes

        cps, ctas, wmax = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        ms = (ctypes.c_double * 4)()
        vms = (ctypes.c_double * 4)()
        _lib.check(_lib.load().zq_batch_plan_shape(self._h, ctypes.byref(cps), ctypes.byref(ctas), ms),
                   "zq_batch_plan_shape")
        _lib.check(_lib.load().zq_batch_plan_variant(self._h, ctypes.byref(wmax), vms), "zq_batch_plan_variant")
        return {"ctas_per_sm": cps.value, "ctas": ctas.value, "tune_ms": list(ms), "warp_max_n": wmax.value,
                "variant_ms": dict(zip((0, 16, 24, 32), list(vms)))}

    def close(self) -> None:
        if getattr(self, "_h", None):
            _lib.load().zq_batch_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
