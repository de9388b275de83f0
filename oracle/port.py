"""CPU restatement of the reference zquatev (test infrastructure ONLY).

This module is the oracle: tests, the smoke check and the CPU-baseline leg of
the benchmark call it to check or time the reference's algorithm. The product
(the CUDA library under zquatev_gb300/) never imports it.

It restates, in numpy on top of scipy's LAPACK, the reference's algorithm:

* zquatev.cc:42-100  -- repack the left half into A and B, set Q0 = I, Q1 = 0,
  reduce, solve the tridiagonal, back-transform, symmetry-fill.
* unblocked.cc:44-131 -- per column: Householder on the B column (zlarfg, then
  tau and v conjugated), symplectic Givens (zlartg/zrot with the conj trick),
  Householder on the A column; each applied two-sided to A and B and one-sided
  to Q0 and Q1 with the same gemv/ger sequence.

The reference runs the blocked panel code (blocked.cc) for all but the last
<= nb+1 columns; blocked.cc applies the same reflectors and rotations in
compact-WY form, so the unblocked restatement produces the same transforms
(only rounding differs). The tridiagonal step calls LAPACK zhbevd (scipy has
no zhbev wrapper) where the reference calls zhbev (zquatev.cc:84); both
return the ascending eigenvalues and orthonormal eigenvectors of the same
Hermitian band matrix.

Third-party arithmetic used here: LAPACK zlarfg, zlartg, zhbevd from the
scipy 1.18 OpenBLAS bundle (the reference pins no BLAS/LAPACK version).
"""
from __future__ import annotations

import numpy as np
import scipy.linalg.lapack as lapack


def _zlarfg(alpha: complex, x: np.ndarray) -> tuple[np.ndarray, complex]:
    """LAPACK zlarfg on [alpha; x]; returns (v tail, tau)."""
    n = x.size + 1
    if x.size == 0:
        x = np.zeros(1, dtype=np.complex128)
        _, _, tau = lapack.zlarfg(1, alpha, x)
        return np.zeros(0, dtype=np.complex128), complex(tau)
    _, v, tau = lapack.zlarfg(n, alpha, np.ascontiguousarray(x))
    return v, complex(tau)


def _zrot(x: np.ndarray, y: np.ndarray, c: float, s: complex) -> None:
    """BLAS zrot in place: x <- c x + s y, y <- c y - conj(s) x."""
    tx = c * x + s * y
    y[...] = c * y - np.conj(s) * x
    x[...] = tx


def unblocked_update(d0: np.ndarray, d1: np.ndarray, q0: np.ndarray, q1: np.ndarray) -> None:
    """unblocked.cc:44-131 on n x n views d0 (A), d1 (B) and norig x n views q0, q1."""
    n = d0.shape[0]
    for k in range(n - 1):
        ln = n - k - 1
        if ln > 1:
            # Householder on the B column (unblocked.cc:53-81)
            vt, tau = _zlarfg(d1[k + 1, k], d1[k + 2:, k].copy())
            tau = np.conj(tau)
            vec = np.concatenate([[1.0 + 0j], vt])
            cvec = vec.conj()
            tmp = d0[k + 1:, k:].conj().T @ cvec
            tmp[1:] += (-np.conj(tau) * 0.5 * np.vdot(tmp[1:], cvec)) * cvec
            d0[k + 1:, k:] += -np.conj(tau) * np.outer(cvec, tmp.conj())
            d0[k:, k + 1:] += -tau * np.outer(tmp, vec)
            tmp = d1[k:, k + 1:] @ cvec
            d1[k + 1:, k:] += tau * np.outer(vec, tmp)
            d1[k:, k + 1:] += -tau * np.outer(tmp, vec)
            tmp = q0[:, k + 1:] @ cvec
            q0[:, k + 1:] += -tau * np.outer(tmp, vec)
            tmp = q1[:, k + 1:] @ cvec
            q1[:, k + 1:] += -tau * np.outer(tmp, vec)

        # symplectic Givens rotation clearing B[k+1, k] (unblocked.cc:83-96)
        c, s, _ = lapack.zlartg(d0[k + 1, k], d1[k + 1, k])
        c = float(c)
        s = complex(s)
        _zrot(d0[k + 1, k:], d1[k + 1, k:], c, s)
        col = d1[k:, k + 1].conj()
        _zrot(col, d0[k:, k + 1], c, s)
        d1[k:, k + 1] = col.conj()
        col = q1[:, k + 1].conj()
        _zrot(col, q0[:, k + 1], c, s)
        q1[:, k + 1] = col.conj()

        if ln > 1:
            # Householder on the A column (unblocked.cc:98-128)
            vt, tau = _zlarfg(d0[k + 1, k], d0[k + 2:, k].copy())
            tau = np.conj(tau)
            vec = np.concatenate([[1.0 + 0j], vt])
            cvec = vec.conj()
            tmp = d0[k + 1:, k:].conj().T @ vec
            tmp[1:] += (-tau * 0.5 * np.vdot(vec, tmp[1:])) * vec
            d0[k + 1:, k:] += -tau * np.outer(vec, tmp.conj())
            d0[k:, k + 1:] += -np.conj(tau) * np.outer(tmp, cvec)
            tmp = d1[k + 1:, k:].T @ vec
            d1[k + 1:, k:] += -np.conj(tau) * np.outer(cvec, tmp)
            d1[k:, k + 1:] += np.conj(tau) * np.outer(tmp, cvec)
            tmp = q0[:, k + 1:] @ vec
            q0[:, k + 1:] += -np.conj(tau) * np.outer(tmp, cvec)
            tmp = -(q1[:, k + 1:] @ vec)
            q1[:, k + 1:] += np.conj(tau) * np.outer(tmp, cvec)


def tridiagonalize(a: np.ndarray, b: np.ndarray):
    """Symplectic reduction of (A, B): returns (diag, subdiag, Q0, Q1).

    On return Q^H H Q = T (x) I2 with T the complex Hermitian tridiagonal whose
    diagonal / first subdiagonal are returned (B is reduced to zero).
    """
    n = a.shape[0]
    d0 = np.array(a, dtype=np.complex128, order="C", copy=True)
    d1 = np.array(b, dtype=np.complex128, order="C", copy=True)
    q0 = np.eye(n, dtype=np.complex128)
    q1 = np.zeros((n, n), dtype=np.complex128)
    unblocked_update(d0, d1, q0, q1)
    return np.real(np.diag(d0)).copy(), np.diag(d0, -1).copy(), q0, q1


def zquatev(n2: int, d: np.ndarray, ld2: int, eig: np.ndarray) -> int:
    """Restatement of ts::zquatev (zquatev.cc:42-100) on a Fortran-ordered D.

    ``d`` is a complex128 array of shape (ld2, n2) in Fortran order (the
    reference's column-major storage); it is overwritten with the eigenvectors
    in the (U -V*; V U*) layout. ``eig[:n]`` receives the ascending
    eigenvalues; ``eig[n:]`` is left untouched, as in the reference. Unlike the
    reference (whose output rows depend on ld2/2), V is written at rows n..2n-1
    for any ld2 >= n2.
    """
    if n2 % 2 or n2 < 0:
        return -1
    if ld2 < max(1, n2):
        return -3
    n = n2 // 2
    if n == 0:
        return 0
    a = d[:n, :n].copy()
    b = d[n:n2, :n].copy()
    diag, sub, q0, q1 = tridiagonalize(a, b)
    # band storage kd=1, lower (zquatev.cc:79-82); zhbev -> zhbevd (see header)
    ab = np.zeros((2, n), dtype=np.complex128, order="F")
    ab[0] = diag
    ab[1, :n - 1] = sub
    w, z, info = lapack.zhbevd(ab, compute_v=1, lower=1)
    if info != 0:
        return int(info)
    u = q0 @ z
    v = q1 @ z
    d[:n, :n] = u
    d[n:n2, :n] = v
    d[:n, n:n2] = -v.conj()
    d[n:n2, n:n2] = u.conj()
    eig[:n] = w
    return 0
