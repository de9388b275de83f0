"""Accuracy metrics for quaternion eigenpairs (numpy; optional torch on GPU).

Eigenvectors of H = (A -B*; B A*) are defined only up to a quaternion phase per
Kramers pair (and a unitary rotation inside clusters), so results are compared
by residual, orthonormality, subspace projection and eigenvalue error, never
element-wise. Norms: ||.||_2 of H is estimated by its largest |eigenvalue|.
"""
from __future__ import annotations

import numpy as np


def h_norm2(eig: np.ndarray) -> float:
    return float(np.max(np.abs(eig))) if eig.size else 0.0


def eig_error(eig: np.ndarray, ref: np.ndarray, hnorm: float) -> float:
    return float(np.max(np.abs(np.asarray(eig) - np.asarray(ref))) / max(hnorm, 1e-300)) if eig.size else 0.0


def residual(h: np.ndarray, v: np.ndarray, eig: np.ndarray) -> float:
    """max_j ||H v_j - lambda_j v_j||_2 / ||H||_2 over all 2n columns."""
    n = eig.size
    lam = np.concatenate([eig, eig])
    r = h @ v - v * lam
    return float(np.max(np.linalg.norm(r, axis=0)) / max(h_norm2(eig), 1e-300)) if n else 0.0


def orthonormality(v: np.ndarray) -> float:
    """max |(V^H V - I)_ij|."""
    if v.size == 0:
        return 0.0
    g = v.conj().T @ v
    return float(np.max(np.abs(g - np.eye(g.shape[0]))))


def structure_exact(d: np.ndarray, n: int) -> bool:
    """Right half equals (-conj(V); conj(U)) bit for bit."""
    u, v = d[:n, :n], d[n:2 * n, :n]
    return bool(np.array_equal(d[:n, n:2 * n], -v.conj()) and np.array_equal(d[n:2 * n, n:2 * n], u.conj()))


def subspace_distance(v: np.ndarray, eig: np.ndarray, vref: np.ndarray, eig_ref: np.ndarray, tol: float) -> float:
    """Largest sin(angle) between the invariant subspaces of matching eigenvalue clusters.

    Clusters are groups of eigenvalues closer than ``tol``; each group's 2k
    columns (both Kramers partners) span a subspace compared with the reference's.
    """
    n = eig.size
    order = np.argsort(eig)
    worst = 0.0
    i = 0
    while i < n:
        j = i + 1
        while j < n and eig[order[j]] - eig[order[j - 1]] <= tol:
            j += 1
        cols = np.concatenate([order[i:j], order[i:j] + n])
        rcols = np.concatenate([np.arange(i, j), np.arange(i, j) + n])
        a = v[:, cols]
        b = vref[:, rcols]
        # sin of the largest principal angle = ||(I - B B^H) A||_2 (accurate for small angles)
        r = a - b @ (b.conj().T @ a)
        worst = max(worst, float(np.linalg.norm(r, 2)))
        i = j
    return worst


def torch_residual(h, v, eig):
    """GPU version of residual() on torch complex128 CUDA tensors (checker only)."""
    import torch

    lam = torch.cat([eig, eig]).to(h.dtype)
    r = h @ v - v * lam
    return float(torch.linalg.vector_norm(r, dim=0).max() / eig.abs().max())


def torch_orthonormality(v):
    import torch

    g = v.conj().T @ v
    g.diagonal().sub_(1.0)
    return float(g.abs().max())


def sketch_matrix(n2: int, k: int = 4, seed: int = 0):
    """(n2, k) complex Gaussian probe S (re, im ~ N(0, 1)) from the portable generator."""
    from .inputs import PortableRNG

    rng = PortableRNG(seed)
    return rng.standard_normal((n2, k)) + 1j * rng.standard_normal((n2, k))


def sketch(v: np.ndarray, s: np.ndarray) -> np.ndarray:
    """W = V^H S: a compact fingerprint of the eigenvector matrix V (n2 x n2)."""
    return v.conj().T @ s


def sketch_distance(v: np.ndarray, eig: np.ndarray, w_ref: np.ndarray, eig_ref: np.ndarray,
                    s: np.ndarray, tol: float) -> float:
    """Subspace comparison against a reference known only through W_ref = V_ref^H S.

    For each cluster C of eigenvalues closer than ``tol`` (both Kramers partners,
    columns i and i + n), W_C^H W_C = S^H P_C S with P_C the projector onto the
    cluster's invariant subspace: independent of the quaternion phases and of any
    rotation inside the cluster. Returns the largest entry of
    |S^H (P_C - P_C,ref) S| over the clusters, divided by mean |s_i|^2 (= 2 for
    unit complex Gaussians): of the order of the sine of the largest principal
    angle between the two subspaces.
    """
    n = eig.size
    scale = float(np.mean(np.abs(s) ** 2))
    order = np.argsort(eig)
    w = v.conj().T @ s
    worst = 0.0
    i = 0
    while i < n:
        j = i + 1
        while j < n and eig[order[j]] - eig[order[j - 1]] <= tol:
            j += 1
        cols = np.concatenate([order[i:j], order[i:j] + n])
        rcols = np.concatenate([np.arange(i, j), np.arange(i, j) + n])
        k_out = w[cols].conj().T @ w[cols]
        k_ref = w_ref[rcols].conj().T @ w_ref[rcols]
        worst = max(worst, float(np.max(np.abs(k_out - k_ref))) / scale)
        i = j
    return worst
