"""Seeded synthetic quaternion-Hermitian inputs for the solver's workloads.

The reference diagonalises H = (A -B*; B A*) with A Hermitian and B complex
antisymmetric (B^T = -B); only the left n2 x n block [A; B] of the column-major
n2 x ld2 array is read (zquatev.cc:47-54). The reference's own driver builds A
and B from rand() (test.cc:58-69); the workloads here use Gaussian entries from
numpy's default_rng instead:

* random:    A = (X + X^H)/2, B = (Y - Y^T)/2, Re/Im of X, Y ~ N(0, 1).
* clustered: H = Q diag(lambda) Q^H with Q quaternion-unitary, lambda 80%
             uniform in [-10, 10] and 20% in clusters of 8 with gaps of 1e-6.

Arrays are numpy complex128 in Fortran order, shape (ld2, n2), matching the
column-major storage the C ABI takes.
"""
from __future__ import annotations

import numpy as np


class PortableRNG:
    """Counter-based generator (splitmix64 + Box-Muller) whose stream depends
    only on the seed: the same numbers on every machine and numpy version (up
    to the last bit of log/cos), so large fixtures can store a seed instead of
    their input. Offers the subset of numpy's Generator the workloads use."""

    _GOLDEN = np.uint64(0x9E3779B97F4A7C15)

    def __init__(self, seed: int):
        self._seed = np.uint64(seed & 0xFFFFFFFFFFFFFFFF)
        self._ctr = 0

    def _u64(self, count: int) -> np.ndarray:
        i = np.arange(self._ctr + 1, self._ctr + 1 + count, dtype=np.uint64)
        self._ctr += count
        with np.errstate(over="ignore"):
            z = self._seed + i * self._GOLDEN
            z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
            z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))

    def random(self, size) -> np.ndarray:
        count = int(np.prod(size))
        u = ((self._u64(count) >> np.uint64(11)).astype(np.float64) + 0.5) * 2.0 ** -53  # in (0, 1)
        return u.reshape(size)

    def uniform(self, lo: float, hi: float, size) -> np.ndarray:
        return lo + (hi - lo) * self.random(size)

    def standard_normal(self, size) -> np.ndarray:
        u1 = self.random(size)
        u2 = self.random(size)
        return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)


def make_rng(seed: int, portable: bool = False):
    return PortableRNG(seed) if portable else np.random.default_rng(seed)


def random_blocks(n: int, seed: int, portable: bool = False) -> tuple[np.ndarray, np.ndarray]:
    """A (Hermitian) and B (antisymmetric), n x n complex128."""
    rng = make_rng(seed, portable)
    x = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    y = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    a = (x + x.conj().T) / 2
    b = (y - y.T) / 2
    return a, b


def full_from_blocks(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """The full 2n x 2n Hermitian matrix (A -B*; B A*)."""
    n = a.shape[0]
    h = np.empty((2 * n, 2 * n), dtype=np.complex128)
    h[:n, :n] = a
    h[n:, :n] = b
    h[:n, n:] = -b.conj()
    h[n:, n:] = a.conj()
    return h


def pack_left_half(a: np.ndarray, b: np.ndarray, ld2: int | None = None,
                   fill_right: complex | None = None) -> np.ndarray:
    """Column-major (ld2, n2) array whose left half holds [A; B].

    The right half is what the caller leaves there; the solver ignores it and
    overwrites it. ``fill_right`` None writes the true right half (-B*; A*).
    """
    n = a.shape[0]
    n2 = 2 * n
    ld2 = n2 if ld2 is None else ld2
    d = np.zeros((ld2, n2), dtype=np.complex128, order="F")
    d[:n, :n] = a
    d[n:n2, :n] = b
    if fill_right is None:
        d[:n, n:] = -b.conj()
        d[n:n2, n:] = a.conj()
    else:
        d[:, n:] = fill_right
    return d


def random_matrix(n: int, seed: int, ld2: int | None = None, portable: bool = False) -> np.ndarray:
    a, b = random_blocks(n, seed, portable)
    return pack_left_half(a, b, ld2)


def quaternion_unitary(n: int, seed: int, portable: bool = False) -> tuple[np.ndarray, np.ndarray]:
    """Left half [Q0; Q1] of a Haar-like random quaternion-unitary 2n x 2n Q.

    Built by structure-preserving Gram-Schmidt on a complex Gaussian in
    quaternion form: column j is orthogonalised (twice) against the previous
    columns and their quaternion partners J*conj(q) = (-conj(q1); conj(q0)).
    """
    rng = make_rng(seed, portable)
    g = rng.standard_normal((2 * n, n)) + 1j * rng.standard_normal((2 * n, n))
    q = np.zeros((2 * n, n), dtype=np.complex128)
    for j in range(n):
        v = g[:, j].copy()
        for _ in range(2):
            if j:
                qq = q[:, :j]
                partner = np.concatenate([-qq[n:].conj(), qq[:n].conj()])
                v -= qq @ (qq.conj().T @ v)
                v -= partner @ (partner.conj().T @ v)
        q[:, j] = v / np.linalg.norm(v)
    return q[:n], q[n:]


def clustered_spectrum(n: int, seed: int, gap: float = 1e-6,
                       cluster: int = 8, frac: float = 0.2, portable: bool = False) -> np.ndarray:
    rng = make_rng(seed + 7919, portable)
    ncl = int(round(frac * n)) // cluster
    nfree = n - ncl * cluster
    lam = list(rng.uniform(-10.0, 10.0, nfree))
    for c in rng.uniform(-10.0, 10.0, ncl):
        lam.extend(c + gap * np.arange(cluster))
    return np.sort(np.asarray(lam))


def clustered_matrix(n: int, seed: int, ld2: int | None = None, portable: bool = False
                     ) -> tuple[np.ndarray, np.ndarray]:
    """(D, lambda): H = Q diag(lambda) Q^H in quaternion form, plus its spectrum."""
    q0, q1 = quaternion_unitary(n, seed, portable)
    lam = clustered_spectrum(n, seed, portable=portable)
    # H = Qf diag(lam, lam) Qf^H with Qf = (Q0 -Q1*; Q1 Q0*); left half only.
    a = (q0 * lam) @ q0.conj().T + (q1.conj() * lam) @ q1.T
    b = (q1 * lam) @ q0.conj().T - (q0.conj() * lam) @ q1.T
    a = (a + a.conj().T) / 2
    b = (b - b.T) / 2
    return pack_left_half(a, b, ld2), lam


def clustered_matrix_device(n: int, seed: int):
    """(D as a torch (n2, n2) complex128 CUDA tensor holding column-major D, lambda).

    Large-n version of clustered_matrix: the quaternion-unitary Q is the
    eigenvector matrix (exactly (U -V*; V U*)-structured, orthonormal to ~1e-14)
    that the GPU drop-in returns for a random quaternion-Hermitian matrix, and
    H = Q diag(lam, lam) Q^H is formed with torch FP64 products on the GPU.
    """
    import torch

    from . import _lib

    lib = _lib.load()
    n2 = 2 * n
    d = random_matrix(n, seed + 104729)
    dq = torch.from_numpy(np.ascontiguousarray(d.T)).cuda()
    de = torch.zeros(n2, dtype=torch.float64, device="cuda")
    rc = lib.zquatev_device(n2, dq.data_ptr(), n2, de.data_ptr(), torch.cuda.current_stream().cuda_stream)
    if rc != 0:
        raise RuntimeError(f"zquatev_device rc={rc}: {_lib.last_error()}")
    q = dq.T  # (n2, n2) column-major view: columns are eigenvectors
    lam = clustered_spectrum(n, seed)
    lt = torch.from_numpy(np.concatenate([lam, lam])).cuda().to(torch.complex128)
    h = (q * lt) @ q.conj().T
    h = (h + h.conj().T) / 2
    del dq, q
    dmat = torch.ascontiguousarray(h.T) if hasattr(torch, "ascontiguousarray") else h.T.contiguous()
    return dmat, lam


def log_uniform_sizes(count: int, lo: int, hi: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return np.floor(np.exp(rng.uniform(np.log(lo), np.log(hi), count))).astype(np.int64).clip(lo, hi)
