"""Generate the golden fixtures in this directory from the compiled reference.

Run where the reference sources are present (the fixtures are committed, so
nothing else needs them):

    make -C oracle && python tests/golden/make_golden.py

Each small fixture (random_*, clustered_*) stores the seeded input left half
[A; B], the reference's eigenvalues (eig[:n]) and its full output matrix D
(eigenvectors in the (U -V*; V U*) layout), all from oracle/_ref/liboracle.so,
the unmodified reference zquatev built by oracle/Makefile.

The large fixtures (sketch_*: the n = 256 config-0 workload and larger) keep
the repository small: the input is regenerated from its seed by the portable
generator (zquatev_gb300.inputs.PortableRNG; a checksum of the input is stored
to catch any drift), and the eigenvectors are stored as the sketch
W = D^H S for a seeded (n2 x 4) complex Gaussian S, which determines every
cluster's invariant subspace through W_C^H W_C = S^H P_C S
(zquatev_gb300.metrics.sketch_distance).
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import ref  # noqa: E402
from zquatev_gb300 import inputs  # noqa: E402

# Boundary sizes around the reference's panel/unblocked switch (n - p > nb + 1
# with nb = 20, zquatev.cc:69) plus a few ordinary ones.
RANDOM_SIZES = [1, 2, 3, 4, 8, 20, 21, 22, 23, 41, 42, 64, 100]
CLUSTERED_SIZES = [24, 64]
# (kind, n, seed): the n = 256 (n2 = 512) random matrix is the config-0 workload
SKETCHED = [("random", 256, 0), ("random", 512, 1), ("random", 1024, 3), ("clustered", 256, 2)]
SKETCH_K = 4


def sketch_seed(n: int) -> int:
    return 7000 + n


def input_checksum(left: np.ndarray) -> np.ndarray:
    n = left.shape[1]
    return np.array([np.sum(np.abs(left) ** 2), left[1 % n, 0].real, left[n + 1 % n, 0].imag, left[-1, -1].real])


def sketched_input(kind: str, n: int, seed: int) -> np.ndarray:
    if kind == "random":
        return inputs.random_matrix(n, seed, portable=True)
    d, _ = inputs.clustered_matrix(n, seed, portable=True)
    return d


def run_reference(d: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    n2 = d.shape[1]
    out = np.array(d, order="F", copy=True)
    eig = np.full(n2, np.nan)
    info = ref.zquatev(n2, out, d.shape[0], eig)
    assert info == 0, info
    return out, eig[: n2 // 2]


def main() -> None:
    if not ref.available():
        raise SystemExit("oracle/_ref/liboracle.so missing: run `make -C oracle` first")
    written = []
    for n in RANDOM_SIZES:
        seed = 1000 + n
        d = inputs.random_matrix(n, seed)
        out, eig = run_reference(d)
        path = os.path.join(HERE, f"random_n{n}.npz")
        np.savez_compressed(path, left=d[:, :n], eig=eig, out=out, seed=seed, kind="random")
        written.append(path)
    for n in CLUSTERED_SIZES:
        seed = 2000 + n
        d, lam = inputs.clustered_matrix(n, seed)
        out, eig = run_reference(d)
        path = os.path.join(HERE, f"clustered_n{n}.npz")
        np.savez_compressed(path, left=d[:, :n], eig=eig, out=out, lam=lam, seed=seed,
                            kind="clustered")
        written.append(path)
    for kind, n, seed in SKETCHED:
        d = sketched_input(kind, n, seed)
        out, eig = run_reference(d)
        from zquatev_gb300 import metrics

        s = metrics.sketch_matrix(2 * n, SKETCH_K, sketch_seed(n))
        path = os.path.join(HERE, f"sketch_{kind}_n{n}.npz")
        np.savez_compressed(path, eig=eig, sketch=metrics.sketch(out, s), seed=seed, kind=kind, n=n,
                            sketch_k=SKETCH_K, sketch_seed=sketch_seed(n), checksum=input_checksum(d[:, :n]))
        written.append(path)
    for p in written:
        print(os.path.relpath(p, ROOT), os.path.getsize(p))


if __name__ == "__main__":
    main()
