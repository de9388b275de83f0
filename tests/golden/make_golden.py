"""Generate the golden fixtures in this directory from the compiled reference.

Run where the reference sources are present (the fixtures are committed, so
nothing else needs them):

    make -C oracle && python tests/golden/make_golden.py

Each fixture stores the seeded input left half [A; B], the reference's
eigenvalues (eig[:n]) and its full output matrix D (eigenvectors in the
(U -V*; V U*) layout), all from oracle/_ref/liboracle.so, the unmodified
reference zquatev built by oracle/Makefile.
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
    for p in written:
        print(os.path.relpath(p, ROOT), os.path.getsize(p))


if __name__ == "__main__":
    main()
