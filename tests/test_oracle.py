"""CPU tests of the oracle: the numpy restatement pinned to the reference's outputs.

The golden fixtures in tests/golden/ were produced by the unmodified reference
(oracle/_ref, built from its sources by oracle/Makefile) through
tests/golden/make_golden.py.
"""
import glob
import os

import numpy as np
import pytest

from oracle import port, ref
from zquatev_gb300 import inputs, metrics

GDIR = os.path.join(os.path.dirname(__file__), "golden")
GOLDEN = sorted(glob.glob(os.path.join(GDIR, "random_*.npz")) + glob.glob(os.path.join(GDIR, "clustered_*.npz")))
SKETCHED = sorted(glob.glob(os.path.join(GDIR, "sketch_*.npz")))


def load_sketched(path):
    """(n, D regenerated from the seed, fixture) of a sketched fixture; the
    regenerated input must match the stored checksum."""
    from tests.golden import make_golden

    z = np.load(path)
    n, kind, seed = int(z["n"]), str(z["kind"]), int(z["seed"])
    d = make_golden.sketched_input(kind, n, seed)
    ck = make_golden.input_checksum(d[:, :n])
    assert np.allclose(ck, z["checksum"], rtol=1e-12, atol=1e-12), "portable generator drifted"
    return n, d, z


def load(path):
    z = np.load(path)
    left = z["left"]
    n = left.shape[1]
    d = np.zeros((2 * n, 2 * n), dtype=np.complex128, order="F")
    d[:, :n] = left
    return n, d, z


def test_golden_present():
    assert len(GOLDEN) >= 10


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_golden_is_a_solution(path):
    """The reference's stored output is an eigen-decomposition of the stored input."""
    n, d, z = load(path)
    h = inputs.full_from_blocks(d[:n, :n], d[n:, :n])
    out, eig = z["out"], z["eig"]
    assert metrics.residual(h, out, eig) < 1e-13
    assert metrics.orthonormality(out) < 1e-12
    assert metrics.structure_exact(out, n)
    ref_eig = np.linalg.eigvalsh(h)[::2]
    assert metrics.eig_error(eig, ref_eig, metrics.h_norm2(ref_eig)) < 1e-13
    assert np.all(np.diff(eig) >= 0)


@pytest.mark.parametrize("path", [p for p in GOLDEN if int(p.split("_n")[-1][:-4]) <= 64],
                         ids=lambda p: os.path.basename(p))
def test_port_matches_golden(path):
    """The numpy restatement reproduces the reference's eigenpairs."""
    n, d, z = load(path)
    out = d.copy(order="F")
    eig = np.full(2 * n, 7.5)
    assert port.zquatev(2 * n, out, 2 * n, eig) == 0
    hn = metrics.h_norm2(z["eig"])
    assert metrics.eig_error(eig[:n], z["eig"], hn) < 1e-13
    assert np.all(eig[n:] == 7.5)  # eig[n..] untouched, as in the reference
    assert metrics.structure_exact(out, n)
    h = inputs.full_from_blocks(d[:n, :n], d[n:, :n])
    assert metrics.residual(h, out, eig[:n]) < 1e-13
    tol = 1e-5 * max(hn, 1.0)  # groups the 1e-6-wide clusters of the clustered fixtures
    assert metrics.subspace_distance(out, eig[:n], z["out"], z["eig"], tol) < 1e-8


def test_sketched_present():
    names = [os.path.basename(p) for p in SKETCHED]
    assert "sketch_random_n256.npz" in names  # the n2 = 512 config-0 workload
    assert any(int(p.split("_n")[-1][:-4]) >= 512 for p in SKETCHED)


@pytest.mark.parametrize("path", SKETCHED, ids=lambda p: os.path.basename(p))
def test_sketched_input_and_eigenvalues(path):
    """Regenerated inputs match their checksums; the reference's stored
    eigenvalues match FP64 eigh of the full matrix."""
    n, d, z = load_sketched(path)
    if n > 512:
        pytest.skip("eigh of the full matrix is checked up to n2 = 1024 on the CPU")
    h = inputs.full_from_blocks(d[:n, :n], d[n:, :n])
    w = np.linalg.eigvalsh(h)[::2]
    assert metrics.eig_error(z["eig"], w, metrics.h_norm2(w)) < 1e-13


@pytest.mark.parametrize("path", [p for p in SKETCHED if int(p.split("_n")[-1][:-4]) <= 256],
                         ids=lambda p: os.path.basename(p))
def test_port_matches_sketched(path):
    """The numpy restatement reproduces the reference's eigenvalues and its
    invariant subspaces (through the stored sketch) at the config-0 size."""
    n, d, z = load_sketched(path)
    out = d.copy(order="F")
    eig = np.zeros(2 * n)
    assert port.zquatev(2 * n, out, 2 * n, eig) == 0
    hn = metrics.h_norm2(z["eig"])
    assert metrics.eig_error(eig[:n], z["eig"], hn) < 1e-13
    s = metrics.sketch_matrix(2 * n, int(z["sketch_k"]), int(z["sketch_seed"]))
    tol = 1e-5 * max(hn, 1.0)
    assert metrics.sketch_distance(out, eig[:n], z["sketch"], z["eig"], s, tol) < 1e-9


def test_sketch_detects_rotation():
    """A 1e-6 rotation between two eigenvectors shows up in the sketch metric."""
    n = 16
    d = inputs.random_matrix(n, 3, portable=True)
    h = inputs.full_from_blocks(d[:n, :n], d[n:, :n])
    out = d.copy(order="F")
    eig = np.zeros(2 * n)
    assert port.zquatev(2 * n, out, 2 * n, eig) == 0
    s = metrics.sketch_matrix(2 * n, 4, 1)
    w = metrics.sketch(out, s)
    assert metrics.sketch_distance(out, eig[:n], w, eig[:n], s, 1e-9) < 1e-13
    rot = out.copy()
    c, sn = np.cos(1e-6), np.sin(1e-6)
    rot[:, 3], rot[:, 4] = c * out[:, 3] + sn * out[:, 4], -sn * out[:, 3] + c * out[:, 4]
    assert metrics.sketch_distance(rot, eig[:n], w, eig[:n], s, 1e-9) > 1e-7
    assert metrics.residual(h, out, eig[:n]) < 1e-13


def test_port_argument_errors():
    d = np.zeros((4, 4), dtype=np.complex128, order="F")
    eig = np.zeros(4)
    assert port.zquatev(3, d, 4, eig) == -1
    assert port.zquatev(4, d, 3, eig) == -3
    assert port.zquatev(0, d, 4, eig) == 0


@pytest.mark.skipif(not ref.available(), reason="compiled reference not built here")
@pytest.mark.parametrize("n", [5, 30])
def test_reference_vs_port_random(n):
    d = inputs.random_matrix(n, 99 + n)
    a = d.copy(order="F")
    b = d.copy(order="F")
    ea, eb = np.zeros(2 * n), np.zeros(2 * n)
    assert ref.zquatev(2 * n, a, 2 * n, ea) == 0
    assert port.zquatev(2 * n, b, 2 * n, eb) == 0
    assert metrics.eig_error(ea[:n], eb[:n], metrics.h_norm2(ea[:n])) < 1e-13


def test_generators():
    a, b = inputs.random_blocks(6, 1)
    assert np.allclose(a, a.conj().T) and np.allclose(b, -b.T)
    d, lam = inputs.clustered_matrix(16, 3)
    h = inputs.full_from_blocks(d[:16, :16], d[16:, :16])
    w = np.linalg.eigvalsh(h)[::2]
    assert np.max(np.abs(np.sort(lam) - w)) < 1e-12
    q0, q1 = inputs.quaternion_unitary(12, 4)
    qf = np.block([[q0, -q1.conj()], [q1, q0.conj()]])
    assert np.max(np.abs(qf.conj().T @ qf - np.eye(24))) < 1e-13
