"""GPU tests of the request server (zq_server_*): results alone and in a mix,
admission by HBM footprint, routing of small requests to the batched kernel.

Each result is checked against the accuracy bar (eigenvalues within
1e-12 * ||H||_2 of FP64 eigh, residual and orthonormality <= 1e-12, exact
(U -V*; V U*) structure) and against the same request served alone:
eigenvalues within 1e-12 * ||H||_2, eigenvector subspaces per eigenvalue
cluster within 1e-8.
"""
import numpy as np
import pytest

from zquatev_gb300 import _lib, inputs, metrics
from zquatev_gb300.serve import Server

pytestmark = pytest.mark.gpu

TOL = 1e-12
SIZES = [1, 8, 20, 64, 100, 256, 257, 300, 550, 700]


def _mix():
    mats = []
    for i, n in enumerate(SIZES):
        if i % 3 == 2:
            d, _ = inputs.clustered_matrix(n, 60 + i)
        else:
            d = inputs.random_matrix(n, 60 + i)
        mats.append(d)
    return mats


def _copy(d):
    return np.array(d, dtype=np.complex128, order="F", copy=True)


def _check(d, out, eig):
    n = d.shape[1] // 2
    h = inputs.full_from_blocks(d[:n, :n], d[n:2 * n, :n])
    ref = np.linalg.eigvalsh(h)[::2]
    hn = metrics.h_norm2(ref)
    v = out[:2 * n, :2 * n]
    assert metrics.eig_error(eig[:n], ref, hn) <= TOL
    assert metrics.residual(h, v, eig[:n]) <= TOL
    assert metrics.orthonormality(v) <= TOL
    assert metrics.structure_exact(out, n)
    return hn


def test_mix_equals_alone(gpu):
    mats = _mix()
    with Server(lanes=4, batch_max_n2=512) as srv:
        alone = []
        for d in mats:
            out, eig = _copy(d), np.zeros(d.shape[1])
            rid = srv.submit(d.shape[1], out, d.shape[0], eig)
            info, t = srv.wait(rid)
            assert info == 0, _lib.last_error()
            alone.append((out, eig, t["path"]))
        outs = [(_copy(d), np.zeros(d.shape[1])) for d in mats]
        ids = [srv.submit(d.shape[1], o, d.shape[0], e) for d, (o, e) in zip(mats, outs)]
        res = [srv.wait(i) for i in ids]
        st = srv.stats()
    assert all(info == 0 for info, _ in res)
    assert st["completed"] == st["submitted"] == 2 * len(mats)
    for d, (out, eig), (aout, aeig, apath), (_, t) in zip(mats, outs, alone, res):
        n = d.shape[1] // 2
        hn = _check(d, out, eig)
        _check(d, aout, aeig)
        assert t["path"] == apath
        assert np.abs(eig[:n] - aeig[:n]).max() <= TOL * hn
        tol = 1e-6 * max(hn, 1.0)
        assert metrics.subspace_distance(out, eig[:n], aout, aeig[:n], tol) < 1e-8


@pytest.mark.parametrize("batch_max_n2", [512, 128, 0])
def test_routing_and_timestamps(gpu, batch_max_n2):
    mats = _mix()
    with Server(lanes=2, batch_max_n2=batch_max_n2) as srv:
        outs = [(_copy(d), np.zeros(d.shape[1])) for d in mats]
        ids = [srv.submit(d.shape[1], o, d.shape[0], e) for d, (o, e) in zip(mats, outs)]
        res = [srv.wait(i) for i in ids]
    for n, (info, t) in zip(SIZES, res):
        assert info == 0
        if 2 * n <= batch_max_n2:
            assert t["path"] == "batched"
        elif n >= 48:
            assert t["path"] in ("refined", "refined->fp64")
        else:
            assert t["path"] == "fp64"
        assert t["submit"] <= t["admit"] <= t["start"] <= t["done"]


def test_admission_respects_budget(gpu):
    mats = [inputs.random_matrix(n, 70 + n) for n in (600, 40, 520, 300, 16, 610)]
    # room for the largest request alone plus a little
    big = mats[-1]
    out, eig = _copy(big), np.zeros(big.shape[1])
    with Server(lanes=4) as srv:
        rid = srv.submit(big.shape[1], out, big.shape[0], eig)
        srv.wait(rid)
        one = srv.stats()["peak_reserved_bytes"]
    budget = int(one * 1.05)
    with Server(hbm_budget_bytes=budget, lanes=4) as srv:
        outs = [(_copy(d), np.zeros(d.shape[1])) for d in mats]
        ids = [srv.submit(d.shape[1], o, d.shape[0], e) for d, (o, e) in zip(mats, outs)]
        res = [srv.wait(i) for i in ids]
        st = srv.stats()
    assert st["peak_reserved_bytes"] <= budget
    assert st["reserved_bytes"] == 0
    for d, (o, e), (info, _) in zip(mats, outs, res):
        assert info == 0
        _check(d, o, e)


def test_oversized_request_rejected(gpu):
    d = inputs.random_matrix(300, 5)
    with Server(hbm_budget_bytes=1 << 20, lanes=1) as srv:
        with pytest.raises(_lib.ZquatevError):
            srv.submit(d.shape[1], _copy(d), d.shape[0], np.zeros(d.shape[1]))
        # small requests still fit
        s = inputs.random_matrix(8, 6)
        out, eig = _copy(s), np.zeros(16)
        info, t = srv.wait(srv.submit(16, out, 16, eig))
        assert info == 0 and t["path"] == "batched"
        _check(s, out, eig)


def test_argument_errors(gpu):
    with Server(lanes=1) as srv:
        with pytest.raises(_lib.ZquatevError):
            srv.submit(3, np.zeros((3, 3), dtype=np.complex128, order="F"), 3, np.zeros(3))
        info, _ = srv.wait(srv.submit(0, np.zeros((1, 1), dtype=np.complex128, order="F"), 1, np.zeros(1)))
        assert info == 0
