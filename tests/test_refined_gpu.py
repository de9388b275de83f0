"""GPU tests of the mixed-precision refined path (zquatev_refined_device).

The result must meet the same bar as the FP64 path: eigenvalues within
1e-12 * ||H||_2 of FP64 eigh, residual and orthonormality <= 1e-12, exact
(U -V*; V U*) structure, ascending order.
"""
import numpy as np
import pytest

from zquatev_gb300 import _lib, inputs, metrics

pytestmark = pytest.mark.gpu
TOL = 1e-12


def refined(lib, d, mode):
    import torch

    n2 = d.shape[1]
    dt = torch.from_numpy(np.ascontiguousarray(d.T)).cuda()
    de = torch.zeros(n2, dtype=torch.float64, device="cuda")
    rc = lib.zquatev_refined_device(n2, dt.data_ptr(), d.shape[0], de.data_ptr(),
                                    torch.cuda.current_stream().cuda_stream, mode)
    torch.cuda.synchronize()
    assert rc == 0, (rc, _lib.last_error())
    return np.asfortranarray(dt.cpu().numpy().T), de.cpu().numpy()


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("n", [2, 5, 33, 128, 300])
def test_refined_random(gpu, n, mode):
    d = inputs.random_matrix(n, 6000 + n)
    out, eig = refined(gpu, d, mode)
    h = inputs.full_from_blocks(d[:n, :n], d[n:, :n])
    ref = np.linalg.eigvalsh(h)[::2]
    hn = metrics.h_norm2(ref)
    assert metrics.eig_error(eig[:n], ref, hn) <= TOL
    assert metrics.residual(h, out, eig[:n]) <= TOL
    assert metrics.orthonormality(out) <= TOL
    assert metrics.structure_exact(out, n)
    assert np.all(np.diff(eig[:n]) >= 0)


@pytest.mark.parametrize("kernel", [0, 1, 2, 3], ids=["mma_sync", "tcgen05", "tcgen05_multicast", "tcgen05_2sm"])
@pytest.mark.parametrize("opa,opb,m,n,k", [(2, 0, 70, 50, 300), (1, 0, 70, 50, 300), (0, 0, 70, 50, 300),
                                           (0, 3, 70, 50, 300), (0, 0, 128, 128, 32), (2, 0, 300, 260, 700),
                                           (0, 0, 130, 140, 5000)])
def test_accurate_zgemm(gpu, kernel, opa, opb, m, n, k):
    """The Ozaki tensor-core product (either kernel) agrees with an extended-precision product to ~1e-15 relative."""
    import torch

    default = gpu.zq_get_ozaki_kernel()
    assert gpu.zq_set_ozaki_kernel(kernel) == 0
    rng = np.random.default_rng(opa * 10 + opb + m)
    ash = (k, m) if opa in (1, 2) else (m, k)
    bsh = (n, k) if opb in (1, 2) else (k, n)
    a = rng.standard_normal(ash) + 1j * rng.standard_normal(ash)
    b = rng.standard_normal(bsh) + 1j * rng.standard_normal(bsh)
    a[3] *= 1e-5  # rows of very different scale
    def op(x, o):
        return {0: x, 1: x.T, 2: x.conj().T, 3: x.conj()}[o]
    al = op(a.astype(np.clongdouble), opa)
    bl = op(b.astype(np.clongdouble), opb)
    exact = al @ bl
    da = torch.from_numpy(np.ascontiguousarray(a.T)).cuda()
    db = torch.from_numpy(np.ascontiguousarray(b.T)).cuda()
    dc = torch.zeros((n, m), dtype=torch.complex128, device="cuda")
    rc = gpu.zq_zgemm_accurate(opa, opb, m, n, k, da.data_ptr(), ash[0], db.data_ptr(), bsh[0], dc.data_ptr(), m,
                               torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert rc == 0, _lib.last_error()
    c = dc.cpu().numpy().T
    gpu.zq_set_ozaki_kernel(default)
    scale = np.abs(op(a, opa)) @ np.abs(op(b, opb))
    err = np.abs(c - exact.astype(np.complex128)) / scale
    assert err.max() < 2e-15


@pytest.mark.parametrize("kernel", [2, 3], ids=["multicast", "2sm"])
@pytest.mark.parametrize("n", [64, 300, 700])
def test_refined_cluster_products(gpu, n, kernel):
    """The refined path with its Ozaki products on the two-CTA cluster kernels
    (B shared by multicast, or 2-SM MMAs) — lower-triangle and full-tile
    launches, odd tile counts that leave a tile past the matrix in the last
    cluster — meets the same bar."""
    default = gpu.zq_get_ozaki_kernel()
    assert gpu.zq_set_ozaki_kernel(kernel) == 0
    try:
        d = inputs.random_matrix(n, 6300 + n)
        out, eig = refined(gpu, d, 1)
    finally:
        gpu.zq_set_ozaki_kernel(default)
    h = inputs.full_from_blocks(d[:n, :n], d[n:, :n])
    ref = np.linalg.eigvalsh(h)[::2]
    hn = metrics.h_norm2(ref)
    assert metrics.eig_error(eig[:n], ref, hn) <= TOL
    assert metrics.residual(h, out, eig[:n]) <= TOL
    assert metrics.orthonormality(out) <= TOL
    assert metrics.structure_exact(out, n)


@pytest.fixture
def mma_sync(gpu):
    default = gpu.zq_get_ozaki_kernel()
    assert gpu.zq_set_ozaki_kernel(0) == 0
    yield gpu
    gpu.zq_set_ozaki_kernel(default)


@pytest.mark.parametrize("n", [5, 64, 300, 700])
def test_refined_mma_sync_products(mma_sync, n):
    """The refined path with its Ozaki products on the mma.sync kernel meets the same bar."""
    d = inputs.random_matrix(n, 6100 + n)
    out, eig = refined(mma_sync, d, 1)
    h = inputs.full_from_blocks(d[:n, :n], d[n:, :n])
    ref = np.linalg.eigvalsh(h)[::2]
    hn = metrics.h_norm2(ref)
    assert metrics.eig_error(eig[:n], ref, hn) <= TOL
    assert metrics.residual(h, out, eig[:n]) <= TOL
    assert metrics.orthonormality(out) <= TOL
    assert metrics.structure_exact(out, n)


@pytest.mark.parametrize("n", [300, 700, 1500])
def test_refined_converges_without_fallback(gpu, n):
    """The FP32 decomposition (reduction, divide and conquer, Q formation and
    back-transform on the FP32 GEMM kernels) is accurate enough for the
    refinement to converge in at most three steps, without the FP64 fallback
    that would otherwise hide an FP32 error behind a correct result."""
    from zquatev_gb300 import solver

    d = inputs.random_matrix(n, 6200 + n)
    out, eig = refined(gpu, d, 1)
    iters, last_corr, fell_back = solver.refine_stats()
    assert not fell_back
    assert 1 <= iters <= 3, iters
    assert last_corr <= 1e-7
    h = inputs.full_from_blocks(d[:n, :n], d[n:, :n])
    ref = np.linalg.eigvalsh(h)[::2]
    assert metrics.eig_error(eig[:n], ref, metrics.h_norm2(ref)) <= TOL
    assert metrics.residual(h, out, eig[:n]) <= TOL


def _accurate_product(lib, m, n, k, seed):
    import torch

    rng = np.random.default_rng(seed)
    a = rng.standard_normal((m, k)) + 1j * rng.standard_normal((m, k))
    b = rng.standard_normal((k, n)) + 1j * rng.standard_normal((k, n))
    da = torch.from_numpy(np.ascontiguousarray(a.T)).cuda()
    db = torch.from_numpy(np.ascontiguousarray(b.T)).cuda()
    dc = torch.zeros((n, m), dtype=torch.complex128, device="cuda")
    rc = lib.zq_zgemm_accurate(0, 0, m, n, k, da.data_ptr(), m, db.data_ptr(), k, dc.data_ptr(), m,
                               torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return rc, a, b, dc.cpu().numpy().T


def test_pipeline_wait_timeout_reports_and_recovers(gpu):
    """A tcgen05 pipeline wait that runs out (a limit of a few hundred cycles,
    far below one tensor-memory copy) stops the kernel cleanly: the call returns
    -104 with its message, the device keeps answering, and the next call at the
    default limit is correct."""
    import torch

    default = gpu.zq_get_ozaki_kernel()
    assert gpu.zq_set_ozaki_kernel(1) == 0
    try:
        assert gpu.zq_set_pipeline_wait(300) == 0
        rc, _, _, _ = _accurate_product(gpu, 256, 256, 256, 5)
        assert rc == -104, (rc, _lib.last_error())
        assert "ran out of time" in _lib.last_error()
    finally:
        gpu.zq_set_pipeline_wait(0)
    assert float(torch.ones(1024, device="cuda").sum()) == 1024.0  # the context still answers
    try:
        rc, a, b, c = _accurate_product(gpu, 256, 256, 256, 5)
    finally:
        gpu.zq_set_ozaki_kernel(default)
    assert rc == 0, _lib.last_error()
    exact = a.astype(np.clongdouble) @ b.astype(np.clongdouble)
    err = np.abs(c - exact.astype(np.complex128)) / (np.abs(a) @ np.abs(b))
    assert err.max() < 2e-15
