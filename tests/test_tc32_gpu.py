"""GPU tests of the FP32-accurate tensor-core product (zq_gemm_tf32x3: tcgen05
kind::tf32, three passes) against FP64 products of the same FP32 inputs. Bar:
every element within 1e-5 of sum_k |a_ik| |b_kj| (single-pass TF32 would be at
~1e-3); the accumulation in tensor memory loses precision with K, so long
products are measured too."""
import numpy as np
import pytest

from zquatev_gb300 import _lib

pytestmark = pytest.mark.gpu


def op(x, o):
    return {0: x, 1: x.T, 2: x.conj().T, 3: x.conj()}[o]


def run(gpu, cplx, opa, opb, m, n, k, splits=1, lda_pad=0, ldb_pad=0, seed=0):
    import torch

    rng = np.random.default_rng(seed + 7 * m + n)
    ash = (k, m) if opa in (1, 2) else (m, k)
    bsh = (n, k) if opb in (1, 2) else (k, n)
    dt = np.complex64 if cplx else np.float32

    def mk(shape):
        x = rng.standard_normal(shape)
        if cplx:
            x = x + 1j * rng.standard_normal(shape)
        return x.astype(dt)

    a, b = mk(ash), mk(bsh)
    if a.shape[0] > 1:
        a[1] *= 1e-3  # rows of different scale
    lda, ldb = ash[0] + lda_pad, bsh[0] + ldb_pad
    ta = torch.zeros((ash[1], lda), dtype=torch.complex64 if cplx else torch.float32)
    ta[:, :ash[0]] = torch.from_numpy(np.ascontiguousarray(a.T))
    tb = torch.zeros((bsh[1], ldb), dtype=ta.dtype)
    tb[:, :bsh[0]] = torch.from_numpy(np.ascontiguousarray(b.T))
    da, db = ta.cuda(), tb.cuda()
    dc = torch.full((n, m), 3.0, dtype=ta.dtype, device="cuda")
    rc = gpu.zq_gemm_tf32x3(cplx, opa, opb, m, n, k, da.data_ptr(), lda, db.data_ptr(), ldb, dc.data_ptr(), m,
                            splits, torch.cuda.current_stream().cuda_stream)
    assert rc == 0, (rc, _lib.last_error())
    c = dc.cpu().numpy().T
    a64, b64 = a.astype(np.complex128 if cplx else np.float64), b.astype(np.complex128 if cplx else np.float64)
    exact = op(a64, opa) @ op(b64, opb)
    scale = np.abs(op(a64, opa)) @ np.abs(op(b64, opb))
    return np.max(np.abs(c - exact) / scale)


@pytest.mark.parametrize("opa,opb", [(0, 0), (2, 0), (1, 0), (0, 2), (0, 1), (3, 0), (0, 3)])
@pytest.mark.parametrize("m,n,k", [(128, 128, 64), (300, 257, 700), (70, 50, 16), (1, 1, 1), (257, 129, 33)])
def test_complex(gpu, opa, opb, m, n, k):
    assert run(gpu, 1, opa, opb, m, n, k) < 1e-5


@pytest.mark.parametrize("opa,opb", [(0, 0), (1, 0), (0, 1), (1, 1)])
@pytest.mark.parametrize("m,n,k", [(128, 256, 64), (600, 300, 1000), (33, 17, 5)])
def test_real(gpu, opa, opb, m, n, k):
    assert run(gpu, 0, opa, opb, m, n, k) < 1e-5


@pytest.mark.parametrize("cplx", [1, 0])
def test_split_k_and_padding(gpu, cplx):
    assert run(gpu, cplx, 0, 0, 200, 150, 2000, splits=5, lda_pad=3, ldb_pad=1) < 1e-5
    assert run(gpu, cplx, 1, 0, 64, 64, 4096, splits=16) < 1e-5


def test_accuracy_beyond_single_tf32(gpu):
    """Three passes: far more accurate than one TF32 pass (~5e-4)."""
    assert run(gpu, 1, 0, 0, 256, 256, 512) < 3e-6


def test_timeout_path(gpu):
    import torch

    try:
        assert gpu.zq_set_pipeline_wait(200) == 0
        a = torch.ones((512, 512), dtype=torch.complex64, device="cuda")
        c = torch.zeros_like(a)
        rc = gpu.zq_gemm_tf32x3(1, 0, 0, 512, 512, 512, a.data_ptr(), 512, a.data_ptr(), 512, c.data_ptr(), 512, 1,
                                torch.cuda.current_stream().cuda_stream)
        assert rc == -104, (rc, _lib.last_error())
    finally:
        gpu.zq_set_pipeline_wait(0)
    assert run(gpu, 1, 0, 0, 128, 128, 128) < 1e-5
