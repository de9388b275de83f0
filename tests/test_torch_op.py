"""torch custom operators (zquatev_gb300/torch_ops.py): registration, shapes
under meta tensors and the absence of a CPU fallback on the CPU; the GPU
results against FP64 eigh and the plain device entry point."""
import numpy as np
import pytest
import torch

from zquatev_gb300 import inputs, metrics, torch_ops  # noqa: F401  (registers the operators)

TOL = 1e-12


def test_registered():
    assert hasattr(torch.ops.zquatev_gb300, "zquatev")
    assert hasattr(torch.ops.zquatev_gb300, "eigvalsh")


def test_meta_shapes():
    x = torch.empty((8, 4), dtype=torch.complex128, device="meta")
    eig, v = torch.ops.zquatev_gb300.zquatev(x)
    assert eig.shape == (4,) and eig.dtype == torch.float64
    assert v.shape == (8, 8) and v.dtype == torch.complex128
    assert torch.ops.zquatev_gb300.eigvalsh(x).shape == (4,)


def test_no_cpu_fallback():
    x = torch.zeros((8, 4), dtype=torch.complex128)
    with pytest.raises(Exception):
        torch.ops.zquatev_gb300.zquatev(x)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [40, 300])
def test_op_solves(gpu, n):
    d = inputs.random_matrix(n, 5150 + n)
    h_left = torch.from_numpy(np.ascontiguousarray(d[:, :n])).cuda()
    eig, v = torch.ops.zquatev_gb300.zquatev(h_left)
    vals = torch.ops.zquatev_gb300.eigvalsh(h_left)
    torch.cuda.synchronize()
    h = inputs.full_from_blocks(d[:n, :n], d[n:, :n])
    ref = np.linalg.eigvalsh(h)[::2]
    hn = metrics.h_norm2(ref)
    e, out = eig.cpu().numpy(), v.cpu().numpy()
    assert metrics.eig_error(e, ref, hn) <= TOL
    assert metrics.eig_error(vals.cpu().numpy(), ref, hn) <= TOL
    assert metrics.residual(h, out, e) <= TOL
    assert metrics.orthonormality(out) <= TOL
    assert metrics.structure_exact(np.asfortranarray(out), n)
    assert torch.equal(h_left.cpu(), torch.from_numpy(np.ascontiguousarray(d[:, :n])))  # input not modified
