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
