"""GPU test of zquatev_device_noalloc, the entry point that allocates nothing.

It exists for callers that cannot call cudaMalloc (code running under an
external allocator that owns the device memory, or where allocating device
memory is not allowed); its scratch is a fixed array inside the library. The
test calls it through the C ABI twice in a row (a larger matrix, then a smaller
one, so the second call runs on scratch left over from the first) and checks
each result against the existing device entry point zquatev_device, with the
tolerances of the other parity tests. This file is collected last.
"""
import ctypes

import numpy as np
import pytest

from zquatev_gb300 import _lib, inputs, metrics

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _device_solve(lib, fn_name, d):
    import torch

    n2 = d.shape[1]
    dt = torch.from_numpy(np.ascontiguousarray(d.T)).cuda()   # column-major (ld2, n2)
    de = torch.zeros(n2, dtype=torch.float64, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    rc = getattr(lib, fn_name)(n2, dt.data_ptr(), d.shape[0], de.data_ptr(), st)
    torch.cuda.synchronize()
    assert rc == 0, (fn_name, rc, _lib.last_error())
    return np.asfortranarray(dt.cpu().numpy().T), de.cpu().numpy()


@pytest.mark.parametrize("n", [200, 37])   # two calls in a row, larger first
def test_noalloc_matches_device_entry_point(gpu, n):
    d = inputs.random_matrix(n, 4000 + n)
    out, eig = _device_solve(gpu, "zquatev_device_noalloc", d)
    ref_out, ref_eig = _device_solve(gpu, "zquatev_device", d)
    h = inputs.full_from_blocks(d[:n, :n], d[n:, :n])
    hn = metrics.h_norm2(ref_eig[:n])
    assert metrics.eig_error(eig[:n], ref_eig[:n], hn) <= TOL
    assert metrics.residual(h, out, eig[:n]) <= TOL
    assert metrics.orthonormality(out) <= TOL
    assert metrics.structure_exact(out, n)
    # eigenvectors agree with the existing entry point's up to the quaternion phase
    assert metrics.subspace_distance(out, eig[:n], ref_out, ref_eig[:n], 1e-6 * hn) < 1e-8


def test_noalloc_rejects_sizes_above_limit(gpu):
    buf = (ctypes.c_double * 8)()
    assert gpu.zquatev_device_noalloc(514, ctypes.addressof(buf), 514, ctypes.addressof(buf), None) == -103
    assert "limit" in _lib.last_error()
