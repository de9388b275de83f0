"""GPU tests of the panel-width autotuner and the graph-captured batch plan."""
import numpy as np
import pytest

from zquatev_gb300 import _lib, inputs, metrics, solver

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_autotune_nb(gpu, precision):
    best, ms = solver.autotune_nb(1024, precision)
    try:
        assert best in (16, 32, 64, 128)
        assert len(ms) == 4 and all(m > 0 for m in ms)
        assert gpu.zq_tuned_nb(1024, 0 if precision == "fp64" else 1) == best
        # solves in the tuned bucket still meet the accuracy bar
        n = 600
        d = inputs.random_matrix(n, 77)
        out = np.array(d, order="F", copy=True)
        eig = np.zeros(2 * n)
        fn = solver.zquatev_fp64 if precision == "fp64" else solver.zquatev_refined
        assert fn(2 * n, out, 2 * n, eig) == 0
        h = inputs.full_from_blocks(d[:n, :n], d[n:, :n])
        ref = np.linalg.eigvalsh(h)[::2]
        assert metrics.eig_error(eig[:n], ref, metrics.h_norm2(ref)) <= 1e-12
        assert metrics.residual(h, out, eig[:n]) <= 1e-12
    finally:
        assert gpu.zq_set_tuned_nb(1024, 0 if precision == "fp64" else 1, 0) == 0
    assert gpu.zq_tuned_nb(1024, 0 if precision == "fp64" else 1) == 0


def _batch(count, seed):
    import torch

    ns = inputs.log_uniform_sizes(count, 2, 256, seed).astype(np.int64)
    sizes = (2 * ns) ** 2
    offs = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
    eoffs = np.concatenate([[0], np.cumsum(ns)[:-1]]).astype(np.int64)
    host = np.empty(int(sizes.sum()), np.complex128)
    for i, n in enumerate(ns):
        host[offs[i]:offs[i] + sizes[i]] = inputs.random_matrix(int(n), seed + i).ravel(order="F")
    return ns, offs, eoffs, torch.from_numpy(host).cuda()


def test_batch_plan_matches_batched_call(gpu):
    import torch

    ns, offs, eoffs, master = _batch(300, 900)
    n2s = (2 * ns).astype(np.int32)
    st = torch.cuda.current_stream().cuda_stream
    plan = solver.BatchPlan(n2s, n2s, offs, eoffs)
    work = master.clone()
    e = torch.zeros(int(ns.sum()), dtype=torch.float64, device="cuda")
    plan.run(work, e)  # tunes the launch shape and the per-size variant, captures, replays
    assert plan.info() == 0
    shape = plan.shape()
    assert 1 <= shape["ctas_per_sm"] <= 4 and shape["ctas"] >= 1
    assert shape["warp_max_n"] in (0, 16, 24, 32) and all(v > 0 for v in shape["variant_ms"].values())
    # the unplanned call with the same variant switch: each matrix is solved by
    # the same kind of group whatever the launch shape, so results are identical
    assert gpu.zq_set_batch_warp_max(shape["warp_max_n"]) == 0
    try:
        ref = master.clone()
        eref = torch.zeros_like(e)
        assert gpu.zquatev_batched_device(len(ns), n2s.ctypes.data, n2s.ctypes.data, offs.ctypes.data,
                                          eoffs.ctypes.data, ref.data_ptr(), eref.data_ptr(), st) == 0
    finally:
        gpu.zq_set_batch_warp_max(-1)
    assert torch.equal(work, ref) and torch.equal(e, eref)
    for _ in range(2):  # replays of the captured graph
        work.copy_(master)
        e.zero_()
        plan.run(work, e)
        assert plan.info() == 0
        assert torch.equal(work, ref) and torch.equal(e, eref)
    plan.close()
    # accuracy of a few results
    for i in (0, 7, 150, 299):
        n = int(ns[i])
        d = master[offs[i]:offs[i] + 4 * n * n].cpu().numpy().reshape(2 * n, 2 * n, order="F")
        out = work[offs[i]:offs[i] + 4 * n * n].cpu().numpy().reshape(2 * n, 2 * n, order="F")
        h = inputs.full_from_blocks(d[:n, :n], d[n:, :n])
        w = e[eoffs[i]:eoffs[i] + n].cpu().numpy()
        assert metrics.residual(h, out, w) <= 1e-12
        assert metrics.structure_exact(out, n)


def test_batch_plan_fixed_shape_and_pointer_change(gpu):
    import torch

    ns, offs, eoffs, master = _batch(40, 31)
    n2s = (2 * ns).astype(np.int32)
    plan = solver.BatchPlan(n2s, n2s, offs, eoffs, ctas_per_sm=2)
    a, b = master.clone(), master.clone()
    ea = torch.zeros(int(ns.sum()), dtype=torch.float64, device="cuda")
    eb = torch.zeros_like(ea)
    plan.run(a, ea)
    plan.run(b, eb)  # different buffers: recaptured
    assert plan.info() == 0
    assert plan.shape()["ctas_per_sm"] == 2
    assert torch.equal(a, b) and torch.equal(ea, eb)
    plan.close()


def test_batch_plan_rejects_large(gpu):
    with pytest.raises(_lib.ZquatevError):
        solver.BatchPlan([514], [514], [0], [0])


def test_batch_variants_agree(gpu):
    """The warp-per-matrix variant (orders <= 32) and the CTA-per-matrix one
    give the same eigenpairs within the parity tolerance."""
    import torch

    ns, offs, eoffs, master = _batch(120, 4400)
    assert (ns <= 32).sum() >= 20  # log-uniform in [2, 256]: plenty for the warp variant
    n2s = (2 * ns).astype(np.int32)
    st = torch.cuda.current_stream().cuda_stream
    outs = []
    for wmax in (0, 32):
        assert gpu.zq_set_batch_warp_max(wmax) == 0
        try:
            work = master.clone()
            e = torch.zeros(int(ns.sum()), dtype=torch.float64, device="cuda")
            assert gpu.zquatev_batched_device(len(ns), n2s.ctypes.data, n2s.ctypes.data, offs.ctypes.data,
                                              eoffs.ctypes.data, work.data_ptr(), e.data_ptr(), st) == 0
        finally:
            gpu.zq_set_batch_warp_max(-1)
        outs.append((work.cpu().numpy(), e.cpu().numpy()))
    (w0, e0), (w1, e1) = outs
    for i in range(len(ns)):
        n = int(ns[i])
        d = master[offs[i]:offs[i] + 4 * n * n].cpu().numpy().reshape(2 * n, 2 * n, order="F")
        h = inputs.full_from_blocks(d[:n, :n], d[n:, :n])
        o1 = w1[offs[i]:offs[i] + 4 * n * n].reshape(2 * n, 2 * n, order="F")
        o0 = w0[offs[i]:offs[i] + 4 * n * n].reshape(2 * n, 2 * n, order="F")
        l0, l1 = e0[eoffs[i]:eoffs[i] + n], e1[eoffs[i]:eoffs[i] + n]
        hn = metrics.h_norm2(l0)
        assert metrics.eig_error(l1, l0, hn) <= 1e-12
        assert metrics.residual(h, o1, l1) <= 1e-12
        assert metrics.orthonormality(o1) <= 1e-12
        assert metrics.structure_exact(o1, n)
        assert metrics.subspace_distance(o1, l1, o0, l0, 1e-6 * hn) < 1e-8
