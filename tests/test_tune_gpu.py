"""GPU tests of the panel-width autotuner and the graph-captured batch plan."""
import numpy as np
import pytest

from zquatev_gb300 import _lib, inputs, metrics, solver

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_autotune_nb(gpu, precision):
    best, ms = solver.autotune_nb(1024, precision)
    try:
        assert best in (16, 32, 64)
        assert all(m > 0 for m in ms)
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
    ref = master.clone()
    eref = torch.zeros(int(ns.sum()), dtype=torch.float64, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    assert gpu.zquatev_batched_device(len(ns), n2s.ctypes.data, n2s.ctypes.data, offs.ctypes.data, eoffs.ctypes.data,
                                      ref.data_ptr(), eref.data_ptr(), st) == 0
    plan = solver.BatchPlan(n2s, n2s, offs, eoffs)
    work = master.clone()
    e = torch.zeros_like(eref)
    plan.run(work, e)  # tunes the launch shape, captures, replays
    assert plan.info() == 0
    shape = plan.shape()
    assert 1 <= shape["ctas_per_sm"] <= 4 and shape["ctas"] >= 1
    # one CTA solves one matrix whatever the launch shape: results are identical
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
