"""CPU checks (numpy) of the identities the GPU kernels are built on.

* The refinement forms HX from P1 = [A;B]U and P2 = [A;B]conj(V), then the
  residual R = HX - X diag(lam) for an arbitrary real lam, and recovers
  S1 = X^H H X and S2 = U^T (HX)_bot - V^T (HX)_top as X^H R + G1 diag(lam) and
  U^T R_bot - V^T R_top + G2 diag(lam); S1 is Hermitian and S2 antisymmetric,
  so their lower triangles (of the non-structured residual products plus
  G diag(lam)) determine them (zq_refine.cu, refined_solve).
* The tridiagonalisation's quaternion reflector P = I - W W^H, W = [w, J conj(w)],
  w = f (x + s x_1 e_1), s = |x| / |x_1|, f = 1 / sqrt(|x| (|x| + |x_1|)), is
  unitary, quaternion-structured, and maps x to -s x_1 e_1 (zq_tridiag.cu,
  reflector_head and w_from_x).
"""
import numpy as np

from zquatev_gb300 import inputs


def _hx(a, b, u, v):
    n = a.shape[0]
    ab = np.vstack([a, b])
    p1 = ab @ u
    p2 = ab @ v.conj()
    top = p1[:n] - p2[n:].conj()
    bot = p1[n:] + p2[:n].conj()
    return np.vstack([top, bot])


def test_hx_from_two_products():
    n = 11
    a, b = inputs.random_blocks(n, 3)
    rng = np.random.default_rng(4)
    u = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    v = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    h = inputs.full_from_blocks(a, b)
    assert np.allclose(_hx(a, b, u, v), h @ np.vstack([u, v]), atol=1e-12)


def test_residual_form_of_s():
    n = 13
    a, b = inputs.random_blocks(n, 5)
    rng = np.random.default_rng(6)
    u = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    v = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    x = np.vstack([u, v])
    hx = _hx(a, b, u, v)
    lam = rng.standard_normal(n)
    r = hx - x * lam  # R = HX - X diag(lam)
    g1 = x.conj().T @ x
    g2 = u.T @ v - v.T @ u
    s1 = x.conj().T @ hx
    s2 = u.T @ hx[n:] - v.T @ hx[:n]
    s1r = x.conj().T @ r + g1 * lam
    s2r = u.T @ r[n:] - v.T @ r[:n] + g2 * lam
    assert np.allclose(s1r, s1, atol=1e-11)
    assert np.allclose(s2r, s2, atol=1e-11)
    # S1 Hermitian, S2 antisymmetric for any X: the lower triangles determine them
    assert np.allclose(s1, s1.conj().T, atol=1e-11)
    assert np.allclose(s2, -s2.T, atol=1e-11)
    low1 = np.tril(s1r)
    fill1 = low1 + np.tril(low1, -1).conj().T
    fill1[np.diag_indices(n)] = fill1.diagonal().real
    low2 = np.tril(s2r, -1)
    fill2 = low2 - low2.T
    assert np.allclose(fill1, s1, atol=1e-11)
    assert np.allclose(fill2, s2, atol=1e-11)
    # the residual products alone are not structured (why the fill follows the addition)
    assert not np.allclose(x.conj().T @ r, (x.conj().T @ r).conj().T)


def _reflector(xa, xb):
    nu = np.sqrt(np.sum(np.abs(xa) ** 2 + np.abs(xb) ** 2))
    q1 = np.sqrt(abs(xa[0]) ** 2 + abs(xb[0]) ** 2)
    s = nu / q1
    f = 1.0 / (np.sqrt(nu) * np.sqrt(nu + q1))
    wa, wb = f * xa, f * xb
    wa[0] = f * xa[0] * (1.0 + s)
    wb[0] = f * xb[0] * (1.0 + s)
    return wa, wb, -s * xa[0], -s * xb[0]


def test_quaternion_reflector():
    rng = np.random.default_rng(7)
    L = 9
    xa = rng.standard_normal(L) + 1j * rng.standard_normal(L)
    xb = rng.standard_normal(L) + 1j * rng.standard_normal(L)
    wa, wb, ea, eb = _reflector(xa.copy(), xb.copy())
    w = np.concatenate([wa, wb])
    jw = np.concatenate([-wb.conj(), wa.conj()])  # J conj(w)
    W = np.stack([w, jw], axis=1)
    assert np.allclose(W.conj().T @ W, 2 * np.eye(2), atol=1e-13)
    p = np.eye(2 * L) - W @ W.conj().T
    assert np.allclose(p @ p.conj().T, np.eye(2 * L), atol=1e-13)
    x = np.concatenate([xa, xb])
    e = np.zeros(2 * L, dtype=complex)
    e[0], e[L] = ea, eb
    assert np.allclose(p @ x, e, atol=1e-12)
    # quaternion structure: P (J conj(y)) = J conj(P y)
    y = rng.standard_normal(2 * L) + 1j * rng.standard_normal(2 * L)
    jy = np.concatenate([-y[L:].conj(), y[:L].conj()])
    py = p @ y
    assert np.allclose(p @ jy, np.concatenate([-py[L:].conj(), py[:L].conj()]), atol=1e-12)
