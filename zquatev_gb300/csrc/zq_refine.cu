// Mixed-precision solve with iterative refinement to FP64 accuracy.
//
// Same call and output as ts::zquatev (zquatev.h:54, zquatev.cc:42-100); the
// reference computes everything in FP64. Here:
//   A. an FP32 eigendecomposition: the quaternion reduction (zq_tridiag.cu with
//      R = float), phase reduction and divide and conquer in FP64 on the
//      FP32-derived tridiagonal, Q formation and back-transform in FP32
//      -> X0 = (U0; V0), eigenvalues accurate to ~1e-6 relative;
//   B. Ogita-Aishima refinement (Ogita & Aishima, Japan J. Ind. Appl. Math.
//      35 (2018) 1007-1035), written for the quaternion structure: with
//      X^ = [X, J conj(X)] (2n x 2n, never formed) only the left halves are
//      computed,
//        G = X^^H X = [X^H X; U^T V - V^T U],  R = I - G,
//        S = X^^H H X with H X = [A U - conj(B conj V); B U + conj(A conj V)],
//        lambda_j = S_jj / G_jj,
//        E_pj = (S_pj + lambda_j R_pj) / (lambda_j - lambda_p)   (|gap| > delta)
//             = R_pj / 2                                         (otherwise),
//        X <- X + X E_top + J conj(X) E_bottom,
//      delta = 2 (||S - diag(lambda)||_2 + max|lambda| ||R||_2) as in the paper, with
//      the 2-norms estimated as sqrt(2n) x the largest entry (a Frobenius bound
//      over all 2n^2 entries would exceed typical eigenvalue gaps at n ~ 4096).
//      The products G, H X and S must be accurate to FP64 level; they go
//      through zgemm_accurate (native FP64 or the Ozaki-sliced tensor-core
//      product, zq_ozaki.cu). The update X E only needs relative accuracy
//      |E| * eps32 and runs in FP32.
//   The iteration stops when max|E| (off the Kramers pairs) is below
//   tol_converged; the caller gets the number of iterations and that value.
#include "zq_common.cuh"
#include "zq_kernels.h"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <vector>

namespace zq {

// ----------------------------------------------------------------- helpers
__global__ void k_c128_to_c64(const double2* __restrict__ src, int64_t lds, float2* __restrict__ dst, int64_t ldd,
                              int rows, int cols) {
  const int64_t total = (int64_t)rows * cols;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(t % rows), c = (int)(t / rows);
    const double2 v = src[r + (int64_t)c * lds];
    dst[r + (int64_t)c * ldd] = make_float2((float)v.x, (float)v.y);
  }
}
__global__ void k_c64_to_c128(const float2* __restrict__ src, int64_t lds, double2* __restrict__ dst, int64_t ldd,
                              int rows, int cols) {
  const int64_t total = (int64_t)rows * cols;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(t % rows), c = (int)(t / rows);
    const float2 v = src[r + (int64_t)c * lds];
    dst[r + (int64_t)c * ldd] = make_double2((double)v.x, (double)v.y);
  }
}
// x += y   (2D, complex FP64)
__global__ void k_add_c128(const double2* __restrict__ y, int64_t ldy, double2* __restrict__ x, int64_t ldx, int rows,
                           int cols) {
  const int64_t total = (int64_t)rows * cols;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(t % rows), c = (int)(t / rows);
    const double2 v = y[r + (int64_t)c * ldy];
    double2 w = x[r + (int64_t)c * ldx];
    w.x += v.x; w.y += v.y;
    x[r + (int64_t)c * ldx] = w;
  }
}

// H X from P1 = [A;B] U and P2 = [A;B] conj(V) (both 2n x n, ld):
//   (HX)_top = P1_top - conj(P2_bot),  (HX)_bot = P1_bot + conj(P2_top)
__global__ void k_hx_combine(const double2* __restrict__ P1, const double2* __restrict__ P2, int64_t ldp, int n,
                             double2* __restrict__ HX, int64_t ldh, const double2* __restrict__ X, int64_t ldx,
                             const double* __restrict__ lam) {
  // HX (left half) from P1 = [A;B] U and P2 = [A;B] conj(V); with lam given,
  // the residual R = HX - X diag(lam) instead
  const int64_t total = (int64_t)n * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(t % n), c = (int)(t / n);
    const double2 p1t = P1[r + (int64_t)c * ldp], p1b = P1[n + r + (int64_t)c * ldp];
    const double2 p2t = P2[r + (int64_t)c * ldp], p2b = P2[n + r + (int64_t)c * ldp];
    double2 top = make_double2(p1t.x - p2b.x, p1t.y + p2b.y);
    double2 bot = make_double2(p1b.x + p2t.x, p1b.y - p2t.y);
    if (lam) {
      const double l = lam[c];
      const double2 xt = X[r + (int64_t)c * ldx], xb = X[n + r + (int64_t)c * ldx];
      top.x -= xt.x * l; top.y -= xt.y * l;
      bot.x -= xb.x * l; bot.y -= xb.y * l;
    }
    HX[r + (int64_t)c * ldh] = top;
    HX[n + r + (int64_t)c * ldh] = bot;
  }
}

// S += G diag(lam) (n x n, ld n): S = X^H R + G Lambda (and the same for the
// antisymmetric pair) recovers X^H H X from the residual products
__global__ void k_add_glam(double2* __restrict__ S, const double2* __restrict__ G, int n, const double* __restrict__ lam) {
  const int64_t total = (int64_t)n * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const double l = lam[t / n];
    const double2 g = G[t];
    double2 v = S[t];
    v.x += g.x * l; v.y += g.y * l;
    S[t] = v;
  }
}

// lambda_j = Re S1_jj / Re G1_jj
__global__ void k_oa_lambda(const double2* __restrict__ S1, const double2* __restrict__ G1, int64_t ld, int n,
                            double* __restrict__ lam) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) lam[j] = S1[j + (int64_t)j * ld].x / G1[j + (int64_t)j * ld].x;
}

// partial maxima for delta: max |S - diag(lam)| and max |R| over the left half (2n x n), max |lam|
__global__ void k_oa_norms(const double2* __restrict__ S1, const double2* __restrict__ S2, const double2* __restrict__ G1,
                           const double2* __restrict__ G2, int64_t ld, int n, const double* __restrict__ lam,
                           double* __restrict__ part) {
  __shared__ double sh[32];
  unsigned long long ssb = 0, rrb = 0;  // maxima as bits (integer instructions)
  double lm = 0.0;
  const int64_t total = (int64_t)n * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % n), j = (int)(t / n);
    const int64_t o = i + (int64_t)j * ld;
    double2 s1 = S1[o], g1 = G1[o];
    if (i == j) { s1.x -= lam[j]; g1.x -= 1.0; }
    const double2 s2 = S2[o], g2 = G2[o];
    ssb = max(ssb, max(absmax_bits(s1), absmax_bits(s2)));
    rrb = max(rrb, max(absmax_bits(g1), absmax_bits(g2)));
    if (i == 0) lm = fmax(lm, fabs(lam[j]));
  }
  const double ss = block_max(bits_to_double(ssb), sh);
  const double rr = block_max(bits_to_double(rrb), sh);
  lm = block_max(lm, sh);
  if (threadIdx.x == 0) {
    part[3 * blockIdx.x + 0] = ss;
    part[3 * blockIdx.x + 1] = rr;
    part[3 * blockIdx.x + 2] = lm;
  }
}

// E_top (n x n) and E_bot (n x n), written as complex64 for the FP32 update.
// A pair (p, j) is corrected by the first-order formula only when its
// coupling c = S_pj + lambda_j R_pj is small against its gap,
// |c| <= eps_pair |lambda_j - lambda_p|; otherwise the pair belongs to an
// eigenvalue cluster: E_pj = R_pj / 2 (orthogonalisation only) and the pair is
// recorded, so the host can group the clusters and rotate inside them.
// Outputs: per-block max |E| (convergence) and max in-cluster coupling
// relative to max |lambda|.
__global__ void k_oa_build_e(const double2* __restrict__ S1, const double2* __restrict__ S2,
                             const double2* __restrict__ G1, const double2* __restrict__ G2, int64_t ld, int n,
                             const double* __restrict__ lam, const double* __restrict__ part, int nparts,
                             double2* __restrict__ Et, double2* __restrict__ Eb, int64_t lde, double* __restrict__ emax,
                             int* __restrict__ pair_count, int2* __restrict__ pairs, int pair_cap, double eps_pair) {
  __shared__ double sh[32];
  __shared__ double s_lm;
  if (threadIdx.x == 0) {
    double lm = 0.0;
    for (int q = 0; q < nparts; ++q) lm = fmax(lm, part[3 * q + 2]);
    s_lm = lm;
  }
  __syncthreads();
  const double inv_lm = s_lm > 0.0 ? 1.0 / s_lm : 1.0;
  double em = 0.0, cm = 0.0;
  const int64_t total = (int64_t)n * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % n), j = (int)(t / n);
    const int64_t o = i + (int64_t)j * ld;
    const double lj = lam[j], li = lam[i];
    const double gap = lj - li;
    // R = I - G
    double2 r1 = G1[o];
    r1.x = -r1.x; r1.y = -r1.y;
    if (i == j) r1.x += 1.0;
    const double2 g2 = G2[o];
    const double2 r2 = make_double2(-g2.x, -g2.y);
    const double2 s1 = S1[o], s2 = S2[o];
    const double2 c1 = make_double2(s1.x + lj * r1.x, s1.y + lj * r1.y);
    const double2 c2 = make_double2(s2.x + lj * r2.x, s2.y + lj * r2.y);
    // The pair test is symmetric in (i, j): the transposed entry's coupling has
    // the magnitude of S_ij + lambda_i R_ij (S1, G1 Hermitian, S2, G2
    // antisymmetric), and testing each entry with its own lambda could flag a
    // pair through (j, i) alone. Only i < j is recorded as a cluster pair, so
    // that entry would take R/2 while (i, j) took the first-order value: half
    // the pair's rotation per step (seen: |E| halving from 2.5e-5 each step).
    const double2 c1t = make_double2(s1.x + li * r1.x, s1.y + li * r1.y);
    const double2 c2t = make_double2(s2.x + li * r2.x, s2.y + li * r2.y);
    const double a1 = fmax(fmax(fabs(c1.x), fabs(c1.y)), fmax(fabs(c1t.x), fabs(c1t.y)));
    const double a2 = fmax(fmax(fabs(c2.x), fabs(c2.y)), fmax(fabs(c2t.x), fabs(c2t.y)));
    double2 e1, e2;
    bool cl = false;
    // one FP64 division per entry instead of four (FP64 divisions bounded this
    // kernel; E is a correction, its last bit does not matter)
    const double igap = (i == j) ? 0.0 : 1.0 / gap;
    if (i == j) {
      e1 = make_double2(0.5 * r1.x, 0.5 * r1.y);
    } else if (a1 <= eps_pair * fabs(gap)) {
      e1 = make_double2(c1.x * igap, c1.y * igap);
    } else {
      e1 = make_double2(0.5 * r1.x, 0.5 * r1.y);
      cl = true;
      cm = fmax(cm, a1 * inv_lm);
    }
    if (i == j || a2 > eps_pair * fabs(gap)) {
      // i == j: the Kramers partner (same eigenvalue, zero coupling by structure)
      e2 = make_double2(0.5 * r2.x, 0.5 * r2.y);
      if (i != j) { cl = true; cm = fmax(cm, a2 * inv_lm); }
    } else {
      e2 = make_double2(c2.x * igap, c2.y * igap);
    }
    if (cl && i < j) {
      const int q = atomicAdd(pair_count, 1);
      if (q < pair_cap) pairs[q] = make_int2(i, j);
    }
    Et[i + (int64_t)j * lde] = e1;
    Eb[i + (int64_t)j * lde] = e2;
    em = fmax(em, fmax(fabs(e1.x), fabs(e1.y)));
    em = fmax(em, fmax(fabs(e2.x), fabs(e2.y)));
  }
  em = block_max(em, sh);
  cm = block_max(cm, sh);
  if (threadIdx.x == 0) { emax[blockIdx.x] = em; emax[gridDim.x + blockIdx.x] = cm; }
}

// ---------------------------------------------------------------- clusters
// Gather the quaternion block of every cluster into the left half of a small
// (2k x 2k) matrix for the batched solver. The block is the orthogonalised
// Rayleigh block S + lbar (I - G) (lbar = the cluster's mean Rayleigh
// quotient): the basis is only orthonormal to ~1e-7 after the FP32 start, and
// lbar (I - G) is far larger than in-cluster gaps of 1e-6, so S alone would
// rotate by the wrong angles.
__global__ void k_cl_gather(const double2* __restrict__ S1, const double2* __restrict__ S2,
                            const double2* __restrict__ G1, const double2* __restrict__ G2, int64_t lds,
                            const double* __restrict__ lam, const int* __restrict__ members,
                            const int* __restrict__ cstart, const long long* __restrict__ coff, int ncl,
                            double2* __restrict__ blocks) {
  __shared__ double sh[32];
  const int c = blockIdx.x;
  if (c >= ncl) return;
  const int b = cstart[c], k = cstart[c + 1] - b;
  double ls = 0.0;
  for (int r = threadIdx.x; r < k; r += blockDim.x) ls += lam[members[b + r]];
  const double lbar = block_sum(ls, sh) / k;
  double2* D = blocks + coff[c];
  const int k2 = 2 * k;
  for (int t = threadIdx.x; t < k * k; t += blockDim.x) {
    const int r = t % k, q = t / k;
    const int gi = members[b + r], gj = members[b + q];
    const int64_t o = gi + (int64_t)gj * lds;
    const double2 s1 = S1[o], s2 = S2[o], g1 = G1[o], g2 = G2[o];
    const double d = (r == q) ? 1.0 : 0.0;
    D[r + (int64_t)q * k2] = make_double2(s1.x + lbar * (d - g1.x), s1.y - lbar * g1.y);
    D[k + r + (int64_t)q * k2] = make_double2(s2.x - lbar * g2.x, s2.y - lbar * g2.y);
  }
}

// X_C <- X_C W_U + J conj(X_C) W_V  (W = cluster eigenvectors, left half [W_U; W_V]);
// cluster eigenvalues replace the Rayleigh quotients.
__global__ void k_cl_rotate(double2* __restrict__ X, int64_t ldx, int n, const int* __restrict__ members,
                            const int* __restrict__ cstart, const long long* __restrict__ coff, const long long* __restrict__ eoff,
                            int ncl, const double2* __restrict__ blocks, const double* __restrict__ ceig,
                            double2* __restrict__ tmp, double* __restrict__ lam) {
  const int c = blockIdx.y;
  if (c >= ncl) return;
  const int b = cstart[c], k = cstart[c + 1] - b;
  const double2* W = blocks + coff[c];
  const int k2 = 2 * k;
  // rows of the 2n x k result, one thread per (row, column)
  const int64_t total = (int64_t)2 * n * k;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int row = (int)(t % (2 * n)), q = (int)(t / (2 * n));
    double2 acc = make_double2(0.0, 0.0);
    for (int p = 0; p < k; ++p) {
      const int col = members[b + p];
      const double2 xa = X[(row < n ? row : row - n) + (int64_t)col * ldx];
      const double2 xb = X[(row < n ? row + n : row) + (int64_t)col * ldx];
      // X_C row value and the partner J conj(X_C) row value (-conj(V) on top, conj(U) below)
      const double2 x = row < n ? xa : xb;
      const double2 y = row < n ? make_double2(-xb.x, xb.y) : make_double2(xa.x, -xa.y);
      const double2 wu = W[p + (int64_t)q * k2], wv = W[k + p + (int64_t)q * k2];
      cfma(acc, x, wu);
      cfma(acc, y, wv);
    }
    tmp[row + (int64_t)(b + q) * 2 * n] = acc;
    if (row == 0) lam[members[b + q]] = ceig[eoff[c] + q];
  }
}
__global__ void k_cl_writeback(double2* __restrict__ X, int64_t ldx, int n, const int* __restrict__ members, int total_m,
                               const double2* __restrict__ tmp) {
  const int64_t total = (int64_t)2 * n * total_m;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int row = (int)(t % (2 * n)), q = (int)(t / (2 * n));
    X[row + (int64_t)members[q] * ldx] = tmp[row + (int64_t)q * 2 * n];
  }
}

// Quaternion congruence of a structured pair (M1 Hermitian, M2 antisymmetric,
// the two halves of the Rayleigh or Gram matrix of X) by the cluster rotations
// X_C <- X_C W_U + J conj(X_C) W_V. Columns first:
//   M1[:, C] <- M1[:, C] W_U - conj(M2[:, C]) W_V
//   M2[:, C] <- M2[:, C] W_U + conj(M1[:, C]) W_V
// into tmp (n x m per matrix, m = all cluster members), blockIdx.z picks S or G.
__global__ void k_cl_congr_cols(const double2* __restrict__ S1, const double2* __restrict__ S2,
                                const double2* __restrict__ G1, const double2* __restrict__ G2, int64_t ld, int n,
                                const int* __restrict__ members, const int* __restrict__ cstart,
                                const long long* __restrict__ coff, int ncl, const double2* __restrict__ blocks, int m,
                                double2* __restrict__ tmpS, double2* __restrict__ tmpG) {
  const int c = blockIdx.y;
  if (c >= ncl) return;
  const double2* M1 = blockIdx.z ? G1 : S1;
  const double2* M2 = blockIdx.z ? G2 : S2;
  double2* T = blockIdx.z ? tmpG : tmpS;
  const int b = cstart[c], k = cstart[c + 1] - b;
  const double2* W = blocks + coff[c];
  const int k2 = 2 * k;
  const int64_t total = (int64_t)n * k;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % n), q = (int)(t / n);
    double2 a1 = make_double2(0.0, 0.0), a2 = make_double2(0.0, 0.0);
    for (int p = 0; p < k; ++p) {
      const int64_t o = i + (int64_t)members[b + p] * ld;
      const double2 m1 = M1[o], m2 = M2[o];
      const double2 wu = W[p + (int64_t)q * k2], wv = W[k + p + (int64_t)q * k2];
      cfma(a1, m1, wu);
      cfma(a1, make_double2(-m2.x, m2.y), wv);
      cfma(a2, m2, wu);
      cfma(a2, make_double2(m1.x, -m1.y), wv);
    }
    T[i + (int64_t)(b + q) * n] = a1;
    T[i + (int64_t)(b + q) * n + (int64_t)n * m] = a2;
  }
}
__global__ void k_cl_cols_writeback(double2* __restrict__ S1, double2* __restrict__ S2, double2* __restrict__ G1,
                                    double2* __restrict__ G2, int64_t ld, int n, const int* __restrict__ members, int m,
                                    const double2* __restrict__ tmpS, const double2* __restrict__ tmpG) {
  double2* M1 = blockIdx.z ? G1 : S1;
  double2* M2 = blockIdx.z ? G2 : S2;
  const double2* T = blockIdx.z ? tmpG : tmpS;
  const int64_t total = (int64_t)n * m;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % n), r = (int)(t / n);
    const int64_t o = i + (int64_t)members[r] * ld;
    M1[o] = T[t];
    M2[o] = T[t + total];
  }
}
// Rows second, on the column-transformed pair M':
//   N1[C, j] = W_U^H M1'[C, j] + W_V^H M2'[C, j],  N2[C, j] = W_U^T M2'[C, j] - W_V^T M1'[C, j]
// for member columns j; for the other columns the result's structure gives the
// row from the (already final) column: N1[C_q, j] = conj(N1[j, C_q]),
// N2[C_q, j] = -N2[j, C_q]. Into tmp (m x n per matrix).
__global__ void k_cl_congr_rows(const double2* __restrict__ S1, const double2* __restrict__ S2,
                                const double2* __restrict__ G1, const double2* __restrict__ G2, int64_t ld, int n,
                                const int* __restrict__ members, const int* __restrict__ cstart,
                                const long long* __restrict__ coff, int ncl, const double2* __restrict__ blocks,
                                const int* __restrict__ pos, int m, double2* __restrict__ tmpS, double2* __restrict__ tmpG) {
  const int c = blockIdx.y;
  if (c >= ncl) return;
  const double2* M1 = blockIdx.z ? G1 : S1;
  const double2* M2 = blockIdx.z ? G2 : S2;
  double2* T = blockIdx.z ? tmpG : tmpS;
  const int b = cstart[c], k = cstart[c + 1] - b;
  const double2* W = blocks + coff[c];
  const int k2 = 2 * k;
  const int64_t total = (int64_t)n * k;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(t % n), q = (int)(t / n);
    double2 v1, v2;
    if (pos[j] < 0) {
      const int64_t o = j + (int64_t)members[b + q] * ld;
      const double2 m1 = M1[o], m2 = M2[o];
      v1 = make_double2(m1.x, -m1.y);
      v2 = make_double2(-m2.x, -m2.y);
    } else {
      v1 = make_double2(0.0, 0.0);
      v2 = make_double2(0.0, 0.0);
      for (int p = 0; p < k; ++p) {
        const int64_t o = members[b + p] + (int64_t)j * ld;
        const double2 m1 = M1[o], m2 = M2[o];
        const double2 wu = W[p + (int64_t)q * k2], wv = W[k + p + (int64_t)q * k2];
        cfmac(v1, wu, m1);  // conj(wu) * m1
        cfmac(v1, wv, m2);
        cfma(v2, wu, m2);
        cfma(v2, make_double2(-wv.x, -wv.y), m1);
      }
    }
    T[(b + q) + (int64_t)j * m] = v1;
    T[(b + q) + (int64_t)j * m + (int64_t)n * m] = v2;
  }
}
__global__ void k_cl_rows_writeback(double2* __restrict__ S1, double2* __restrict__ S2, double2* __restrict__ G1,
                                    double2* __restrict__ G2, int64_t ld, int n, const int* __restrict__ members, int m,
                                    const double2* __restrict__ tmpS, const double2* __restrict__ tmpG) {
  double2* M1 = blockIdx.z ? G1 : S1;
  double2* M2 = blockIdx.z ? G2 : S2;
  const double2* T = blockIdx.z ? tmpG : tmpS;
  const int64_t total = (int64_t)n * m;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(t % m), j = (int)(t / m);
    const int64_t o = members[r] + (int64_t)j * ld;
    M1[o] = T[t];
    M2[o] = T[t + total];
  }
}

// ascending order after refinement: rank of each eigenvalue
__global__ void k_rank(const double* __restrict__ lam, int n, int* __restrict__ dst_of) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const double v = lam[k];
  int r = 0;
  for (int q = 0; q < n; ++q) r += (lam[q] < v) || (lam[q] == v && q < k);
  dst_of[k] = r;
}
__global__ void k_permute_cols(const double2* __restrict__ X, int64_t ldx, int rows, int n, const int* __restrict__ dst_of,
                               double2* __restrict__ Y, int64_t ldy, const double* __restrict__ lam, double* __restrict__ lam_out) {
  const int64_t total = (int64_t)rows * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(t % rows), c = (int)(t / rows);
    Y[r + (int64_t)dst_of[c] * ldy] = X[r + (int64_t)c * ldx];
    if (r == 0) lam_out[dst_of[c]] = lam[c];
  }
}

static int grid_for(int64_t total) {
  int64_t b = (total + 255) / 256;
  return (int)(b > 8192 ? 8192 : (b < 1 ? 1 : b));
}

// ----------------------------------------------------------------------------
// host driver
// ----------------------------------------------------------------------------
size_t refine_workspace_bytes(int n, int nbq) {
  const size_t nn = (size_t)n * n;
  size_t b = 0;
  b += sizeof(double2) * 2 * nn;        // H0 = [A; B] copy
  b += sizeof(float2) * 4 * nn;         // Mf: n2 x n2 complex64 (left: reduction / X0, right: X for form_q)
  b += sizeof(double2) * 2 * nn * 2;    // P1, P2 (2n x n each)
  b += sizeof(double2) * 2 * nn;        // HX
  b += sizeof(double2) * 4 * nn;        // G1, G2, S1, S2
  b += sizeof(double2) * 2 * nn;        // Et, Eb
  b += tridiag_workspace_bytes<float>(n, NBMAX);
  b += form_q_workspace_bytes(n, nbq);  // sized for double2, enough for float2
  b += sizeof(double) * (46 * (size_t)n + 3 * 8192 + 8192 + 2048 + 64);
  b += sizeof(int) * (size_t)n;
  b += 256;                             // tensor-core pipeline timeout flag
  b += 64 * 256;
  return b;
}

// accurate complex product: native FP64 (mode 0) or Ozaki-sliced tensor-core products (mode 1).
// Structured outputs (G1, S1 Hermitian; G2, S2 antisymmetric) are made exactly
// structured from their lower triangles, so that the symmetric part of E is R
// exactly and the orthogonality of the update does not depend on eigenvalue gaps.
// structured: 0 general; +-1 Hermitian / antisymmetric square output (lower
// tiles computed, upper filled); +-2 the lower triangle only, the caller fills
static int zgemm_acc(int mode, int opa1, int opb1, int opa2, int opb2, const ZgemmArgs& g, void* ows, size_t ows_bytes,
                     cudaStream_t st, int slices, int structured, int reuse_a) {
  const int sym = structured > 0 ? 1 : (structured < 0 ? -1 : 0);
  const bool fill = structured == 1 || structured == -1;
  if (mode == 1) {
    OzOpts o{};
    o.slices = slices; o.structured = sym; o.reuse_a = reuse_a; o.nofill = fill ? 0 : 1;
    return zgemm_ozaki(opa1, opb1, opa2, opb2, g, ows, ows_bytes, st, o);
  }
  if (int rc = zgemm<double>(opa1, opb1, opa2, opb2, g, 1, st)) return rc;
  if (fill) return structured_fill(g.C, g.ldc, g.m, sym, st);
  return ZQ_OK;
}

// Eigenvalue clusters (consecutive eigenvalues closer than delta): for each,
// the quaternion block [S1_CC; S2_CC] is diagonalised by the batched small
// solver and the cluster's columns are rotated by its eigenvectors.
long long batched_ws_stride();
int batched_max_n();
int batched_launch(const void* dev_tasks, int count, int* dev_counter, double2* D, double* eig, double* ws,
                   int ctas, int* dev_info, cudaStream_t st, int wmax);
size_t batched_task_bytes();
void batched_fill_task(void* dst, long long off, long long eoff, int n, int ld, int slot);

// Rayleigh-Ritz inside each eigenvalue cluster, on the current basis: group the
// coupled pairs (union-find), solve every cluster's orthogonalised quaternion
// block with the batched kernel, rotate X_C, and carry the rotation through
// S and G (rows and columns of the members), so that E is then built in the
// rotated basis and the update stays consistent with the rotation.
// tmpa / tmpb: 2 n^2 double2 each of scratch (free at this point of a step).
static int resolve_clusters(RefineArgs& ra, double2* X, int64_t ldd, double2* S1, double2* S2, double2* G1, double2* G2,
                            double* lam, const int2* dpairs, int npairs, double2* tmpa, double2* tmpb) {
  const int n = ra.n;
  cudaStream_t st = ra.st;
  std::vector<int2> hp(npairs);
  if (npairs > 0)
    ZQ_CUDA(cudaMemcpyAsync(hp.data(), dpairs, sizeof(int2) * npairs, cudaMemcpyDeviceToHost, st));
  ZQ_CUDA(cudaStreamSynchronize(st));
  std::vector<int> parent(n);
  for (int i = 0; i < n; ++i) parent[i] = i;
  auto find = [&](int x) { while (parent[x] != x) { parent[x] = parent[parent[x]]; x = parent[x]; } return x; };
  for (const int2& pr : hp) {
    const int a = find(pr.x), b = find(pr.y);
    if (a != b) parent[a > b ? a : b] = a < b ? a : b;
  }
  std::vector<std::vector<int>> groups(n);
  for (int i = 0; i < n; ++i) groups[find(i)].push_back(i);
  std::vector<int> members, cstart, pos(n, -1);
  for (int i = 0; i < n; ++i) {
    if (groups[i].size() < 2) continue;
    cstart.push_back((int)members.size());
    for (int m : groups[i]) { pos[m] = (int)members.size(); members.push_back(m); }
  }
  const int ncl = (int)cstart.size();
  ra.clusters = ncl;
  if (ncl == 0) return ZQ_OK;
  cstart.push_back((int)members.size());
  std::vector<long long> coff(ncl), eoff(ncl);
  long long off = 0, eo = 0;
  int kmax = 0;
  for (int c = 0; c < ncl; ++c) {
    const int k = cstart[c + 1] - cstart[c];
    kmax = k > kmax ? k : kmax;
    coff[c] = off; eoff[c] = eo;
    off += 4LL * k * k;
    eo += 2 * k;
  }
  if (kmax > batched_max_n()) { ra.clusters = -1; return ZQ_OK; }  // too large: leave to the FP64 fallback
  ra.cluster_max = kmax > ra.cluster_max ? kmax : ra.cluster_max;
  const int m = (int)members.size();
  const int ctas = ncl < 304 ? ncl : 304;
  const size_t tb = batched_task_bytes();
  size_t need = sizeof(double2) * (size_t)off + sizeof(double) * (size_t)eo +
                sizeof(int) * (members.size() + cstart.size() + 2 * ncl + 8 + (size_t)n) + sizeof(long long) * 2 * ncl +
                tb * ncl + sizeof(double) * (size_t)batched_ws_stride() * ctas + 16 * 256;
  void* mem = nullptr;
  ZQ_CUDA(cudaMallocAsync(&mem, need, st));
  char* p = reinterpret_cast<char*>(mem);
  auto take = [&](size_t bytes) { char* q = p; p += (bytes + 255) & ~(size_t)255; return q; };
  double2* blocks = reinterpret_cast<double2*>(take(sizeof(double2) * (size_t)off));
  double* ceig = reinterpret_cast<double*>(take(sizeof(double) * (size_t)eo));
  int* dmem = reinterpret_cast<int*>(take(sizeof(int) * members.size()));
  int* dcs = reinterpret_cast<int*>(take(sizeof(int) * cstart.size()));
  int* dpos = reinterpret_cast<int*>(take(sizeof(int) * (size_t)n));
  long long* dco = reinterpret_cast<long long*>(take(sizeof(long long) * ncl));
  long long* deo = reinterpret_cast<long long*>(take(sizeof(long long) * ncl));
  int* dinf = reinterpret_cast<int*>(take(sizeof(int) * (ncl + 8)));
  void* dtasks = take(tb * ncl);
  double* bws = reinterpret_cast<double*>(take(sizeof(double) * (size_t)batched_ws_stride() * ctas));
  std::vector<char> htasks(tb * ncl);
  for (int c = 0; c < ncl; ++c) {
    const int k = cstart[c + 1] - cstart[c];
    batched_fill_task(htasks.data() + c * tb, coff[c], eoff[c], k, 2 * k, c);
  }
  ZQ_CUDA(cudaMemcpyAsync(dmem, members.data(), sizeof(int) * members.size(), cudaMemcpyHostToDevice, st));
  ZQ_CUDA(cudaMemcpyAsync(dcs, cstart.data(), sizeof(int) * cstart.size(), cudaMemcpyHostToDevice, st));
  ZQ_CUDA(cudaMemcpyAsync(dpos, pos.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, st));
  ZQ_CUDA(cudaMemcpyAsync(dco, coff.data(), sizeof(long long) * ncl, cudaMemcpyHostToDevice, st));
  ZQ_CUDA(cudaMemcpyAsync(deo, eoff.data(), sizeof(long long) * ncl, cudaMemcpyHostToDevice, st));
  ZQ_CUDA(cudaMemcpyAsync(dtasks, htasks.data(), tb * ncl, cudaMemcpyHostToDevice, st));
  k_cl_gather<<<ncl, 256, 0, st>>>(S1, S2, G1, G2, n, lam, dmem, dcs, dco, ncl, blocks);
  ZQ_LAUNCH_CHECK();
  // cluster blocks are not queued by size: one CTA per block (no warp variant)
  if (int rc = batched_launch(dtasks, ncl, dinf + ncl, blocks, ceig, bws, ctas, dinf, st, 0)) return rc;
  // X_C (2n x m scratch in tmpa)
  const int gx = ceil_div(2 * n * kmax, 256) > 64 ? 64 : ceil_div(2 * n * kmax, 256);
  k_cl_rotate<<<dim3(gx, ncl), 256, 0, st>>>(X, ldd, n, dmem, dcs, dco, deo, ncl, blocks, ceig, tmpa, lam);
  ZQ_LAUNCH_CHECK();
  k_cl_writeback<<<grid_for((int64_t)2 * n * m), 256, 0, st>>>(X, ldd, n, dmem, m, tmpa);
  ZQ_LAUNCH_CHECK();
  // S, G: columns, then rows (2 n m double2 of scratch per pair)
  const int gc = ceil_div(n * kmax, 256) > 64 ? 64 : ceil_div(n * kmax, 256);
  const int gw = grid_for((int64_t)n * m) > 4096 ? 4096 : grid_for((int64_t)n * m);
  k_cl_congr_cols<<<dim3(gc, ncl, 2), 256, 0, st>>>(S1, S2, G1, G2, n, n, dmem, dcs, dco, ncl, blocks, m, tmpa, tmpb);
  ZQ_LAUNCH_CHECK();
  k_cl_cols_writeback<<<dim3(gw, 1, 2), 256, 0, st>>>(S1, S2, G1, G2, n, n, dmem, m, tmpa, tmpb);
  ZQ_LAUNCH_CHECK();
  k_cl_congr_rows<<<dim3(gc, ncl, 2), 256, 0, st>>>(S1, S2, G1, G2, n, n, dmem, dcs, dco, ncl, blocks, dpos, m, tmpa,
                                                    tmpb);
  ZQ_LAUNCH_CHECK();
  k_cl_rows_writeback<<<dim3(gw, 1, 2), 256, 0, st>>>(S1, S2, G1, G2, n, n, dmem, m, tmpa, tmpb);
  ZQ_LAUNCH_CHECK();
  ZQ_CUDA(cudaFreeAsync(mem, st));
  return ZQ_OK;
}

int refined_solve(RefineArgs& ra) {
  const int n = ra.n;
  const int n2 = 2 * n;
  cudaStream_t st = ra.st;
  const size_t nn = (size_t)n * n;
  char* p = reinterpret_cast<char*>(ra.ws);
  auto take = [&](size_t bytes) { char* q = p; p += (bytes + 255) & ~(size_t)255; return q; };
  double2* H0 = reinterpret_cast<double2*>(take(sizeof(double2) * 2 * nn));
  float2* Mf = reinterpret_cast<float2*>(take(sizeof(float2) * 4 * nn));
  double2* P1 = reinterpret_cast<double2*>(take(sizeof(double2) * 2 * nn));
  double2* P2 = reinterpret_cast<double2*>(take(sizeof(double2) * 2 * nn));
  double2* HX = reinterpret_cast<double2*>(take(sizeof(double2) * 2 * nn));
  double2* G1 = reinterpret_cast<double2*>(take(sizeof(double2) * nn));
  double2* G2 = reinterpret_cast<double2*>(take(sizeof(double2) * nn));
  double2* S1 = reinterpret_cast<double2*>(take(sizeof(double2) * nn));
  double2* S2 = reinterpret_cast<double2*>(take(sizeof(double2) * nn));
  double2* Et = reinterpret_cast<double2*>(take(sizeof(double2) * nn));
  double2* Eb = reinterpret_cast<double2*>(take(sizeof(double2) * nn));
  void* tri_ws = take(tridiag_workspace_bytes<float>(n, NBMAX));
  void* fq_ws = take(form_q_workspace_bytes(n, ra.nbq));
  double* sm = reinterpret_cast<double*>(take(sizeof(double) * (46 * (size_t)n + 3 * 8192 + 8192 + 2048 + 64)));
  int* rank = reinterpret_cast<int*>(take(sizeof(int) * (size_t)n));
  int* tc_err = reinterpret_cast<int*>(take(256));
  double* d = sm; sm += n;
  double* e = sm; sm += 4 * (size_t)n;
  double* tau = sm; sm += n;
  double* offd = sm; sm += n;
  double* phi = sm; sm += 4 * (size_t)n;
  double* lam = sm; sm += n;
  double* lam2 = sm; sm += n;
  double* lamr = sm; sm += n;   // the diagonal of the current step's residual R = HX - X diag(lamr)
  double* part = sm; sm += 3 * 8192;
  double* emax = sm; sm += 2048;
  int* pair_count = reinterpret_cast<int*>(sm); sm += 8;
  int2* pairs = reinterpret_cast<int2*>(sm);
  const int pair_cap = 32 * n;  // 13 n doubles above, 32 n int2 here
  const int64_t ldd = ra.ldd;
  double2* X = ra.dD;  // (U; V) lives in the output's left half

  // ZQ_REFINE_TRACE: per-step history and the stage timeline (events) on stderr
  const bool trace = getenv("ZQ_REFINE_TRACE") != nullptr;
  cudaEvent_t tev[9];
  if (trace)
    for (auto& e : tev) cudaEventCreate(&e);
  auto mark = [&](int i, cudaStream_t s2) { if (trace) cudaEventRecord(tev[i], s2); };

  // A. FP32 eigendecomposition
  mark(0, st);
  ZQ_CUDA(cudaMemcpy2DAsync(H0, sizeof(double2) * n2, ra.dD, sizeof(double2) * ldd, sizeof(double2) * n2, n,
                            cudaMemcpyDeviceToDevice, st));
  k_c128_to_c64<<<grid_for((int64_t)n2 * n), 256, 0, st>>>(H0, n2, Mf, n2, n2, n);
  ZQ_LAUNCH_CHECK();
  ZQ_CUDA(cudaMemsetAsync(tc_err, 0, sizeof(int), st));
  TridiagView<float> vf = tridiag_bind<float>(tri_ws, Mf, n, n2, NBMAX, d, e, tau);
  vf.tc_err = tc_err;  // tensor-core products where fp32_products_on_tensor_cores allows them
  vf.coop = ra.coop;
  if (int rc = tridiagonalize<float>(vf, ra.nb, st)) return rc;
  if (int rc = phase_reduce(e, n, offd, phi, st)) return rc;
  mark(1, st);
  float2* XfQ = Mf + (int64_t)n * n2;  // right half of Mf
  // Q Phi (FP32) on the second stream while the divide and conquer runs
  ZQ_CUDA(cudaEventRecord(ra.ev_fork, st));
  ZQ_CUDA(cudaStreamWaitEvent(ra.st2, ra.ev_fork, 0));
  if (int rc = form_q<float>(Mf, n2, n, phi, XfQ, n2, ra.nbq, fq_ws, ra.st2, tc_err)) return rc;
  mark(2, ra.st2);
  ZQ_CUDA(cudaEventRecord(ra.ev_join, ra.st2));
  float* Zf = nullptr;  // FP32 divide and conquer: Z in the plan's workspace
  ra.dc->tc_err = tc_err;
  const int dc_rc = ra.dc->run_single(d, offd, lam, Zf, st);
  ra.dc->tc_err = nullptr;
  if (dc_rc) return dc_rc;
  mark(3, st);
  ZQ_CUDA(cudaStreamWaitEvent(st, ra.ev_join, 0));
  if (int rc = apply_z<float>(XfQ, n2, Zf, n, n, Mf, n2, ra.fdesc, st, tc_err)) return rc;
  k_c64_to_c128<<<grid_for((int64_t)n2 * n), 256, 0, st>>>(Mf, n2, X, ldd, n2, n);
  ZQ_LAUNCH_CHECK();
  {
    // a tensor-core pipeline wait that ran out leaves X0 unusable: report it
    int herr = 0;
    ZQ_CUDA(cudaMemcpyAsync(&herr, tc_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    ZQ_CUDA(cudaStreamSynchronize(st));
    if (herr) {
      set_error_message("k_tc32: a pipeline wait ran out of time (kernel stopped)");
      return ZQ_ERR_TIMEOUT;
    }
  }
  mark(4, st);

  // B. refinement
  prof_begin(PC_REFINE, st);
  const double2 one = make_double2(1.0, 0.0), zero = make_double2(0.0, 0.0);
  const int nparts = 1024;
  ra.iters = 0;
  ra.last_emax = 1.0;
  const int ne = 1024;
  std::vector<double> hemax(2 * ne);
  for (int it = 0; it < ra.max_iter; ++it) {
    // the first correction only has to reach ~1e-8 (the next step squares the
    // error): ZQ_REFINE_SLICES0 slices (default 5 = 35 bits); later steps use 8
    // (56 bits: 7 slices would save a fifth of the products but cost ~25x in
    // eigenvalue accuracy)
    const int sl = (it == 0) ? ra.slices0 : 8;
    // the correction X E is small (|E| <= 1e-4 in the first step, ~1e-8 after):
    // 3 slices (21 bits) first, 4 (28 bits) after keep its error below what
    // the next step removes / below 1e-14
    const int sl_upd = (it == 0) ? 3 : 4;
    // the residual products: |R| <= ~1e-4 ||H|| in the first step, ~1e-8 after,
    // so 4 slices (28 bits) leave their error below what each step needs
    const int ss_slices = ra.slices_res;
    double2* U = X;
    double2* V = X + n;
    ZgemmArgs g{};
    // Consecutive products share their A operand, so the second one reuses its
    // slices: (P1, P2) with [A;B], (G1, S1) with X^H, (G2, S2) with [U^T | V^T].
    // P1 = [A;B] U, P2 = [A;B] conj(V)
    g = ZgemmArgs{};
    g.m = n2; g.n = n; g.k1 = n; g.A1 = H0; g.lda1 = n2; g.B1 = U; g.ldb1 = ldd;
    g.alpha = one; g.beta = zero; g.C = P1; g.ldc = n2;
    if (int rc = zgemm_acc(ra.mode, OP_N, OP_N, OP_N, OP_N, g, ra.ows, ra.ows_bytes, st, sl, 0, 0)) return rc;
    g.B1 = V; g.C = P2;
    if (int rc = zgemm_acc(ra.mode, OP_N, OP_R, OP_N, OP_N, g, ra.ows, ra.ows_bytes, st, sl, 0, 1)) return rc;
    // R = HX - X diag(lamr), lamr the current eigenvalue estimates (the
    // divide-and-conquer values, then the previous step's Rayleigh quotients).
    // S = X^H H X = X^H R + G diag(lamr) for any diagonal lamr; with R small
    // (~ the eigenvector error times ||H||) the products with R need only
    // ss_slices, while G keeps sl.
    ZQ_CUDA(cudaMemcpyAsync(lamr, lam, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    k_hx_combine<<<grid_for((int64_t)nn), 256, 0, st>>>(P1, P2, n2, n, HX, n2, X, ldd, lamr);
    ZQ_LAUNCH_CHECK();
    // G1 = X^H X ; S1 = X^H R + G1 Lambda
    g = ZgemmArgs{};
    g.m = n; g.n = n; g.k1 = n2; g.A1 = X; g.lda1 = ldd; g.B1 = X; g.ldb1 = ldd;
    g.alpha = one; g.beta = zero; g.C = G1; g.ldc = n;
    if (int rc = zgemm_acc(ra.mode, OP_C, OP_N, OP_N, OP_N, g, ra.ows, ra.ows_bytes, st, sl, 1, 0)) return rc;
    g.B1 = HX; g.ldb1 = n2; g.C = S1;
    if (int rc = zgemm_acc(ra.mode, OP_C, OP_N, OP_N, OP_N, g, ra.ows, ra.ows_bytes, st, ss_slices, 2, 1)) return rc;
    // G2 = U^T V - V^T U ; S2 = U^T R_bot - V^T R_top + G2 Lambda
    g = ZgemmArgs{};
    g.m = n; g.n = n; g.k1 = n; g.k2 = n;
    g.A1 = U; g.lda1 = ldd; g.B1 = V; g.ldb1 = ldd; g.A2 = V; g.lda2 = ldd; g.B2 = U; g.ldb2 = ldd; g.s2 = -1.0;
    g.alpha = one; g.beta = zero; g.C = G2; g.ldc = n;
    if (int rc = zgemm_acc(ra.mode, OP_T, OP_N, OP_T, OP_N, g, ra.ows, ra.ows_bytes, st, sl, -1, 0)) return rc;
    g.B1 = HX + n; g.ldb1 = n2; g.B2 = HX; g.ldb2 = n2; g.C = S2;
    if (int rc = zgemm_acc(ra.mode, OP_T, OP_N, OP_T, OP_N, g, ra.ows, ra.ows_bytes, st, ss_slices, -2, 1)) return rc;
    k_add_glam<<<grid_for((int64_t)nn), 256, 0, st>>>(S1, G1, n, lamr);
    ZQ_LAUNCH_CHECK();
    k_add_glam<<<grid_for((int64_t)nn), 256, 0, st>>>(S2, G2, n, lamr);
    ZQ_LAUNCH_CHECK();
    if (int rc = structured_fill(S1, n, n, 1, st)) return rc;
    if (int rc = structured_fill(S2, n, n, -1, st)) return rc;
    // Rayleigh quotients, coupling norms, E; pairs that fail the first-order
    // test are grouped into clusters, rotated (Rayleigh-Ritz on the current
    // basis, S and G carried along), and E is rebuilt in the rotated basis
    double em = 0.0, cm = 0.0;
    int hcount = 0, clusters = 0;
    for (int pass = 0; pass < 2; ++pass) {
      k_oa_lambda<<<ceil_div(n, 256), 256, 0, st>>>(S1, G1, n, n, lam);
      ZQ_LAUNCH_CHECK();
      k_oa_norms<<<nparts, 256, 0, st>>>(S1, S2, G1, G2, n, n, lam, part);
      ZQ_LAUNCH_CHECK();
      ZQ_CUDA(cudaMemsetAsync(pair_count, 0, sizeof(int), st));
      k_oa_build_e<<<ne, 256, 0, st>>>(S1, S2, G1, G2, n, n, lam, part, nparts, Et, Eb, n, emax, pair_count, pairs,
                                       pair_cap, it == 0 ? ra.pair_eps : ra.pair_eps_late);
      ZQ_LAUNCH_CHECK();
      ZQ_CUDA(cudaMemcpyAsync(hemax.data(), emax, sizeof(double) * 2 * ne, cudaMemcpyDeviceToHost, st));
      ZQ_CUDA(cudaMemcpyAsync(&hcount, pair_count, sizeof(int), cudaMemcpyDeviceToHost, st));
      ZQ_CUDA(cudaStreamSynchronize(st));
      em = 0.0; cm = 0.0;
      for (int q = 0; q < ne; ++q) { em = hemax[q] > em ? hemax[q] : em; cm = hemax[ne + q] > cm ? hemax[ne + q] : cm; }
      if (pass == 1 || !(cm > ra.cluster_tol)) break;
      if (hcount > pair_cap) { ra.clusters = -1; break; }
      if (int rc = resolve_clusters(ra, X, ldd, S1, S2, G1, G2, lam, pairs, hcount, P1, P2)) return rc;
      if (ra.clusters < 0) break;
      clusters = ra.clusters;
    }
    if (ra.clusters < 0) break;
    ra.last_emax = em;
    ra.last_cluster = cm;
    // X += X E_top + J conj(X) E_bot with sl_upd slices; FP64 accumulation
    //   P1_top = U E_top - conj(V) E_bot,  P1_bot = V E_top + conj(U) E_bot
    g = ZgemmArgs{};
    g.m = n; g.n = n; g.k1 = n; g.k2 = n;
    g.A1 = U; g.lda1 = ldd; g.B1 = Et; g.ldb1 = n; g.A2 = V; g.lda2 = ldd; g.B2 = Eb; g.ldb2 = n; g.s2 = -1.0;
    g.alpha = one; g.beta = zero; g.C = P1; g.ldc = n2;
    if (int rc = zgemm_acc(ra.mode, OP_N, OP_N, OP_R, OP_N, g, ra.ows, ra.ows_bytes, st, sl_upd, 0, 0)) return rc;
    g.A1 = V; g.A2 = U; g.s2 = 1.0; g.C = P1 + n;
    if (int rc = zgemm_acc(ra.mode, OP_N, OP_N, OP_R, OP_N, g, ra.ows, ra.ows_bytes, st, sl_upd, 0, 0)) return rc;
    k_add_c128<<<grid_for((int64_t)n2 * n), 256, 0, st>>>(P1, n2, X, ldd, n2, n);
    ZQ_LAUNCH_CHECK();
    ra.iters = it + 1;
    if (trace) {
      mark(5 + (it < 3 ? it : 2), st);
      fprintf(stderr, "zq refine n=%d step %d slices %d emax %.3e coupling %.3e pairs %d clusters %d\n", n, it, sl,
              em, cm, hcount, clusters);
    }
    // A step that rotated clusters is not the last: the E it applies was built
    // on a basis rotated with the previous step's accuracy (seen on a clustered
    // n = 64 input: orthonormality 1.6e-12 when stopping there, 9e-16 after one
    // more step), so the final update is always a plain first-order one.
    if (em <= ra.tol && (ra.mode == 0 || sl == 8) && clusters == 0) break;
  }
  prof_end(PC_REFINE, st);
  if (trace) {
    mark(8, st);
    cudaEventSynchronize(tev[8]);
    float t[9];
    for (int i = 1; i < 9; ++i) t[i] = -1.f;
    const int last = 5 + (ra.iters - 1 < 2 ? ra.iters - 1 : 2);
    for (int i : {1, 2, 3, 4, 5, 6, 7, 8})
      if (i <= 4 || i <= last || i == 8) cudaEventElapsedTime(&t[i], tev[0], tev[i]);
    fprintf(stderr, "zq refine timeline ms from start: tridiag+phase %.2f | form_q done (2nd stream) %.2f | "
            "d&c done %.2f | apply_z done %.2f | step0 %.2f step1 %.2f step2 %.2f | end %.2f\n",
            t[1], t[2], t[3], t[4], t[5], t[6], t[7], t[8]);
    for (auto& e : tev) cudaEventDestroy(e);
  }
  // ascending order
  k_rank<<<ceil_div(n, 128), 128, 0, st>>>(lam, n, rank);
  ZQ_LAUNCH_CHECK();
  k_permute_cols<<<grid_for((int64_t)n2 * n), 256, 0, st>>>(X, ldd, n2, n, rank, P1, n2, lam, lam2);
  ZQ_LAUNCH_CHECK();
  ZQ_CUDA(cudaMemcpy2DAsync(X, sizeof(double2) * ldd, P1, sizeof(double2) * n2, sizeof(double2) * n2, n,
                            cudaMemcpyDeviceToDevice, st));
  ZQ_CUDA(cudaMemcpyAsync(ra.deig, lam2, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
  if (int rc = symmetry_fill(ra.dD, ldd, n, st)) return rc;
  return ZQ_OK;
}

}  // namespace zq
