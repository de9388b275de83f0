// Stage (a)+(b): blocked, structure-preserving tridiagonalisation of a
// quaternion-Hermitian matrix on the GPU.
//
// Reference: ts::impl::panel_update (blocked.cc:45-546) and
// ts::impl::unblocked_update (unblocked.cc:44-131), driven by the panel loop at
// zquatev.cc:68-72. The reference zeroes each column with a Householder on the
// B part (blocked.cc:167-178), a symplectic Givens (blocked.cc:234-337) and a
// Householder on the A part (blocked.cc:339-413), keeping a Kressner compact-WY
// form with 3x3-block T, R, S matrices.
//
// Here each column k is zeroed by ONE quaternion Householder reflector
//   P_k = I - W_k W_k^H,   W_k = [w, J conj(w)]  (2L x 2, W^H W = 2 I),
// with w = (wa, wb) built from the quaternion column x = (A[k+1:,k], B[k+1:,k]):
//   w = f * (x + s * x_1 e_1),  s = |x| / |x_1|,  f = 1 / sqrt(|x| (|x| + |x_1|)),
// which maps x to the quaternion -s * x_1 e_1 (the subdiagonal entry e_k; its
// quaternion phase is removed later by a diagonal quaternion similarity, see
// zq_backtransform.cu). This is the same family of symplectic unitary
// transforms as the reference (Householder + Givens + Householder is one
// quaternion reflector followed by a quaternion phase), with one reflector
// and one quaternion matrix-vector product per column instead of two.
//
// Blocking follows the LAPACK zlatrd/zhetrd scheme lifted to quaternions: for
// a panel of nb columns, keep W (in the reduced columns of M) and the aux
// vectors Y with  H_current = H_panelstart - sum_i (W_i Y_i^H + Y_i W_i^H),
//   y = g - (c/2) w,  g = H_current w,  c = w^H g (real),
// and after the panel apply the structured rank-4nb update (her2k-like) to the
// lower triangles of the trailing A (Hermitian) and B (antisymmetric):
//   A -= Wa Ya^H + conj(Wb) conj(Yb)^H + Ya Wa^H + conj(Yb) conj(Wb)^H
//   B -= Wb Ya^H - conj(Wa) conj(Yb)^H + Yb Wa^H - conj(Ya) conj(Wb)^H
//
// Per column the launch sequence is
//   colupd  (finish y_{k-1}; apply the panel's deferred updates to column k;
//            norm partials)
//   reflect (build w in place of x; dot-product partials vs previous W, Y)
//   hemv    (quaternion Hermitian mat-vec of the panel-start trailing matrix,
//            lower triangles of A and B only, per-tile deterministic partials)
//   hreduce (sum tile partials and the dot partials, subtract the
//            deferred-update corrections -> g; partials of c)
// The kernels are launched with programmatic dependent launch (each starts
// with pdl_wait), so a kernel's launch overlaps the tail of the previous one.
// All arithmetic is FP64 (template R = double) for the plain path; the same
// kernels instantiate with R = float for the mixed-precision path, where norms
// and reflector scalars are still formed in double.
#include "zq_common.cuh"
#include "zq_kernels.h"

namespace zq {

constexpr int RB = 32;        // rows per CTA for the row-parallel kernels
constexpr int NG = 8;         // reflector groups per CTA in the row kernels (NT / RB)
constexpr int TB = 64;        // tile edge of the trailing update
constexpr int NT = 256;       // threads per CTA

// ----------------------------------------------------------------------------
// colupd: rows [j, n) of column j
// ----------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(NT) k_colupd(TridiagView<R> v, int p, int j, int k, int ncp, int do_update) {
  pdl_wait();  // launched with launch_pdl: the previous kernel's results first
  using Z = cplx<R>;
  const int n = v.n;
  const int64_t ld = v.ld;
  Z* A = v.M;
  Z* B = v.M + n;
  const int r0 = j + blockIdx.x * RB;
  const int tid = threadIdx.x;
  const int row = tid & (RB - 1);
  const int grp = tid >> 5;
  const int r = r0 + row;
  __shared__ Z s_sc[4 * 64];        // per i: ya_i[j], yb_i[j], wa_i[j], wb_i[j]
  __shared__ Z s_red[NG][RB][2];
  __shared__ double s_red_d[2][NT / 32];
  __shared__ double s_c;

  // c_{k-1} = sum of partials (deterministic order)
  if (k > 0 && tid < 32) {
    double c = 0;
    for (int i = tid; i < ncp; i += 32) c += v.cpart[i];
    c = warp_sum(c);
    if (tid == 0) s_c = c;
  }
  __syncthreads();
  const R half_c = (k > 0) ? (R)(0.5 * s_c) : (R)0;

  // finish y_{k-1} = g - (c/2) w_{k-1} on this CTA's rows (rows >= j)
  if (k > 0 && grp == 0 && r < n) {
    const Z wa = A[r + (int64_t)(j - 1) * ld], wb = B[r + (int64_t)(j - 1) * ld];
    v.Ya[r + (int64_t)(k - 1) * v.ldy] = csub(v.ga[r], cscale(wa, half_c));
    v.Yb[r + (int64_t)(k - 1) * v.ldy] = csub(v.gb[r], cscale(wb, half_c));
  }
  if (!do_update) return;

  // scalars at row j for every previous reflector of the panel
  for (int i = tid; i < k; i += NT) {
    Z ya, yb;
    const Z wa = A[j + (int64_t)(p + i) * ld], wb = B[j + (int64_t)(p + i) * ld];
    if (i == k - 1) {
      ya = csub(v.ga[j], cscale(wa, half_c));
      yb = csub(v.gb[j], cscale(wb, half_c));
    } else {
      ya = v.Ya[j + (int64_t)i * v.ldy];
      yb = v.Yb[j + (int64_t)i * v.ldy];
    }
    s_sc[4 * i + 0] = ya; s_sc[4 * i + 1] = yb; s_sc[4 * i + 2] = wa; s_sc[4 * i + 3] = wb;
  }
  __syncthreads();

  Z da = czero<Z>(), db = czero<Z>();
  if (r < n) {
    for (int i = grp; i < k; i += NG) {
      const Z sya = s_sc[4 * i + 0], syb = s_sc[4 * i + 1], swa = s_sc[4 * i + 2], swb = s_sc[4 * i + 3];
      const Z wa = A[r + (int64_t)(p + i) * ld], wb = B[r + (int64_t)(p + i) * ld];
      Z ya, yb;
      if (i == k - 1) {
        ya = csub(v.ga[r], cscale(wa, half_c));
        yb = csub(v.gb[r], cscale(wb, half_c));
      } else {
        ya = v.Ya[r + (int64_t)i * v.ldy];
        yb = v.Yb[r + (int64_t)i * v.ldy];
      }
      // A part: wa conj(ya_j) + conj(wb) yb_j + ya conj(wa_j) + conj(yb) wb_j
      cfmacb(da, wa, sya); cfmac(da, wb, syb); cfmacb(da, ya, swa); cfmac(da, yb, swb);
      // B part: wb conj(ya_j) - conj(wa) yb_j + yb conj(wa_j) - conj(ya) wb_j
      cfmacb(db, wb, sya); cfmac(db, cneg(wa), syb); cfmacb(db, yb, swa); cfmac(db, cneg(ya), swb);
    }
  }
  s_red[grp][row][0] = da;
  s_red[grp][row][1] = db;
  __syncthreads();

  double sc = 0.0;  // local max-abs of x (rows >= j+1)
  Z xa = czero<Z>(), xb = czero<Z>();
  if (grp == 0 && r < n) {
    Z ta = s_red[0][row][0], tb = s_red[0][row][1];
    for (int g2 = 1; g2 < NG; ++g2) { ta = cadd(ta, s_red[g2][row][0]); tb = cadd(tb, s_red[g2][row][1]); }
    xa = csub(A[r + (int64_t)j * ld], ta);
    xb = csub(B[r + (int64_t)j * ld], tb);
    A[r + (int64_t)j * ld] = xa;
    B[r + (int64_t)j * ld] = xb;
    if (r == j) v.d[j] = (double)xa.x;
    if (r == j + 1) {
      v.scal[0] = (double)xa.x; v.scal[1] = (double)xa.y;
      v.scal[2] = (double)xb.x; v.scal[3] = (double)xb.y;
    }
    if (r > j) {
      sc = fmax(fmax(fabs((double)xa.x), fabs((double)xa.y)), fmax(fabs((double)xb.x), fabs((double)xb.y)));
    }
  }
  // scaled sum of squares (LAPACK lassq style, combined across CTAs in reflect)
  const double bmax = block_max(sc, s_red_d[0]);
  double ss = 0.0;
  if (grp == 0 && r < n && r > j && bmax > 0.0) {
    const double inv = 1.0 / bmax;
    const double a0 = xa.x * inv, a1 = xa.y * inv, b0 = xb.x * inv, b1 = xb.y * inv;
    ss = a0 * a0 + a1 * a1 + b0 * b0 + b1 * b1;
  }
  const double bss = block_sum(ss, s_red_d[1]);
  if (tid == 0) {
    v.npart[2 * blockIdx.x + 0] = bmax;
    v.npart[2 * blockIdx.x + 1] = bss;
  }
}

// ----------------------------------------------------------------------------
// reflect: rows [j+1, n); builds w in place of x, writes e_j, dot partials.
// ----------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(NT) k_reflect(TridiagView<R> v, int p, int j, int k, int nnp) {
  pdl_wait();  // launched with launch_pdl: the previous kernel's results first
  using Z = cplx<R>;
  const int n = v.n;
  const int64_t ld = v.ld;
  Z* A = v.M;
  Z* B = v.M + n;
  const int L = n - 1 - j;
  const int tid = threadIdx.x;
  __shared__ double s_sc[5];  // f, first element of w (a.re, a.im, b.re, b.im)
  double nu = 0.0;
  if (tid < 32) {
    // combine norm partials: nu = scale * sqrt(ssq)
    double scale = 0.0;
    for (int i = tid; i < nnp; i += 32) scale = fmax(scale, v.npart[2 * i]);
    scale = warp_max(scale);
    double ssq = 0.0;
    if (scale > 0.0)
      for (int i = tid; i < nnp; i += 32) {
        const double si = v.npart[2 * i];
        if (si > 0.0) { const double q = si / scale; ssq += v.npart[2 * i + 1] * q * q; }
      }
    ssq = warp_sum(ssq);
    nu = scale * sqrt(ssq);
  }
  if (tid == 0) {
    const double qa0 = v.scal[0], qa1 = v.scal[1], qb0 = v.scal[2], qb1 = v.scal[3];
    const double q1 = sqrt(qa0 * qa0 + qa1 * qa1 + qb0 * qb0 + qb1 * qb1);
    double f = 0.0, m[4] = {0.0, 0.0, 0.0, 0.0};
    double ee[4] = {qa0, qa1, qb0, qb1};   // L == 1: the entry itself is e_j
    if (L >= 2) {
      if (nu > 0.0) {
        if (q1 > 0.0) {
          const double s = nu / q1;
          f = 1.0 / (sqrt(nu) * sqrt(nu + q1));
          m[0] = qa0 * (1.0 + s); m[1] = qa1 * (1.0 + s); m[2] = qb0 * (1.0 + s); m[3] = qb1 * (1.0 + s);
          ee[0] = -s * qa0; ee[1] = -s * qa1; ee[2] = -s * qb0; ee[3] = -s * qb1;
        } else {
          f = 1.0 / nu;
          m[0] = nu;
          ee[0] = -nu; ee[1] = 0.0; ee[2] = 0.0; ee[3] = 0.0;
        }
      } else {
        ee[0] = ee[1] = ee[2] = ee[3] = 0.0;  // x == 0: nothing to reduce
      }
    }
    s_sc[0] = f;
    for (int q = 0; q < 4; ++q) s_sc[1 + q] = m[q] * f;
    if (blockIdx.x == 0) {
      for (int q = 0; q < 4; ++q) v.e[4 * j + q] = ee[q];
      v.tau[j] = (f > 0.0) ? 1.0 : 0.0;
    }
  }
  __syncthreads();
  const double f = s_sc[0];
  const int r0 = j + 1 + blockIdx.x * RB;
  const int row = tid & (RB - 1);
  const int grp = tid >> 5;
  const int r = r0 + row;
  __shared__ Z s_wa[RB], s_wb[RB];
  if (grp == 0) {
    Z wa = czero<Z>(), wb = czero<Z>();
    if (r < n) {
      if (f > 0.0) {
        if (r == j + 1) {
          wa = mk((R)s_sc[1], (R)s_sc[2]);
          wb = mk((R)s_sc[3], (R)s_sc[4]);
        } else {
          wa = cscale(A[r + (int64_t)j * ld], (R)f);
          wb = cscale(B[r + (int64_t)j * ld], (R)f);
        }
      }
      A[r + (int64_t)j * ld] = wa;
      B[r + (int64_t)j * ld] = wb;
    }
    s_wa[row] = wa; s_wb[row] = wb;
  }
  // dot partials vs previous reflectors / aux vectors of the panel
  if (k == 0 || L < 2) return;
  __syncthreads();
  const int warp = tid >> 5, lane = tid & 31;
  const int gr = r0 + lane;
  const Z xa = s_wa[lane], xb = s_wb[lane];
  for (int i = warp; i < k; i += NT / 32) {
    Z d1 = czero<Z>(), d2 = czero<Z>(), d3 = czero<Z>(), d4 = czero<Z>();
    if (gr < n) {
      const Z ya = v.Ya[gr + (int64_t)i * v.ldy], yb = v.Yb[gr + (int64_t)i * v.ldy];
      const Z qa = A[gr + (int64_t)(p + i) * ld], qb = B[gr + (int64_t)(p + i) * ld];
      // <y,w> = ya^H xa + yb^H xb ; [y,w] = ya^T xb - yb^T xa
      cfmac(d1, ya, xa); cfmac(d1, yb, xb);
      cfma(d2, ya, xb); cfma(d2, cneg(yb), xa);
      cfmac(d3, qa, xa); cfmac(d3, qb, xb);
      cfma(d4, qa, xb); cfma(d4, cneg(qb), xa);
    }
    d1.x = warp_sum(d1.x); d1.y = warp_sum(d1.y);
    d2.x = warp_sum(d2.x); d2.y = warp_sum(d2.y);
    d3.x = warp_sum(d3.x); d3.y = warp_sum(d3.y);
    d4.x = warp_sum(d4.x); d4.y = warp_sum(d4.y);
    if (lane == 0) {
      Z* o = v.dpart + ((int64_t)blockIdx.x * v.nbmax + i) * 4;
      o[0] = d1; o[1] = d2; o[2] = d3; o[3] = d4;
    }
  }
}

// ----------------------------------------------------------------------------
// hemv: quaternion Hermitian mat-vec of the panel-start trailing matrix.
//   Region rows/cols [r0, n); lower-triangle 32x32 tiles, one CTA per tile.
//   The A and B tiles are staged in shared memory (padded, conflict-free for
//   both row and column sweeps) and four warps each own one product:
//     warp 0: rows,  A x and A z          warp 2: columns, A^H x and A^H z
//     warp 1: rows,  B x and B z          warp 3: columns, -B^T x and -B^T z
//   (x = wa, z = conj(wb)), so every lower-triangle element is read once from
//   HBM and used for its row and its (conjugate-)transposed column without any
//   cross-thread reduction: all FP64 work is DFMA. Per T-row block R and source
//   block S the CTA stores the partial sums of v0 = A x, v1 = A z, v2 = B x,
//   v3 = B z.
// ----------------------------------------------------------------------------
constexpr int HT = 32;        // hemv tile edge
constexpr int HLD = HT + 1;   // padded shared leading dimension
template <typename R>
__global__ void __launch_bounds__(128) k_hemv(TridiagView<R> v, int j) {
  pdl_wait();  // launched with launch_pdl: the previous kernel's results first
  using Z = cplx<R>;
  const int n = v.n;
  const int64_t ld = v.ld;
  const Z* A = v.M;
  const Z* B = v.M + n;
  const int r0 = j + 1;
  const int t = blockIdx.x;
  int I, J;
  tri_tile(t, I, J);
  const bool diag = (I == J);
  const int tid = threadIdx.x;
  const int rbase = r0 + I * HT, cbase = r0 + J * HT;
  __shared__ Z sA[HT * HLD], sB[HT * HLD];
  __shared__ Z sx[2][HT], sz[2][HT];   // [0]: rows of block I, [1]: rows of block J
  __shared__ Z sout[HT][4];
  for (int e = tid; e < HT * HT; e += 128) {
    const int r = e & (HT - 1), c = e >> 5;
    const int gr = rbase + r, gc = cbase + c;
    Z a = czero<Z>(), b = czero<Z>();
    if (gr < n && gc < n && (!diag || r >= c)) {
      a = A[gr + (int64_t)gc * ld];
      b = B[gr + (int64_t)gc * ld];
      if (diag && r == c) { a.y = 0; b = czero<Z>(); }
    }
    sA[r + c * HLD] = a;
    sB[r + c * HLD] = b;
  }
  if (tid < 2 * HT) {
    const int s = tid >> 5, q = tid & (HT - 1);
    const int g = (s == 0 ? rbase : cbase) + q;
    Z x = czero<Z>(), z = czero<Z>();
    if (g < n) { x = A[g + (int64_t)j * ld]; z = cconj(B[g + (int64_t)j * ld]); }
    sx[s][q] = x;
    sz[s][q] = z;
  }
  __syncthreads();
  const int role = tid >> 5, q = tid & (HT - 1);
  // two accumulators per product (even / odd k) for independent FMA chains
  Z p0 = czero<Z>(), p1 = czero<Z>(), p2 = czero<Z>(), p3 = czero<Z>();
  if (role < 2) {
    const Z* S = role == 0 ? sA : sB;
#pragma unroll 8
    for (int c = 0; c < HT; c += 2) {
      const Z m0 = S[q + c * HLD], m1 = S[q + (c + 1) * HLD];
      cfma(p0, m0, sx[1][c]); cfma(p1, m0, sz[1][c]);
      cfma(p2, m1, sx[1][c + 1]); cfma(p3, m1, sz[1][c + 1]);
    }
  } else if (role == 2) {
    for (int r = diag ? q + 1 : 0; r < HT; ++r) {
      const Z m = sA[r + q * HLD];
      if (r & 1) { cfmac(p2, m, sx[0][r]); cfmac(p3, m, sz[0][r]); }
      else { cfmac(p0, m, sx[0][r]); cfmac(p1, m, sz[0][r]); }
    }
  } else {
    for (int r = diag ? q + 1 : 0; r < HT; ++r) {
      const Z m = sB[r + q * HLD];
      if (r & 1) { cfma(p2, m, sx[0][r]); cfma(p3, m, sz[0][r]); }
      else { cfma(p0, m, sx[0][r]); cfma(p1, m, sz[0][r]); }
    }
    p0 = cneg(p0); p1 = cneg(p1); p2 = cneg(p2); p3 = cneg(p3);
  }
  const Z u0 = cadd(p0, p2), u1 = cadd(p1, p3);   // this warp's two products
  const int nbm = v.hblk;
  if (role >= 2) {
    if (diag) { sout[q][2 * (role - 2)] = u0; sout[q][2 * (role - 2) + 1] = u1; }
    else {
      Z* o = v.hpart + (((int64_t)J * nbm + I) * HT + q) * 4 + 2 * (role - 2);
      o[0] = u0; o[1] = u1;
    }
  }
  if (diag) __syncthreads();
  if (role < 2) {
    Z a0 = u0, a1 = u1;
    if (diag) { a0 = cadd(a0, sout[q][2 * role]); a1 = cadd(a1, sout[q][2 * role + 1]); }
    Z* o = v.hpart + (((int64_t)I * nbm + J) * HT + q) * 4 + 2 * role;
    o[0] = a0; o[1] = a1;
  }
}

// ----------------------------------------------------------------------------
// hreduce: g = H_panelstart w - corrections, for rows [j+1, n); c partials.
//   T is the hemv tile edge used for this column; nblk its number of blocks.
//   HRB rows per CTA; four threads per (row, product) sum the hemv tile
//   partials (fixed split and combine order: deterministic). Every CTA also
//   sums the reflect kernel's dot partials (ndp of them) itself, in the same
//   fixed order, so no separate reduction launch sits between reflect and hemv.
// ----------------------------------------------------------------------------
constexpr int HRB = 16;          // rows per CTA
constexpr int HNG = NT / HRB;    // reflector groups for the corrections
template <typename R>
__global__ void __launch_bounds__(NT) k_hreduce(TridiagView<R> v, int p, int j, int k, int T, int nblk, int zero_mode,
                                                int ndp) {
  pdl_wait();  // launched with launch_pdl: the previous kernel's results first
  using Z = cplx<R>;
  const int n = v.n;
  const int64_t ld = v.ld;
  const Z* A = v.M;
  const Z* B = v.M + n;
  const int r0 = j + 1;
  const int tid = threadIdx.x;
  const int row = tid & (HRB - 1), grp = tid >> 4;
  const int lrow = blockIdx.x * HRB + row;   // row index inside the region
  const int r = r0 + lrow;
  __shared__ Z s_v[HRB][4];
  __shared__ Z s_dots[4 * 64];
  __shared__ Z s_part[4][4 * HRB];
  __shared__ Z s_dsub[NT];
  __shared__ Z s_red[HNG][HRB][2];
  __shared__ double s_redd[NT / 32];
  if (!zero_mode) {
    // (1) tile partials: output o = (row, product), quarter q sums blocks S = q, q + 4, ...
    const int o = tid & (4 * HRB - 1), quarter = tid >> 6;
    const int orow = o >> 2, ou = o & 3;
    const int lr = blockIdx.x * HRB + orow;
    Z s0 = czero<Z>(), s1 = czero<Z>();
    if (r0 + lr < n) {
      const int Rb = lr / T, off = lr % T;
      const int nbm = v.hblk;
      const Z* base = v.hpart + (((int64_t)Rb * nbm) * T + off) * 4 + ou;
      const int64_t stride = (int64_t)T * 4;
      int S = quarter;
      for (; S + 4 < nblk; S += 8) { s0 = cadd(s0, base[S * stride]); s1 = cadd(s1, base[(S + 4) * stride]); }
      for (; S < nblk; S += 4) s0 = cadd(s0, base[S * stride]);
    }
    s_part[quarter][o] = cadd(s0, s1);
    // (2) dot products of the panel: 4k outputs, the ndp partials split over NT / 4k threads each
    if (k > 0) {
      const int no = 4 * k;
      const int nsub = NT / no;
      const int t = tid % no, sub = tid / no;
      Z acc = czero<Z>();
      if (sub < nsub) {
        const int i = t >> 2, q = t & 3;
        for (int c = sub; c < ndp; c += nsub) acc = cadd(acc, v.dpart[((int64_t)c * v.nbmax + i) * 4 + q]);
      }
      s_dsub[tid] = acc;
    }
  }
  __syncthreads();
  if (!zero_mode) {
    if (tid < 4 * HRB)
      s_v[tid >> 2][tid & 3] = cadd(cadd(s_part[0][tid], s_part[1][tid]), cadd(s_part[2][tid], s_part[3][tid]));
    if (k > 0 && tid < 4 * k) {
      const int no = 4 * k, nsub = NT / no;
      Z d = s_dsub[tid];
      for (int sub = 1; sub < nsub; ++sub) d = cadd(d, s_dsub[sub * no + tid]);
      s_dots[tid] = d;
    }
  }
  __syncthreads();
  // deferred-update corrections, reflectors split over the groups
  Z ta = czero<Z>(), tb = czero<Z>();
  if (!zero_mode && r < n) {
    for (int i = grp; i < k; i += HNG) {
      const Z s1 = s_dots[4 * i + 0], s2 = s_dots[4 * i + 1], s3 = s_dots[4 * i + 2], s4 = s_dots[4 * i + 3];
      const Z wa = A[r + (int64_t)(p + i) * ld], wb = B[r + (int64_t)(p + i) * ld];
      const Z ya = v.Ya[r + (int64_t)i * v.ldy], yb = v.Yb[r + (int64_t)i * v.ldy];
      // ga -= wa s1 - conj(wb) s2 + ya s3 - conj(yb) s4
      // gb -= wb s1 + conj(wa) s2 + yb s3 + conj(ya) s4
      cfma(ta, wa, s1); cfmac(ta, cneg(wb), s2); cfma(ta, ya, s3); cfmac(ta, cneg(yb), s4);
      cfma(tb, wb, s1); cfmac(tb, wa, s2); cfma(tb, yb, s3); cfmac(tb, ya, s4);
    }
  }
  s_red[grp][row][0] = ta;
  s_red[grp][row][1] = tb;
  __syncthreads();
  double cp = 0.0;
  if (grp == 0 && r < n) {
    Z ga = czero<Z>(), gb = czero<Z>();
    if (!zero_mode) {
      // ha = A x - conj(B z), hb = B x + conj(A z)
      ga = csub(s_v[row][0], cconj(s_v[row][3]));
      gb = cadd(s_v[row][2], cconj(s_v[row][1]));
      for (int g2 = 0; g2 < HNG; ++g2) { ga = csub(ga, s_red[g2][row][0]); gb = csub(gb, s_red[g2][row][1]); }
      const Z wa = A[r + (int64_t)j * ld], wb = B[r + (int64_t)j * ld];
      cp = (double)(wa.x * ga.x + wa.y * ga.y + wb.x * gb.x + wb.y * gb.y);
    }
    v.ga[r] = ga;
    v.gb[r] = gb;
  }
  const double bs = block_sum(cp, s_redd);
  if (tid == 0) v.cpart[blockIdx.x] = bs;
}

// ----------------------------------------------------------------------------
// trailing update of the lower triangles of A (incl. diagonal) and B (strict)
// region [t0, n) x [t0, n), rank-4*nbp structured update.
// ----------------------------------------------------------------------------
constexpr int KC = 4;  // reflectors per smem stage
template <typename R>
__global__ void __launch_bounds__(NT) k_trail(TridiagView<R> v, int p, int nbp, int t0) {
  pdl_wait();  // launched with launch_pdl: the previous kernel's results first
  using Z = cplx<R>;
  const int n = v.n;
  const int64_t ld = v.ld;
  Z* A = v.M;
  Z* B = v.M + n;
  const int t = blockIdx.x;
  int I, J;
  tri_tile(t, I, J);
  const int tid = threadIdx.x;
  const int tr = tid & 15, tc = tid >> 4;
  const int rb = t0 + I * TB, cb = t0 + J * TB;
  // [vector: wa, wb, ya, yb][kk][row]
  __shared__ Z s_r[4][KC][TB];
  __shared__ Z s_c[4][KC][TB];
  Z accA[4][4], accB[4][4];
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int c = 0; c < 4; ++c) { accA[q][c] = czero<Z>(); accB[q][c] = czero<Z>(); }

  for (int k0 = 0; k0 < nbp; k0 += KC) {
    __syncthreads();
    for (int e = tid; e < 4 * KC * TB; e += NT) {
      const int row = e % TB, kk = (e / TB) % KC, vec = e / (TB * KC);
      const int kg = k0 + kk;
      Z vr = czero<Z>(), vc = czero<Z>();
      if (kg < nbp) {
        const int gr = rb + row, gc = cb + row;
        if (gr < n) {
          if (vec == 0) vr = A[gr + (int64_t)(p + kg) * ld];
          else if (vec == 1) vr = B[gr + (int64_t)(p + kg) * ld];
          else if (vec == 2) vr = v.Ya[gr + (int64_t)kg * v.ldy];
          else vr = v.Yb[gr + (int64_t)kg * v.ldy];
        }
        if (gc < n) {
          if (vec == 0) vc = A[gc + (int64_t)(p + kg) * ld];
          else if (vec == 1) vc = B[gc + (int64_t)(p + kg) * ld];
          else if (vec == 2) vc = v.Ya[gc + (int64_t)kg * v.ldy];
          else vc = v.Yb[gc + (int64_t)kg * v.ldy];
        }
      }
      s_r[vec][kk][row] = vr;
      s_c[vec][kk][row] = vc;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < KC; ++kk) {
      Z rwa[4], rwb[4], rya[4], ryb[4], cwa[4], cwb[4], cya[4], cyb[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        rwa[q] = s_r[0][kk][4 * tr + q]; rwb[q] = s_r[1][kk][4 * tr + q];
        rya[q] = s_r[2][kk][4 * tr + q]; ryb[q] = s_r[3][kk][4 * tr + q];
        cwa[q] = s_c[0][kk][4 * tc + q]; cwb[q] = s_c[1][kk][4 * tc + q];
        cya[q] = s_c[2][kk][4 * tc + q]; cyb[q] = s_c[3][kk][4 * tc + q];
      }
#pragma unroll
      for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
          // A += wa conj(ya) + conj(wb) yb + ya conj(wa) + conj(yb) wb
          cfmacb(accA[q][c], rwa[q], cya[c]); cfmac(accA[q][c], rwb[q], cyb[c]);
          cfmacb(accA[q][c], rya[q], cwa[c]); cfmac(accA[q][c], ryb[q], cwb[c]);
          // B += wb conj(ya) - conj(wa) yb + yb conj(wa) - conj(ya) wb
          cfmacb(accB[q][c], rwb[q], cya[c]); cfmac(accB[q][c], cneg(rwa[q]), cyb[c]);
          cfmacb(accB[q][c], ryb[q], cwa[c]); cfmac(accB[q][c], cneg(rya[q]), cwb[c]);
        }
    }
  }
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const int gc = cb + 4 * tc + c;
    if (gc >= n) continue;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int gr = rb + 4 * tr + q;
      if (gr >= n || gr < gc) continue;
      const int64_t o = gr + (int64_t)gc * ld;
      A[o] = csub(A[o], accA[q][c]);
      if (gr > gc) B[o] = csub(B[o], accB[q][c]);
    }
  }
}

// ----------------------------------------------------------------------------
// host driver
// ----------------------------------------------------------------------------
template <typename R>
int tridiagonalize(TridiagView<R> v, int nb, cudaStream_t st) {
  const int n = v.n;
  if (n <= 0) return ZQ_OK;
  if (nb > v.nbmax) nb = v.nbmax;
  if (nb < 1) nb = 1;
  int ncp = 0;  // number of c partials of the previous column
  for (int p = 0; p < n; p += nb) {
    const int nbp = (nb < n - p) ? nb : (n - p);
    for (int k = 0; k < nbp; ++k) {
      const int j = p + k;
      const int L = n - 1 - j;
      const int ncta1 = ceil_div(n - j, RB);
      prof_begin(PC_PANEL, st);
      ZQ_CUDA(launch_pdl(k_colupd<R>, dim3(ncta1), dim3(NT), st, v, p, j, k, ncp, 1));
      count_launch();
      if (L < 1) { prof_end(PC_PANEL, st); ncp = 0; continue; }
      const int ncta2 = ceil_div(L, RB);
      ZQ_CUDA(launch_pdl(k_reflect<R>, dim3(ncta2), dim3(NT), st, v, p, j, k, ncta1));
      count_launch();
      const int T = HT;
      const int nblk = ceil_div(L, T);
      prof_end(PC_PANEL, st);
      if (L >= 2) {
        prof_begin(PC_HEMV, st);
        ZQ_CUDA(launch_pdl(k_hemv<R>, dim3(nblk * (nblk + 1) / 2), dim3(128), st, v, j));
        count_launch();
        prof_end(PC_HEMV, st);
      }
      prof_begin(PC_PANEL, st);
      const int nhr = ceil_div(L, HRB);
      ZQ_CUDA(launch_pdl(k_hreduce<R>, dim3(nhr), dim3(NT), st, v, p, j, k, T, nblk, L < 2 ? 1 : 0, ncta2));
      count_launch();
      prof_end(PC_PANEL, st);
      ncp = nhr;
    }
    const int t0 = p + nbp;
    if (t0 < n) {
      // finish y of the panel's last reflector (rows >= t0), then update
      prof_begin(PC_PANEL, st);
      ZQ_CUDA(launch_pdl(k_colupd<R>, dim3(ceil_div(n - t0, RB)), dim3(NT), st, v, p, t0, nbp, ncp, 0));
      count_launch();
      prof_end(PC_PANEL, st);
      const int nblk = ceil_div(n - t0, TB);
      prof_begin(PC_TRAIL, st);
      ZQ_CUDA(launch_pdl(k_trail<R>, dim3(nblk * (nblk + 1) / 2), dim3(NT), st, v, p, nbp, t0));
      count_launch();
      prof_end(PC_TRAIL, st);
      ncp = 0;
    }
  }
  return ZQ_OK;
}

template <typename R>
size_t tridiag_workspace_bytes(int n, int nbmax) {
  using Z = cplx<R>;
  const size_t hblk = (size_t)ceil_div(n > 0 ? n : 1, 32);
  size_t b = 0;
  b += sizeof(Z) * (2 * (size_t)n * nbmax);          // Ya, Yb
  b += sizeof(Z) * (2 * (size_t)n);                   // ga, gb
  b += sizeof(Z) * ((hblk + 2) * (hblk + 2) * 32 * 4);  // hpart: 32-tiles, or 64-tiles at the same block stride
  b += sizeof(Z) * (hblk * nbmax * 4);                // dpart
  b += sizeof(Z) * (4 * (size_t)nbmax);               // dots
  b += sizeof(double) * (4 * hblk + 8);               // npart (2 hblk), cpart (one per 16 rows), scal
  return b + 16 * 256;
}

template <typename R>
TridiagView<R> tridiag_bind(void* ws, cplx<R>* M, int n, int64_t ld, int nbmax, double* d, double* e, double* tau) {
  using Z = cplx<R>;
  TridiagView<R> v{};
  const int hblk = ceil_div(n > 0 ? n : 1, 32);
  char* p = reinterpret_cast<char*>(ws);
  auto take = [&](size_t bytes) { char* q = p; p += (bytes + 255) & ~(size_t)255; return q; };
  v.M = M; v.n = n; v.ld = ld; v.nbmax = nbmax; v.ldy = n > 0 ? n : 1; v.hblk = hblk;
  v.Ya = reinterpret_cast<Z*>(take(sizeof(Z) * (size_t)n * nbmax));
  v.Yb = reinterpret_cast<Z*>(take(sizeof(Z) * (size_t)n * nbmax));
  v.ga = reinterpret_cast<Z*>(take(sizeof(Z) * (size_t)n));
  v.gb = reinterpret_cast<Z*>(take(sizeof(Z) * (size_t)n));
  v.hpart = reinterpret_cast<Z*>(take(sizeof(Z) * (size_t)(hblk + 2) * (hblk + 2) * 32 * 4));
  v.dpart = reinterpret_cast<Z*>(take(sizeof(Z) * (size_t)hblk * nbmax * 4));
  v.dots = reinterpret_cast<Z*>(take(sizeof(Z) * 4 * (size_t)nbmax));
  v.npart = reinterpret_cast<double*>(take(sizeof(double) * 2 * hblk));
  v.cpart = reinterpret_cast<double*>(take(sizeof(double) * 2 * hblk));
  v.scal = reinterpret_cast<double*>(take(sizeof(double) * 8));
  v.d = d; v.e = e; v.tau = tau;
  return v;
}

template size_t tridiag_workspace_bytes<double>(int, int);
template size_t tridiag_workspace_bytes<float>(int, int);
template TridiagView<double> tridiag_bind<double>(void*, cplx<double>*, int, int64_t, int, double*, double*, double*);
template TridiagView<float> tridiag_bind<float>(void*, cplx<float>*, int, int64_t, int, double*, double*, double*);

template int tridiagonalize<double>(TridiagView<double>, int, cudaStream_t);
template int tridiagonalize<float>(TridiagView<float>, int, cudaStream_t);

}  // namespace zq
