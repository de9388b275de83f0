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
//            norm partials; the last CTA to finish combines them into the
//            reflector head f, f m and the subdiagonal entry e_j)
//   hemv    (quaternion Hermitian mat-vec of the panel-start trailing matrix
//            with w = f x formed on the fly, lower triangles of A and B only,
//            per-tile deterministic partials; extra CTAs form the dot-product
//            partials of w against the panel's previous W, Y)
//   hreduce (sum tile partials and the dot partials, subtract the
//            deferred-update corrections -> g; partials of c; w written in
//            place of x)
// The kernels are launched with programmatic dependent launch (each starts
// with pdl_wait), so a kernel's launch overlaps the tail of the previous one.
// All arithmetic is FP64 (template R = double) for the plain path; the same
// kernels instantiate with R = float for the mixed-precision path, where norms
// and reflector scalars are still formed in double.
#include "zq_common.cuh"
#include "zq_kernels.h"
#include "zq_tc32.h"

#include <cuda.h>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <type_traits>

namespace zq {

constexpr int RB = 32;        // rows per CTA for the row-parallel kernels
constexpr int TB = 64;        // tile edge of the trailing update
constexpr int NT = 256;       // threads per CTA

// ----------------------------------------------------------------------------
// reflector head of column j (warp 0 of one CTA): combines the colupd norm
// partials into nu = |x| and, with x_1 = (scal[0..3]), forms
//   f = 1 / sqrt(nu (nu + |x_1|)),  head of w = f (1 + nu/|x_1|) x_1,
//   e_j = -(nu/|x_1|) x_1  (x_1 = 0: head f nu, e_j = -nu; x = 0: no reflector),
// written to scal[4] (f), scal[5..8] (f m), e[4j..4j+3] and tau[j]. The reads
// bypass L1: the partials come from other CTAs of the running grid.
// ----------------------------------------------------------------------------
// The head's arithmetic (warp 0; lane 0 returns true with the results)
template <typename R>
__device__ bool head_math(const TridiagView<R>& v, int j, int nnp, double& f, double (&m)[4], double (&ee)[4]) {
  const int lane = threadIdx.x;
  const int L = v.n - 1 - j;
  if (lane >= 32 || L < 1) return false;  // the last column has no subdiagonal entry
  const double qa0 = __ldcg(v.scal + 0), qa1 = __ldcg(v.scal + 1), qb0 = __ldcg(v.scal + 2), qb1 = __ldcg(v.scal + 3);
  // nu = scale * sqrt(sum of ssq_i (s_i / scale)^2), scale = max s_i: up to
  // 256 partials are loaded once into registers (one memory latency, one
  // division); more fall back to two passes over memory
  constexpr int PL = 8;
  double sc = 0.0, sq = 0.0;
  if (nnp <= 32 * PL) {
    double ps[PL], pq[PL];
#pragma unroll
    for (int u = 0; u < PL; ++u) {
      const int i = lane + 32 * u;
      ps[u] = (i < nnp) ? __ldcg(v.npart + 2 * i) : 0.0;
      pq[u] = (i < nnp) ? __ldcg(v.npart + 2 * i + 1) : 0.0;
    }
#pragma unroll
    for (int u = 0; u < PL; ++u) sc = fmax(sc, ps[u]);
    sc = warp_max(sc);
    const double inv = sc > 0.0 ? 1.0 / sc : 0.0;
#pragma unroll
    for (int u = 0; u < PL; ++u) { const double q = ps[u] * inv; sq += pq[u] * q * q; }
  } else {
    for (int i = lane; i < nnp; i += 32) sc = fmax(sc, __ldcg(v.npart + 2 * i));
    sc = warp_max(sc);
    const double inv = sc > 0.0 ? 1.0 / sc : 0.0;
    for (int i = lane; i < nnp; i += 32) {
      const double q = __ldcg(v.npart + 2 * i) * inv;
      sq += __ldcg(v.npart + 2 * i + 1) * q * q;
    }
  }
  sq = warp_sum(sq);
  const double nu = sc * sqrt(sq);
  if (lane != 0) return false;
  const double q1 = sqrt(qa0 * qa0 + qa1 * qa1 + qb0 * qb0 + qb1 * qb1);
  f = 0.0;
  m[0] = m[1] = m[2] = m[3] = 0.0;
  ee[0] = qa0; ee[1] = qa1; ee[2] = qb0; ee[3] = qb1;   // L == 1: the entry itself is e_j
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
  return true;
}

template <typename R>
__device__ void head_write(const TridiagView<R>& v, int j, double f, const double (&m)[4], const double (&ee)[4]) {
  v.scal[4] = f;
  for (int q = 0; q < 4; ++q) v.scal[5 + q] = m[q] * f;
  // the same head rounded to R once (scal[12..15] as floats): the FP32 kernels
  // then read it without double-precision conversions
  float* hf = reinterpret_cast<float*>(v.scal + 12);
  hf[0] = (float)f;
  for (int q = 0; q < 4; ++q) hf[1 + q] = (float)(m[q] * f);
  hf[5] = (f > 0.0) ? 1.f : 0.f;
  for (int q = 0; q < 4; ++q) v.e[4 * j + q] = ee[q];
  v.tau[j] = (f > 0.0) ? 1.0 : 0.0;
}

template <typename R>
__device__ void reflector_head(const TridiagView<R>& v, int j, int nnp) {
  double f, m[4], ee[4];
  if (head_math(v, j, nnp, f, m, ee)) head_write(v, j, f, m, ee);
}

// the reflector head in the kernel's precision: f, f m (4 reals), and whether
// a reflector exists (f > 0)
template <typename R>
struct WHead {
  R f, m[4];
  bool live;
};

// The FP32 head of column j formed by warp 0 of every CTA of the persistent
// panel kernel from the norm partials (the same arithmetic as reflector_head,
// so every CTA gets the same bits); CTA 0 also writes it to memory (the
// subdiagonal entry and tau are used after the reduction). Lane 0 stores the
// head in *out.
__device__ void reflector_head_all(const TridiagView<float>& v, int j, int nnp, WHead<float>* out, bool write) {
  double f, m[4], ee[4];
  if (!head_math(v, j, nnp, f, m, ee)) return;
  if (write) head_write(v, j, f, m, ee);
  out->f = (float)f;
  for (int q = 0; q < 4; ++q) out->m[q] = (float)(m[q] * f);
  out->live = f > 0.0;
}

__device__ __forceinline__ void load_head(const TridiagView<float>& v, WHead<float>& h) {
  const float* hf = reinterpret_cast<const float*>(v.scal + 12);
  h.f = hf[0]; h.m[0] = hf[1]; h.m[1] = hf[2]; h.m[2] = hf[3]; h.m[3] = hf[4];
  h.live = hf[5] != 0.f;
}
__device__ __forceinline__ void load_head(const TridiagView<double>& v, WHead<double>& h) {
  h.f = v.scal[4]; h.m[0] = v.scal[5]; h.m[1] = v.scal[6]; h.m[2] = v.scal[7]; h.m[3] = v.scal[8];
  h.live = h.f > 0.0;
}

// w at row r of column j from x (= the stored column before hreduce writes w):
// the head row j+1 takes f m, the others f x; no reflector gives 0.
template <typename R>
__device__ __forceinline__ void w_from_x(const WHead<R>& h, int r, int j, cplx<R>& wa, cplx<R>& wb) {
  if (!h.live) { wa = czero<cplx<R>>(); wb = czero<cplx<R>>(); return; }
  if (r == j + 1) {
    wa = mk(h.m[0], h.m[1]);
    wb = mk(h.m[2], h.m[3]);
  } else {
    wa = cscale(wa, h.f);
    wb = cscale(wb, h.f);
  }
}

// ----------------------------------------------------------------------------
// colupd: rows [j, n) of column j
// ----------------------------------------------------------------------------
// Row block `bid` (rows j + RB bid ..) of column j with NTH threads; writes
// the block's norm partials npart[2 bid], npart[2 bid + 1]. Returns false when
// do_update is 0 (only y_{k-1} finished). Used by k_colupd (one CTA per row
// block) and by the persistent panel kernel.
template <typename R, int NTH>
__device__ bool colupd_block(const TridiagView<R>& v, int p, int j, int k, int ncp, int do_update, int bid) {
  constexpr int NGR = NTH / RB;  // reflector groups
  using Z = cplx<R>;
  const int n = v.n;
  const int64_t ld = v.ld;
  Z* A = v.M;
  Z* B = v.M + n;
  const int r0 = j + bid * RB;
  const int tid = threadIdx.x;
  const int row = tid & (RB - 1);
  const int grp = tid >> 5;
  const int r = r0 + row;
  __shared__ Z s_sc[4 * NBMAX];     // per i: ya_i[j], yb_i[j], wa_i[j], wb_i[j]
  __shared__ Z s_red[NGR][RB][2];
  __shared__ double s_red_d[2][NTH / 32];

  // Every load that does not depend on c_{k-1} is issued first, so the kernel
  // waits about one memory latency instead of one per phase. Reflector i of
  // the panel contributes through (w_i, y_i); y_{k-1} = g - (c/2) w_{k-1} is
  // formed once c is known.
  const bool live = r < n;
  // (1) y_{k-1} on this CTA's rows: w_{k-1} and g
  Z fwa = czero<Z>(), fwb = czero<Z>(), fga = czero<Z>(), fgb = czero<Z>();
  if (k > 0 && grp == 0 && live) {
    fwa = A[r + (int64_t)(j - 1) * ld]; fwb = B[r + (int64_t)(j - 1) * ld];
    fga = v.ga[r]; fgb = v.gb[r];
  }
  // (2) row-j scalars of reflector tid
  Z cwa = czero<Z>(), cwb = czero<Z>(), cya = czero<Z>(), cyb = czero<Z>();
  if (do_update && tid < k) {
    cwa = A[j + (int64_t)(p + tid) * ld]; cwb = B[j + (int64_t)(p + tid) * ld];
    if (tid == k - 1) { cya = v.ga[j]; cyb = v.gb[j]; }
    else { cya = v.Ya[j + (int64_t)tid * v.ldy]; cyb = v.Yb[j + (int64_t)tid * v.ldy]; }
  }
  // (3) this row's entries of the group's first two reflectors (i = grp, grp + NGR)
  Z pw[2][2], py[2][2];
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int i = grp + u * NGR;
    pw[u][0] = pw[u][1] = py[u][0] = py[u][1] = czero<Z>();
    if (do_update && live && i < k) {
      pw[u][0] = A[r + (int64_t)(p + i) * ld]; pw[u][1] = B[r + (int64_t)(p + i) * ld];
      if (i == k - 1) { py[u][0] = v.ga[r]; py[u][1] = v.gb[r]; }
      else { py[u][0] = v.Ya[r + (int64_t)i * v.ldy]; py[u][1] = v.Yb[r + (int64_t)i * v.ldy]; }
    }
  }
  // (4) the column itself
  Z x0a = czero<Z>(), x0b = czero<Z>();
  if (do_update && grp == 0 && live) { x0a = A[r + (int64_t)j * ld]; x0b = B[r + (int64_t)j * ld]; }
  // (5) c_{k-1} = sum of the previous column's partials (deterministic order)
  double cl = 0.0;
  if (k > 0)
    for (int i = tid; i < ncp; i += NTH) cl += v.cpart[i];
  const double csum = (k > 0) ? block_sum(cl, s_red_d[0]) : 0.0;
  const R half_c = (R)(0.5 * csum);

  // finish y_{k-1} = g - (c/2) w_{k-1} on this CTA's rows (rows >= j)
  if (k > 0 && grp == 0 && live) {
    v.Ya[r + (int64_t)(k - 1) * v.ldy] = csub(fga, cscale(fwa, half_c));
    v.Yb[r + (int64_t)(k - 1) * v.ldy] = csub(fgb, cscale(fwb, half_c));
  }
  if (!do_update) return false;

  // scalars at row j for every previous reflector of the panel (k < NBMAX = 128 <= NTH)
  if (tid < k) {
    if (tid == k - 1) { cya = csub(cya, cscale(cwa, half_c)); cyb = csub(cyb, cscale(cwb, half_c)); }
    s_sc[4 * tid + 0] = cya; s_sc[4 * tid + 1] = cyb; s_sc[4 * tid + 2] = cwa; s_sc[4 * tid + 3] = cwb;
  }
  __syncthreads();

  Z da = czero<Z>(), db = czero<Z>();
  auto contrib = [&](int i, Z wa, Z wb, Z ya, Z yb) {
    const Z sya = s_sc[4 * i + 0], syb = s_sc[4 * i + 1], swa = s_sc[4 * i + 2], swb = s_sc[4 * i + 3];
    if (i == k - 1) { ya = csub(ya, cscale(wa, half_c)); yb = csub(yb, cscale(wb, half_c)); }
    // A part: wa conj(ya_j) + conj(wb) yb_j + ya conj(wa_j) + conj(yb) wb_j
    cfmacb(da, wa, sya); cfmac(da, wb, syb); cfmacb(da, ya, swa); cfmac(da, yb, swb);
    // B part: wb conj(ya_j) - conj(wa) yb_j + yb conj(wa_j) - conj(ya) wb_j
    cfmacb(db, wb, sya); cfmac(db, cneg(wa), syb); cfmacb(db, yb, swa); cfmac(db, cneg(ya), swb);
  };
  if (live) {
    if (grp < k) contrib(grp, pw[0][0], pw[0][1], py[0][0], py[0][1]);
    if (grp + NGR < k) contrib(grp + NGR, pw[1][0], pw[1][1], py[1][0], py[1][1]);
    for (int i = grp + 2 * NGR; i < k; i += NGR) {  // panels wider than 2 NGR
      const Z wa = A[r + (int64_t)(p + i) * ld], wb = B[r + (int64_t)(p + i) * ld];
      Z ya, yb;
      if (i == k - 1) { ya = v.ga[r]; yb = v.gb[r]; }
      else { ya = v.Ya[r + (int64_t)i * v.ldy]; yb = v.Yb[r + (int64_t)i * v.ldy]; }
      contrib(i, wa, wb, ya, yb);
    }
  }
  s_red[grp][row][0] = da;
  s_red[grp][row][1] = db;
  __syncthreads();

  double sc = 0.0;  // local max-abs of x (rows >= j+1)
  Z xa = czero<Z>(), xb = czero<Z>();
  if (grp == 0 && r < n) {
    Z ta = s_red[0][row][0], tb = s_red[0][row][1];
    for (int g2 = 1; g2 < NGR; ++g2) { ta = cadd(ta, s_red[g2][row][0]); tb = cadd(tb, s_red[g2][row][1]); }
    xa = csub(x0a, ta);
    xb = csub(x0b, tb);
    A[r + (int64_t)j * ld] = xa;
    B[r + (int64_t)j * ld] = xb;
    if (r == j) v.d[j] = (double)xa.x;
    if (r == j + 1) {
      v.scal[0] = (double)xa.x; v.scal[1] = (double)xa.y;
      v.scal[2] = (double)xb.x; v.scal[3] = (double)xb.y;
      __threadfence();  // before this CTA's arrival is counted
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
    v.npart[2 * bid + 0] = bmax;
    v.npart[2 * bid + 1] = bss;
  }
  return true;
}

template <typename R>
__global__ void __launch_bounds__(NT) k_colupd(TridiagView<R> v, int p, int j, int k, int ncp, int do_update) {
  pdl_wait();  // launched with launch_pdl: the previous kernel's results first
  if (!colupd_block<R, NT>(v, p, j, k, ncp, do_update, (int)blockIdx.x)) return;
  __shared__ bool s_last;
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = atomicAdd(v.counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!s_last) return;
  // every CTA's partials (and x_1) are visible: form the reflector head once
  __threadfence();
  reflector_head(v, j, gridDim.x);
  if (threadIdx.x == 0) *v.counter = 0u;
}

// ----------------------------------------------------------------------------
// dot partials of w (rows [j+1, n)) against the panel's previous reflectors
// and aux vectors, DR rows per CTA (warp = 32 rows, lane = row):
//   <y_i,w> = ya^H wa + yb^H wb,  [y_i,w] = ya^T wb - yb^T wa,  same for w_i.
// The warps' sums meet in `scratch` (4 warps x k x 4) and the CTA writes one
// partial per (i, product).
// ----------------------------------------------------------------------------
constexpr int DR = 128;       // rows per dot-partial CTA
template <typename R>
__device__ void panel_dots(const TridiagView<R>& v, int p, int j, int k, int b, int ndot, cplx<R>* scratch,
                           const WHead<R>* hd = nullptr) {
  using Z = cplx<R>;
  const int n = v.n;
  const int64_t ld = v.ld;
  const Z* A = v.M;
  const Z* B = v.M + n;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gr = j + 1 + b * DR + warp * 32 + lane;
  const bool live = gr < n;
  WHead<R> h;
  Z xa = czero<Z>(), xb = czero<Z>();
  if (live) {
    if (hd) h = *hd; else load_head(v, h);
    xa = A[gr + (int64_t)j * ld];
    xb = B[gr + (int64_t)j * ld];
  }
  Z ya[4], yb[4], qa[4], qb[4];
  for (int i0 = 0; i0 < k; i0 += 4) {
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = i0 + u;
      ya[u] = yb[u] = qa[u] = qb[u] = czero<Z>();
      if (live && i < k) {
        ya[u] = v.Ya[gr + (int64_t)i * v.ldy]; yb[u] = v.Yb[gr + (int64_t)i * v.ldy];
        qa[u] = A[gr + (int64_t)(p + i) * ld]; qb[u] = B[gr + (int64_t)(p + i) * ld];
      }
    }
    if (i0 == 0 && live) w_from_x<R>(h, gr, j, xa, xb);
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = i0 + u;
      if (i >= k) break;
      Z d1 = czero<Z>(), d2 = czero<Z>(), d3 = czero<Z>(), d4 = czero<Z>();
      cfmac(d1, ya[u], xa); cfmac(d1, yb[u], xb);
      cfma(d2, ya[u], xb); cfma(d2, cneg(yb[u]), xa);
      cfmac(d3, qa[u], xa); cfmac(d3, qb[u], xb);
      cfma(d4, qa[u], xb); cfma(d4, cneg(qb[u]), xa);
      d1.x = warp_sum(d1.x); d1.y = warp_sum(d1.y);
      d2.x = warp_sum(d2.x); d2.y = warp_sum(d2.y);
      d3.x = warp_sum(d3.x); d3.y = warp_sum(d3.y);
      d4.x = warp_sum(d4.x); d4.y = warp_sum(d4.y);
      if (lane == 0) {
        Z* o = scratch + ((int64_t)warp * k + i) * 4;
        o[0] = d1; o[1] = d2; o[2] = d3; o[3] = d4;
      }
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < 4 * k; t += blockDim.x) {
    Z acc = scratch[t];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) acc = cadd(acc, scratch[w * 4 * k + t]);
    v.dpart[((int64_t)b * v.nbmax + (t >> 2)) * 4 + (t & 3)] = acc;
  }
  // the last dot CTA to finish sums all ndot partials into dots (fixed order:
  // nsplit threads per output over interleaved partials, then combined in order)
  __threadfence();
  __shared__ unsigned s_ticket;
  __syncthreads();
  if (threadIdx.x == 0) s_ticket = atomicAdd(v.counter + 1, 1u);
  __syncthreads();
  if (s_ticket != (unsigned)(ndot - 1)) return;
  __threadfence();
  const int no = 4 * k;
  if (no > (int)blockDim.x) {  // panels wider than 32: one thread per output
    for (int o = threadIdx.x; o < no; o += blockDim.x) {
      Z d = czero<Z>();
#pragma unroll 8
      for (int c = 0; c < ndot; ++c) d = cadd(d, __ldcg(v.dpart + ((int64_t)c * v.nbmax + (o >> 2)) * 4 + (o & 3)));
      v.dots[o] = d;
    }
  } else {
    const int nsplit = (int)blockDim.x / no;
    const int t = threadIdx.x % no, sp = threadIdx.x / no;
    Z acc = czero<Z>();
    if (sp < nsplit) {
#pragma unroll 8
      for (int c = sp; c < ndot; c += nsplit)
        acc = cadd(acc, __ldcg(v.dpart + ((int64_t)c * v.nbmax + (t >> 2)) * 4 + (t & 3)));
    }
    __syncthreads();  // scratch is free again
    scratch[threadIdx.x] = acc;
    __syncthreads();
    if ((int)threadIdx.x < no) {
      Z d = scratch[threadIdx.x];
      for (int u = 1; u < nsplit; ++u) d = cadd(d, scratch[u * no + threadIdx.x]);
      v.dots[threadIdx.x] = d;
    }
  }
  if (threadIdx.x == 0) v.counter[1] = 0u;
}

// ----------------------------------------------------------------------------
// hemv: quaternion Hermitian mat-vec of the panel-start trailing matrix.
//   Region rows/cols [r0, n); lower-triangle 32x32 tiles, one CTA per tile
//   after the first ndot CTAs, which form the panel dot partials.
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
__global__ void __launch_bounds__(128) k_hemv(TridiagView<R> v, int p, int j, int k, int ndot) {
  pdl_wait();  // launched with launch_pdl: the previous kernel's results first
  using Z = cplx<R>;
  const int n = v.n;
  const int64_t ld = v.ld;
  const Z* A = v.M;
  const Z* B = v.M + n;
  const int r0 = j + 1;
  __shared__ Z sAB[2 * HT * HLD];   // the A and B tiles (also the dot CTAs' scratch: 4 warps x 128 x 4)
  Z* sA = sAB;
  Z* sB = sAB + HT * HLD;
  __shared__ Z sx[2][HT], sz[2][HT];   // [0]: rows of block I, [1]: rows of block J
  __shared__ Z sout[HT][4];
  // the first ndot CTAs form the panel dot partials (they start first and run
  // beside the tiles); sAB (2 HT HLD >= 4 warps x 128 x 4) is their scratch
  if ((int)blockIdx.x < ndot) {
    panel_dots(v, p, j, k, blockIdx.x, ndot, sA);
    return;
  }
  const int t = blockIdx.x - ndot;
  int I, J;
  tri_tile(t, I, J);
  const bool diag = (I == J);
  const int tid = threadIdx.x;
  const int rbase = r0 + I * HT, cbase = r0 + J * HT;
  // all of this thread's loads are issued before any is used: 8 elements of
  // each tile (one column of 32 rows per warp and step: coalesced), the two
  // w segments and the reflector head
  constexpr int PER = HT * HT / 128;
  Z ta[PER], tb[PER];
#pragma unroll
  for (int u = 0; u < PER; ++u) {
    const int e = tid + 128 * u;
    const int r = e & (HT - 1), c = e >> 5;
    const int gr = rbase + r, gc = cbase + c;
    ta[u] = czero<Z>(); tb[u] = czero<Z>();
    if (gr < n && gc < n && (!diag || r >= c)) {
      // streaming loads (evict first): the trailing matrix passes through L2
      // once per column, the tile partials written below are read next
      ta[u] = __ldcs(A + gr + (int64_t)gc * ld);
      tb[u] = __ldcs(B + gr + (int64_t)gc * ld);
    }
  }
  const int ws = tid >> 5, wq = tid & (HT - 1);
  const int wg = (ws == 0 ? rbase : cbase) + wq;
  const bool wrow = tid < 2 * HT && wg < n;
  Z x = czero<Z>(), z = czero<Z>();
  WHead<R> h;
  if (wrow) {
    load_head(v, h);
    x = A[wg + (int64_t)j * ld];
    z = B[wg + (int64_t)j * ld];
  }
#pragma unroll
  for (int u = 0; u < PER; ++u) {
    const int e = tid + 128 * u;
    const int r = e & (HT - 1), c = e >> 5;
    if (diag && r == c) { ta[u].y = 0; tb[u] = czero<Z>(); }
    sA[r + c * HLD] = ta[u];
    sB[r + c * HLD] = tb[u];
  }
  if (tid < 2 * HT) {
    if (wrow) {
      w_from_x<R>(h, wg, j, x, z);
      z = cconj(z);
    }
    sx[ws][wq] = x;
    sz[ws][wq] = z;
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
    // column q: rows above q are zero in a diagonal tile; the diagonal itself
    // belongs to the row products
#pragma unroll
    for (int r = 0; r < HT; r += 2) {
      Z m0 = sA[r + q * HLD], m1 = sA[r + 1 + q * HLD];
      if (diag && r == q) m0 = czero<Z>();
      if (diag && r + 1 == q) m1 = czero<Z>();
      cfmac(p0, m0, sx[0][r]); cfmac(p1, m0, sz[0][r]);
      cfmac(p2, m1, sx[0][r + 1]); cfmac(p3, m1, sz[0][r + 1]);
    }
  } else {
#pragma unroll
    for (int r = 0; r < HT; r += 2) {
      Z m0 = sB[r + q * HLD], m1 = sB[r + 1 + q * HLD];
      if (diag && r == q) m0 = czero<Z>();
      if (diag && r + 1 == q) m1 = czero<Z>();
      cfma(p0, m0, sx[0][r]); cfma(p1, m0, sz[0][r]);
      cfma(p2, m1, sx[0][r + 1]); cfma(p3, m1, sz[0][r + 1]);
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
// hemv, FP32 with TMA staging (even n): the same products and partial layout
// as k_hemv, but
//   * the A and B tiles arrive by cp.async.bulk.tensor: each 32 x 32 complex
//     tile is two 16-row boxes (128 bytes of rows, 128-byte swizzle, zeros
//     outside the matrix) issued by one thread, completed on an mbarrier;
//   * the tile grid starts at the even row b0 = r0 - (r0 & 1), as a TMA box
//     must start on a 16-byte boundary; row / column b0 < r0 carries w = 0 and
//     its output is not read (k_hreduce is told the shift);
//   * a complex multiply-add m v is two packed FP32 FMAs on the natural pair
//     (m.x, m.y): P += (m.x, m.y) (v.x, v.x), Q += (m.x, m.y) (v.y, v.y), and
//     m v = (P.x - Q.y, P.y + Q.x), conj(m) v = (P.x + Q.y, Q.x - P.y), so the
//     vectors are kept in shared memory as (v.x, v.x, v.y, v.y).
// Warp roles as k_hemv: 0 A rows, 1 B rows, 2 A^H columns, 3 -B^T columns.
// ----------------------------------------------------------------------------
constexpr int HM_SMEM = 16384 + 1024;  // two tiles (8 KB each) + alignment
__device__ __forceinline__ void fma2(float2& acc, float2 a, float2 b) {
  asm("{\n\t.reg .b64 ra, rb, rc;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\tmov.b64 rc, {%0, %1};\n\t"
      "fma.rn.f32x2 rc, ra, rb, rc;\n\tmov.b64 {%0, %1}, rc;\n\t}"
      : "+f"(acc.x), "+f"(acc.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
}
__device__ __forceinline__ float2 lds2(uint32_t a) {
  float2 v;
  asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(a));
  return v;
}

// One work item of the TMA hemv grid with 128 threads: items < ndot are panel
// dot partials, the others lower-triangle tiles. `tiles` is a 1024-aligned
// 16 KB shared buffer, `bar` an initialised mbarrier whose next phase has
// parity `par`; `hd` the reflector head when the caller holds it. Returns
// false if the tile copy did not arrive within the wait limit.
__device__ bool hemv_tma_item(const CUtensorMap* tmp, const TridiagView<float>& v, int p, int j, int k, int ndot, int b0,
                              int item, uint32_t tiles, unsigned char* tiles_gen, uint32_t bar, uint32_t par,
                              const WHead<float>* hd) {
  using Z = float2;
  __shared__ float4 s_xd[2][HT], s_zd[2][HT];       // [0]: block I rows, [1]: block J rows
  __shared__ Z sout[HT][4];
  const int n = v.n;
  const int64_t ld = v.ld;
  const Z* A = v.M;
  const Z* B = v.M + n;
  if (item < ndot) {
    panel_dots(v, p, j, k, item, ndot, reinterpret_cast<Z*>(tiles_gen), hd);
    return true;
  }
  const int t = item - ndot;
  int I, J;
  tri_tile(t, I, J);
  const bool diag = (I == J);
  const int tid = threadIdx.x;
  const int rbase = b0 + I * HT, cbase = b0 + J * HT;
  if (tid == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(16384u) : "memory");
    const uint64_t tma = reinterpret_cast<uint64_t>(tmp);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int x = (q >= 2 ? n : 0) + rbase + 16 * (q & 1);   // row: even (b0, n even)
      asm volatile(
          "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
              tiles + 4096u * q),
          "l"(tma), "r"(x), "r"(cbase), "r"(bar)
          : "memory");
    }
  }
  // meanwhile: w on the rows of block I (column products) and block J (row products)
  if (tid < 2 * HT) {
    const int ws = tid >> 5, wq = tid & (HT - 1);
    const int wg = (ws == 0 ? rbase : cbase) + wq;
    Z x = czero<Z>(), z = czero<Z>();
    if (wg > j && wg < n) {
      WHead<float> h;
      if (hd) h = *hd; else load_head(v, h);
      x = A[wg + (int64_t)j * ld];
      z = B[wg + (int64_t)j * ld];
      w_from_x<float>(h, wg, j, x, z);
      z = cconj(z);
    }
    s_xd[ws][wq] = make_float4(x.x, x.x, x.y, x.y);
    s_zd[ws][wq] = make_float4(z.x, z.x, z.y, z.y);
  }
  __syncthreads();
  {
    // bounded wait for the tiles (the copies take microseconds)
    const long long t0 = clock64();
    uint32_t ok = 0;
    while (!ok) {
      asm volatile(
          "{\n\t.reg .pred pp;\n\tmbarrier.try_wait.parity.shared::cta.b64 pp, [%1], %2;\n\tselp.u32 %0, 1, 0, pp;\n\t}"
          : "=r"(ok)
          : "r"(bar), "r"(par)
          : "memory");
      if (!ok && clock64() - t0 > 4000000000LL) break;
    }
    if (!__syncthreads_and(ok != 0)) {
      if (tid == 0 && v.tc_err) atomicExch(v.tc_err, 1);
      return false;
    }
  }
  const int role = tid >> 5, q = tid & (HT - 1);
  Z P0 = czero<Z>(), Q0 = czero<Z>(), P1 = czero<Z>(), Q1 = czero<Z>();
  if (role < 2) {
    // row q of the tile, all 32 columns: element (q, c) of a swizzled 16-row box
    // sits at box * 4096 + c * 128 + (((q & 15) >> 1) ^ (c & 7)) * 16 + (q & 1) * 8
    const uint32_t rowb = tiles + (uint32_t)role * 8192u + (uint32_t)(q >> 4) * 4096u + (uint32_t)(q & 1) * 8u;
    const int hr = (q & 15) >> 1;
    if (!diag) {
#pragma unroll
      for (int c = 0; c < HT; ++c) {
        const float2 m = lds2(rowb + (uint32_t)c * 128u + (uint32_t)((hr ^ (c & 7)) << 4));
        const float4 xd = s_xd[1][c], zd = s_zd[1][c];
        fma2(P0, m, make_float2(xd.x, xd.y)); fma2(Q0, m, make_float2(xd.z, xd.w));
        fma2(P1, m, make_float2(zd.x, zd.y)); fma2(Q1, m, make_float2(zd.z, zd.w));
      }
    } else {
      for (int c = 0; c <= q; ++c) {
        float2 m = lds2(rowb + (uint32_t)c * 128u + (uint32_t)((hr ^ (c & 7)) << 4));
        if (c == q) { if (role == 0) m.y = 0.f; else m = czero<Z>(); }  // real diagonal of A, zero of B
        const float4 xd = s_xd[1][c], zd = s_zd[1][c];
        fma2(P0, m, make_float2(xd.x, xd.y)); fma2(Q0, m, make_float2(xd.z, xd.w));
        fma2(P1, m, make_float2(zd.x, zd.y)); fma2(Q1, m, make_float2(zd.z, zd.w));
      }
    }
  } else {
    // column q, all 32 rows r: element (r, q) at (r >> 4) * 4096 + q * 128 + (((r & 15) >> 1) ^ (q & 7)) * 16 + (r & 1) * 8
    const uint32_t colb = tiles + (uint32_t)(role - 2) * 8192u + (uint32_t)q * 128u;
    const int hq = q & 7;
    if (!diag) {
#pragma unroll
      for (int r = 0; r < HT; ++r) {
        const float2 m = lds2(colb + (uint32_t)(r >> 4) * 4096u + (uint32_t)((((r & 15) >> 1) ^ hq) << 4) + (uint32_t)(r & 1) * 8u);
        const float4 xd = s_xd[0][r], zd = s_zd[0][r];
        fma2(P0, m, make_float2(xd.x, xd.y)); fma2(Q0, m, make_float2(xd.z, xd.w));
        fma2(P1, m, make_float2(zd.x, zd.y)); fma2(Q1, m, make_float2(zd.z, zd.w));
      }
    } else {
      for (int r = q + 1; r < HT; ++r) {  // diagonal tile: strictly below the diagonal
        const float2 m = lds2(colb + (uint32_t)(r >> 4) * 4096u + (uint32_t)((((r & 15) >> 1) ^ hq) << 4) + (uint32_t)(r & 1) * 8u);
        const float4 xd = s_xd[0][r], zd = s_zd[0][r];
        fma2(P0, m, make_float2(xd.x, xd.y)); fma2(Q0, m, make_float2(xd.z, xd.w));
        fma2(P1, m, make_float2(zd.x, zd.y)); fma2(Q1, m, make_float2(zd.z, zd.w));
      }
    }
  }
  // this warp's two products
  Z u0, u1;
  if (role < 2) {            // m v
    u0 = mk(P0.x - Q0.y, P0.y + Q0.x); u1 = mk(P1.x - Q1.y, P1.y + Q1.x);
  } else if (role == 2) {    // conj(m) v
    u0 = mk(P0.x + Q0.y, Q0.x - P0.y); u1 = mk(P1.x + Q1.y, Q1.x - P1.y);
  } else {                   // -m v
    u0 = mk(Q0.y - P0.x, -(P0.y + Q0.x)); u1 = mk(Q1.y - P1.x, -(P1.y + Q1.x));
  }
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
  return true;
}

__global__ void __launch_bounds__(128) k_hemv_tma(const __grid_constant__ CUtensorMap tm, TridiagView<float> v, int p,
                                                  int j, int k, int ndot, int b0) {
  pdl_wait();  // launched with launch_pdl: the previous kernel's results first
  extern __shared__ __align__(1024) unsigned char hm_raw[];
  const uint32_t raw = (uint32_t)__cvta_generic_to_shared(hm_raw);
  const uint32_t tiles = (raw + 1023u) & ~1023u;    // A tile at +0, B tile at +8192
  __shared__ __align__(8) unsigned long long s_bar;
  const uint32_t bar = (uint32_t)__cvta_generic_to_shared(&s_bar);
  if ((int)blockIdx.x >= ndot && threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  hemv_tma_item(&tm, v, p, j, k, ndot, b0, (int)blockIdx.x, tiles, hm_raw + (tiles - raw), bar, 0u, nullptr);
}



// ----------------------------------------------------------------------------
// hreduce: g = H_panelstart w - corrections, for rows [j+1, n); c partials;
//   w = f x written in place of x.
//   T is the hemv tile edge used for this column; nblk its number of blocks.
//   HRB rows per CTA; NSPL threads per (row, product) sum the hemv tile
//   partials (fixed split and combine order: deterministic). The panel dot
//   products come finished from the hemv grid (dots). All loads that do not
//   depend on one another are issued before the first is used.
// ----------------------------------------------------------------------------
constexpr int HRB = 8;                 // rows per CTA
// Row block `bid` (rows j + 1 + HRB bid ..) with NTH threads; `hd` is the
// reflector head when the caller holds it (null: read from scal).
template <typename R, int NTH>
__device__ void hreduce_block(const TridiagView<R>& v, int p, int j, int k, int T, int nblk, int zero_mode, int sh,
                              int bid, const WHead<R>* hd) {
  constexpr int HNG = NTH / HRB;          // reflector groups for the corrections
  constexpr int NSPL = NTH / (4 * HRB);   // threads per (row, product) for the tile partials
  using Z = cplx<R>;
  const int n = v.n;
  const int64_t ld = v.ld;
  Z* A = v.M;
  Z* B = v.M + n;
  const int r0 = j + 1;
  const int tid = threadIdx.x;
  const int row = tid & (HRB - 1), grp = tid / HRB;
  const int r = r0 + bid * HRB + row;
  __shared__ Z s_v[HRB][4];
  __shared__ Z s_dots[4 * NBMAX];
  __shared__ Z s_part[NSPL][4 * HRB];
  __shared__ Z s_red[HNG][HRB][2];
  __shared__ double s_redd[NTH / 32];
  // this row's x and the reflector head (w = f x is written in place at the end)
  WHead<R> h;
  Z xa = czero<Z>(), xb = czero<Z>();
  if (grp == 0 && r < n) {
    if (hd) h = *hd; else load_head(v, h);
    xa = A[r + (int64_t)j * ld];
    xb = B[r + (int64_t)j * ld];
  }
  // the group's first reflector (w_i, y_i) at this row, and the panel dots
  Z cwa = czero<Z>(), cwb = czero<Z>(), cya = czero<Z>(), cyb = czero<Z>(), dt = czero<Z>();
  if (!zero_mode) {
    if (r < n && grp < k) {
      cwa = A[r + (int64_t)(p + grp) * ld]; cwb = B[r + (int64_t)(p + grp) * ld];
      cya = v.Ya[r + (int64_t)grp * v.ldy]; cyb = v.Yb[r + (int64_t)grp * v.ldy];
    }
    if (tid < 4 * k) dt = v.dots[tid];
    // tile partials: output o = (row, product); split sp sums blocks S = sp, sp + NSPL, ...
    const int o = tid & (4 * HRB - 1), sp = tid / (4 * HRB);
    const int lr = bid * HRB + (o >> 2);
    Z s0 = czero<Z>(), s1 = czero<Z>(), s2 = czero<Z>(), s3 = czero<Z>();
    if (r0 + lr < n) {
      const int Rb = (lr + sh) / T, off = (lr + sh) % T;  // the hemv tile grid starts sh rows above r0
      const Z* base = v.hpart + (((int64_t)Rb * v.hblk) * T + off) * 4 + (o & 3);
      const int64_t stride = (int64_t)T * 4;
      int S = sp;
#pragma unroll 2
      for (; S + 3 * NSPL < nblk; S += 4 * NSPL) {
        const Z a0 = base[S * stride], a1 = base[(S + NSPL) * stride], a2 = base[(S + 2 * NSPL) * stride],
                a3 = base[(S + 3 * NSPL) * stride];
        s0 = cadd(s0, a0); s1 = cadd(s1, a1); s2 = cadd(s2, a2); s3 = cadd(s3, a3);
      }
      for (; S < nblk; S += NSPL) s0 = cadd(s0, base[S * stride]);
    }
    s_part[sp][o] = cadd(cadd(s0, s2), cadd(s1, s3));
    if (tid < 4 * k) s_dots[tid] = dt;
    for (int q = tid + NTH; q < 4 * k; q += NTH) s_dots[q] = v.dots[q];  // wide panels
  }
  __syncthreads();
  if (!zero_mode && tid < 4 * HRB) {
    Z t = s_part[0][tid];
#pragma unroll
    for (int u = 1; u < NSPL; ++u) t = cadd(t, s_part[u][tid]);
    s_v[tid >> 2][tid & 3] = t;
  }
  // deferred-update corrections, reflectors split over the groups
  Z ta = czero<Z>(), tb = czero<Z>();
  if (!zero_mode && r < n) {
    for (int i = grp; i < k; i += HNG) {
      Z wa = cwa, wb = cwb, ya = cya, yb = cyb;
      if (i != grp) {
        wa = A[r + (int64_t)(p + i) * ld]; wb = B[r + (int64_t)(p + i) * ld];
        ya = v.Ya[r + (int64_t)i * v.ldy]; yb = v.Yb[r + (int64_t)i * v.ldy];
      }
      const Z s1 = s_dots[4 * i + 0], s2 = s_dots[4 * i + 1], s3 = s_dots[4 * i + 2], s4 = s_dots[4 * i + 3];
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
    Z wa = xa, wb = xb;
    w_from_x<R>(h, r, j, wa, wb);
    A[r + (int64_t)j * ld] = wa;
    B[r + (int64_t)j * ld] = wb;
    Z ga = czero<Z>(), gb = czero<Z>();
    if (!zero_mode) {
      // ha = A x - conj(B z), hb = B x + conj(A z)
      ga = csub(s_v[row][0], cconj(s_v[row][3]));
      gb = cadd(s_v[row][2], cconj(s_v[row][1]));
      const int ng = k < HNG ? k : HNG;   // groups that hold a correction
      for (int g2 = 0; g2 < ng; ++g2) { ga = csub(ga, s_red[g2][row][0]); gb = csub(gb, s_red[g2][row][1]); }
      cp = (double)(wa.x * ga.x + wa.y * ga.y + wb.x * gb.x + wb.y * gb.y);
    }
    v.ga[r] = ga;
    v.gb[r] = gb;
  }
  const double bs = block_sum(cp, s_redd);
  if (tid == 0) v.cpart[bid] = bs;
}

template <typename R>
__global__ void __launch_bounds__(NT) k_hreduce(TridiagView<R> v, int p, int j, int k, int T, int nblk, int zero_mode,
                                                int sh) {
  pdl_wait();  // launched with launch_pdl: the previous kernel's results first
  hreduce_block<R, NT>(v, p, j, k, T, nblk, zero_mode, sh, (int)blockIdx.x, nullptr);
}

// ----------------------------------------------------------------------------
// trailing update of the lower triangles of A (incl. diagonal) and B (strict)
// region [t0, n) x [t0, n), rank-4*nbp structured update.
// ----------------------------------------------------------------------------
constexpr int KC = 4;  // reflectors per smem stage
__device__ __forceinline__ void cp_async8_zfill(void* smem, const void* gmem, bool pred) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(sa), "l"(gmem), "r"(pred ? 8 : 0) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// the rank-4 KC products of one K stage into the 4 x 4 complex micro-tiles
template <typename Z>
__device__ __forceinline__ void trail_stage(const Z (&sr)[4][KC][TB], const Z (&sc)[4][KC][TB], int tr, int tc,
                                            Z (&accA)[4][4], Z (&accB)[4][4]) {
#pragma unroll
  for (int kk = 0; kk < KC; ++kk) {
    Z rwa[4], rwb[4], rya[4], ryb[4], cwa[4], cwb[4], cya[4], cyb[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      rwa[q] = sr[0][kk][4 * tr + q]; rwb[q] = sr[1][kk][4 * tr + q];
      rya[q] = sr[2][kk][4 * tr + q]; ryb[q] = sr[3][kk][4 * tr + q];
      cwa[q] = sc[0][kk][4 * tc + q]; cwb[q] = sc[1][kk][4 * tc + q];
      cya[q] = sc[2][kk][4 * tc + q]; cyb[q] = sc[3][kk][4 * tc + q];
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
  Z accA[4][4], accB[4][4];
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int c = 0; c < 4; ++c) { accA[q][c] = czero<Z>(); accB[q][c] = czero<Z>(); }

  if constexpr (std::is_same<R, float>::value) {
    // FP32: the [vector: wa, wb, ya, yb][kk][row] stages double-buffered by
    // cp.async (zero fill outside the matrix): the next stage's copies are in
    // flight while this stage's products run, instead of each thread's loads
    // waiting in turn before every stage
    __shared__ Z s_r[2][4][KC][TB];
    __shared__ Z s_c[2][4][KC][TB];
    auto issue = [&](int k0, int buf) {
      for (int e = tid; e < 4 * KC * TB; e += NT) {
        const int row = e % TB, kk = (e / TB) % KC, vec = e / (TB * KC);
        const int kg = k0 + kk;
        const bool kok = kg < nbp;
        const int kc = kok ? kg : 0;
        const Z* base = vec == 0 ? A + (int64_t)(p + kc) * ld
                      : vec == 1 ? B + (int64_t)(p + kc) * ld
                      : vec == 2 ? v.Ya + (int64_t)kc * v.ldy
                                 : v.Yb + (int64_t)kc * v.ldy;
        const bool rok = kok && rb + row < n, cok = kok && cb + row < n;
        cp_async8_zfill(&s_r[buf][vec][kk][row], base + (rok ? rb + row : 0), rok);
        cp_async8_zfill(&s_c[buf][vec][kk][row], base + (cok ? cb + row : 0), cok);
      }
      cp_async_commit();
    };
    issue(0, 0);
    for (int k0 = 0, st = 0; k0 < nbp; k0 += KC, ++st) {
      const int buf = st & 1;
      if (k0 + KC < nbp) { issue(k0 + KC, buf ^ 1); cp_async_wait<1>(); } else { cp_async_wait<0>(); }
      __syncthreads();
      trail_stage<Z>(s_r[buf], s_c[buf], tr, tc, accA, accB);
      __syncthreads();  // the buffer is refilled by the issue two stages on
    }
  } else {
    // [vector: wa, wb, ya, yb][kk][row]
    __shared__ Z s_r[4][KC][TB];
    __shared__ Z s_c[4][KC][TB];
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
      trail_stage<Z>(s_r, s_c, tr, tc, accA, accB);
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

// TMA-staged FP32 hemv on (default) or the register-staged k_hemv (environment
// ZQ_HEMV=ldg)
static bool hemv_tma_enabled() {
  static const bool on = [] {
    const char* e = getenv("ZQ_HEMV");
    return !(e && !strcmp(e, "ldg"));
  }();
  return on;
}

// The same trailing update on the tensor cores (zq_tc32.cu), FP32 path, used
// only where ZQ_TC32_USES names it: the lower triangles of the (n - t0)^2
// trailing blocks of A and B take one rank-4 nbp product each,
//   A -= [Wa | conj(Wb) | Ya | conj(Yb)] [conj(Ya) | Yb | conj(Wa) | Wb]^T   (i >= j)
//   B -= [Wb | -conj(Wa) | Yb | -conj(Ya)] [conj(Ya) | Yb | conj(Wa) | Wb]^T (i > j)
// with W the panel's reflectors (stored in place, columns p..p+nbp-1) and Y
// its aux vectors, all read at rows t0.. (128 x 128 lower tiles only).
static Tc32Src trail_src(const float2* p, int64_t ld, int conj, float sign) {
  Tc32Src s{};
  s.p = reinterpret_cast<const float*>(p); s.ld = ld; s.kfast = 0; s.conj = conj; s.sign = sign;
  return s;
}
static int trail_tc32(const TridiagView<float>& v, int p, int nbp, int t0, cudaStream_t st) {
  const int n = v.n;
  const int64_t ld = v.ld;
  const float2* Wa = v.M + t0 + (int64_t)p * ld;
  const float2* Wb = v.M + n + t0 + (int64_t)p * ld;
  const float2* Ya = v.Ya + t0;
  const float2* Yb = v.Yb + t0;
  for (int half = 0; half < 2; ++half) {
    Tc32Args t{};
    t.cplx = 1; t.m = n - t0; t.n = n - t0; t.nseg = 4;
    // column operand, shared by both updates
    t.seg[0].b = trail_src(Ya, v.ldy, 1, 1.f);
    t.seg[1].b = trail_src(Yb, v.ldy, 0, 1.f);
    t.seg[2].b = trail_src(Wa, ld, 1, 1.f);
    t.seg[3].b = trail_src(Wb, ld, 0, 1.f);
    if (half == 0) {
      t.seg[0].a = trail_src(Wa, ld, 0, 1.f);
      t.seg[1].a = trail_src(Wb, ld, 1, 1.f);
      t.seg[2].a = trail_src(Ya, v.ldy, 0, 1.f);
      t.seg[3].a = trail_src(Yb, v.ldy, 1, 1.f);
    } else {
      t.seg[0].a = trail_src(Wb, ld, 0, 1.f);
      t.seg[1].a = trail_src(Wa, ld, 1, -1.f);
      t.seg[2].a = trail_src(Yb, v.ldy, 0, 1.f);
      t.seg[3].a = trail_src(Ya, v.ldy, 1, -1.f);
    }
    for (int q = 0; q < 4; ++q) t.seg[q].k = nbp;
    t.alpha = make_float2(-1.f, 0.f); t.beta = make_float2(1.f, 0.f);
    t.C = reinterpret_cast<float*>(v.M + (half ? n : 0) + t0 + (int64_t)t0 * ld);
    t.ldc = ld;
    t.tri = half ? 2 : 1;
    t.splits = 1;
    t.err = v.tc_err;
    if (int rc = tc32_gemm(t, st)) return rc;
  }
  return ZQ_OK;
}


// ----------------------------------------------------------------------------
// Persistent panel kernel (FP32 with the TMA mat-vec; opt-in, ZQ_TRIDIAG=persist):
// the columns of one panel in a single cooperative launch. Per column the
// three phases of the kernel sequence above (colupd row blocks, hemv items,
// hreduce row blocks) run as loops over the resident CTAs with a grid barrier
// after each, and every CTA forms the reflector head itself after the first
// barrier: 3 nb barriers instead of 3 nb launches. Measured slower than the
// launches at every size (FP32 reduction at n2 = 1024 / 4096 / 8192: 12.6-14.3
// / 64-69 / 198-265 ms with 1-6 CTAs per SM, against 11.6 / 53.2 / 156.4 ms):
// a grid barrier costs about what a dependent launch does, and a fixed grid
// streams the mat-vec tiles more slowly than thousands of one-tile CTAs.
// ----------------------------------------------------------------------------
constexpr int PT = 128;  // threads per CTA of the persistent panel kernel
constexpr int PT_SMEM = 1024 + 16384;  // 1024-aligned 16 KB tile buffer

// Grid barrier of the persistent kernel (cooperative launch: every CTA is
// resident). counter[2] counts arrivals, counter[3] is the generation,
// counter[4] the abort flag. A wait longer than `limit` cycles raises the
// abort flag and tc_err, after which every barrier returns at once (false).
__device__ bool grid_barrier(const TridiagView<float>& v, long long limit) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* gen = v.counter + 3;
    volatile unsigned* abt = v.counter + 4;
    int ok = *abt == 0u;
    if (ok) {
      const unsigned g0 = *gen;  // read before arriving: it cannot advance until this CTA arrives
      __threadfence();
      if (atomicAdd(v.counter + 2, 1u) == gridDim.x - 1) {
        atomicExch(v.counter + 2, 0u);
        __threadfence();
        atomicAdd(v.counter + 3, 1u);
      } else {
        const long long t0 = clock64();
        while (*gen == g0) {
          __nanosleep(64);  // back off: hundreds of CTAs poll the same line
          if (*abt) { ok = 0; break; }
          if (clock64() - t0 > limit) {
            atomicExch(v.counter + 4, 1u);
            if (v.tc_err) atomicExch(v.tc_err, 1);
            ok = 0;
            break;
          }
        }
      }
      __threadfence();
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

__global__ void __launch_bounds__(PT, 4) k_panel_persist(const __grid_constant__ CUtensorMap tm, TridiagView<float> v,
                                                      int p, int nbp, long long limit) {
  extern __shared__ __align__(1024) unsigned char pp_raw[];
  const uint32_t raw = (uint32_t)__cvta_generic_to_shared(pp_raw);
  const uint32_t tiles = (raw + 1023u) & ~1023u;
  __shared__ __align__(8) unsigned long long s_bar;
  __shared__ WHead<float> s_head;
  const uint32_t bar = (uint32_t)__cvta_generic_to_shared(&s_bar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  uint32_t par = 0;  // parity of the tile barrier's next phase
  const int n = v.n, G = (int)gridDim.x, cta = (int)blockIdx.x;
  int ncp = 0;
  for (int k = 0; k < nbp; ++k) {
    const int j = p + k, L = n - 1 - j;
    const int ncta1 = ceil_div(n - j, RB);
    for (int rb = cta; rb < ncta1; rb += G) colupd_block<float, PT>(v, p, j, k, ncp, 1, rb);
    if (!grid_barrier(v, limit)) return;
    if (L < 1) { ncp = 0; continue; }
    reflector_head_all(v, j, ncta1, &s_head, cta == 0);
    __syncthreads();
    const int b0 = (j + 1) & ~1, sh = (j + 1) - b0;
    const int nblk = ceil_div(n - b0, HT);
    if (L >= 2) {
      const int ndot = (k > 0) ? ceil_div(L, DR) : 0;
      const int items = ndot + nblk * (nblk + 1) / 2;
      for (int it = cta; it < items; it += G) {
        // the tile buffer was read by this CTA's threads (generic proxy) before
        // the copy of this item writes it (async proxy)
        if (threadIdx.x == 0) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        const bool ok = hemv_tma_item(&tm, v, p, j, k, ndot, b0, it, tiles, pp_raw + (tiles - raw), bar, par, &s_head);
        if (it >= ndot) par ^= 1u;
        __syncthreads();
        if (!ok) {
          if (threadIdx.x == 0) atomicExch(v.counter + 4, 1u);
          return;
        }
      }
      if (!grid_barrier(v, limit)) return;
    }
    const int nhr = ceil_div(L, HRB);
    for (int rb = cta; rb < nhr; rb += G)
      hreduce_block<float, PT>(v, p, j, k, HT, nblk, L < 2 ? 1 : 0, sh, rb, &s_head);
    if (!grid_barrier(v, limit)) return;
    ncp = nhr;
  }
}

// CTAs of the persistent panel kernel (0: use the per-column kernels). Only
// with ZQ_TRIDIAG=persist; the grid is every SM times min(occupancy,
// ZQ_PANEL_CTAS_PER_SM, default 4).
static int panel_persist_grid() {
  static int grid = -1;
  static std::once_flag once;
  std::call_once(once, [] {
    grid = 0;
    const char* m = getenv("ZQ_TRIDIAG");
    if (!m || strcmp(m, "persist")) return;
    int dev = 0, sms = 0, coop = 0, occ = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return;
    if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop) return;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return;
    if (cudaFuncSetAttribute(k_panel_persist, cudaFuncAttributeMaxDynamicSharedMemorySize, PT_SMEM) != cudaSuccess) return;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_panel_persist, PT, PT_SMEM) != cudaSuccess) return;
    int per = 4;
    if (const char* e = getenv("ZQ_PANEL_CTAS_PER_SM")) per = atoi(e);
    if (per > occ) per = occ;
    grid = per > 0 ? per * sms : 0;
  });
  return grid;
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
  ZQ_CUDA(cudaMemsetAsync(v.counter, 0, 5 * sizeof(unsigned), st));
  // FP32 with even n: the hemv tiles come by TMA from one tensor map over [A; B]
  // (2n x n, 8-byte elements, 16 x 32 boxes, 128-byte swizzle, zeros outside)
  bool use_tma = false;
  CUtensorMap hemv_map;
  if (std::is_same<R, float>::value && (n % 2) == 0 && n >= 4 && hemv_tma_enabled()) {
    using Enc = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*, const cuuint64_t*,
                             const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                             CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
    auto enc = reinterpret_cast<Enc>(tensor_map_encode_fn());
    const cuuint64_t dims[2] = {(cuuint64_t)2 * n, (cuuint64_t)n};
    const cuuint64_t strides[1] = {(cuuint64_t)v.ld * 8};
    const cuuint32_t box[2] = {16u, (cuuint32_t)HT};
    const cuuint32_t es[2] = {1u, 1u};
    use_tma = enc && (reinterpret_cast<uintptr_t>(v.M) % 16) == 0 && (v.ld % 2) == 0 &&
              enc(&hemv_map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, const_cast<void*>(reinterpret_cast<const void*>(v.M)),
                  dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
  }
  int ncp = 0;  // number of c partials of the previous column
  const int pgrid = (use_tma && v.coop) ? panel_persist_grid() : 0;
  for (int p = 0; p < n; p += nb) {
    const int nbp = (nb < n - p) ? nb : (n - p);
    if constexpr (std::is_same<R, float>::value) if (pgrid > 0) {
      // the panel's columns in one cooperative launch
      cudaLaunchConfig_t cfg{};
      cfg.gridDim = dim3((unsigned)pgrid);
      cfg.blockDim = dim3(PT);
      cfg.dynamicSmemBytes = PT_SMEM;
      cfg.stream = st;
      cudaLaunchAttribute attr[1];
      attr[0].id = cudaLaunchAttributeCooperative;
      attr[0].val.cooperative = 1;
      cfg.attrs = attr;
      cfg.numAttrs = 1;
      const long long limit = pipeline_wait_cycles();
      ZQ_CUDA(cudaLaunchKernelEx(&cfg, k_panel_persist, hemv_map, v, p, nbp, limit));
      count_launch();
      const int jl = p + nbp - 1, Ll = n - 1 - jl;
      ncp = Ll >= 1 ? ceil_div(Ll, HRB) : 0;
    }
    for (int k = 0; k < nbp && pgrid == 0; ++k) {
      const int j = p + k;
      const int L = n - 1 - j;
      const int ncta1 = ceil_div(n - j, RB);
      prof_begin(PC_PANEL, st);
      ZQ_CUDA(launch_pdl(k_colupd<R>, dim3(ncta1), dim3(NT), st, v, p, j, k, ncp, 1));
      count_launch();
      if (L < 1) { prof_end(PC_PANEL, st); ncp = 0; continue; }
      const int T = HT;
      // TMA-staged FP32 hemv: its tile grid starts at the even row below r0
      const int b0 = use_tma ? ((j + 1) & ~1) : (j + 1);
      const int sh = (j + 1) - b0;
      const int nblk = ceil_div(n - b0, T);
      const int ndot = (k > 0 && L >= 2) ? ceil_div(L, DR) : 0;  // dot-partial CTAs of the hemv grid
      prof_end(PC_PANEL, st);
      if (L >= 2) {
        prof_begin(PC_HEMV, st);
        const int ntiles = nblk * (nblk + 1) / 2;
        if constexpr (std::is_same<R, float>::value) {
          if (use_tma) {
            ZQ_CUDA(launch_pdl_smem(k_hemv_tma, dim3(ntiles + ndot), dim3(128), HM_SMEM, st, hemv_map, v, p, j, k, ndot, b0));
          } else {
            ZQ_CUDA(launch_pdl(k_hemv<R>, dim3(ntiles + ndot), dim3(128), st, v, p, j, k, ndot));
          }
        } else {
          ZQ_CUDA(launch_pdl(k_hemv<R>, dim3(ntiles + ndot), dim3(128), st, v, p, j, k, ndot));
        }
        count_launch();
        prof_end(PC_HEMV, st);
      }
      prof_begin(PC_PANEL, st);
      const int nhr = ceil_div(L, HRB);
      ZQ_CUDA(launch_pdl(k_hreduce<R>, dim3(nhr), dim3(NT), st, v, p, j, k, T, nblk, L < 2 ? 1 : 0, sh));
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
      if constexpr (std::is_same<R, float>::value) {
        if (v.tc_err && fp32_products_on_tensor_cores(TC_USE_TRAIL)) {
          if (int rc = trail_tc32(v, p, nbp, t0, st)) return rc;
          prof_end(PC_TRAIL, st);
          ncp = 0;
          continue;
        }
      }
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
  b += sizeof(double) * (2 * hblk + 16);              // npart (2 hblk), scal
  b += sizeof(double) * ((size_t)ceil_div(n > 0 ? n : 1, HRB) + 1);  // cpart (one per hreduce CTA)
  b += sizeof(unsigned) * 8;                          // counters (colupd, dots, grid barrier, abort)
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
  v.cpart = reinterpret_cast<double*>(take(sizeof(double) * ((size_t)ceil_div(n > 0 ? n : 1, HRB) + 1)));
  v.scal = reinterpret_cast<double*>(take(sizeof(double) * 16));
  v.counter = reinterpret_cast<unsigned*>(take(sizeof(unsigned) * 8));
  v.coop = 1;
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
