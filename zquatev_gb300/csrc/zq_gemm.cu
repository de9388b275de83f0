// Stage (b) GEMMs: FP64 complex (Gauss 3M) and real matrix products.
//
// The reference forms these products with zgemm3m (blocked.cc:424-543,
// zquatev.cc:87-90). On GB300 the FP64 tensor path (DMMA, mma.sync .f64) issues
// slower than plain DFMA (1.05 vs 1.19 TFLOP/s measured), so the FP64 products
// are register-tiled DFMA kernels: 64x64 output tile per CTA, 256 threads, a
// 4x4 micro-tile per thread, operands staged through shared memory.
//
// zgemm computes  C = alpha * (opA1(A1) opB1(B1) + s2 * opA2(A2) opB2(B2)) + beta * C
// with op in {N, T, C (conj-transpose), R (conj, no transpose)} chosen per
// operand at compile time; the complex products use the 3M (Gauss) scheme:
//   T1 = Ar Br, T2 = Ai Bi, T3 = (Ar + Ai)(Br + Bi); Re = T1 - T2, Im = T3 - T1 - T2,
// i.e. 3 real multiply-adds per complex multiply-add (the reference's zgemm3m).
//
// dgemm_grouped computes a list of independent real products
//   C_g = alpha_g op(A_g) op(B_g) + beta_g C_g
// in one launch (flat tile index over the group), used by the back-transform
// (G Z with complex G viewed as a real array of twice the rows) and by the
// divide-and-conquer merges.
#include "zq_common.cuh"
#include "zq_kernels.h"

#include <type_traits>

namespace zq {

constexpr int GT = 64;   // output tile edge
constexpr int GK = 8;    // k per stage (complex)
constexpr int GKR = 16;  // k per stage (real)
constexpr int GNT = 256;

template <int OP, typename Z>
__device__ __forceinline__ Z load_op(const Z* X, int64_t ldx, int r, int c) {
  // element (r, c) of op(X)
  if (OP == OP_N) return X[r + (int64_t)c * ldx];
  if (OP == OP_R) { Z v = X[r + (int64_t)c * ldx]; v.y = -v.y; return v; }
  if (OP == OP_T) return X[c + (int64_t)r * ldx];
  Z v = X[c + (int64_t)r * ldx]; v.y = -v.y; return v;  // OP_C
}

template <typename R, int OPA1, int OPB1, int OPA2, int OPB2>
__global__ void __launch_bounds__(GNT) k_zgemm(ZgemmArgsT<R> g) {
  using Z = cplx<R>;
  __shared__ R sA[3][GK][GT];
  __shared__ R sB[3][GK][GT];
  const int tid = threadIdx.x;
  const int tr = tid & 15, tc = tid >> 4;
  const int i0 = blockIdx.x * GT, j0 = blockIdx.y * GT;
  const int split = blockIdx.z;
  const Z* A1 = g.A1;
  const Z* B1 = g.B1;
  const Z* A2 = g.A2;
  const Z* B2 = g.B2;
  Z* C = g.C;
  R t1[4][4], t2[4][4], t3[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) { t1[a][b] = 0.0; t2[a][b] = 0.0; t3[a][b] = 0.0; }

  const int nseg = (A2 != nullptr) ? 2 : 1;
  for (int seg = 0; seg < nseg; ++seg) {
    const int K = seg == 0 ? g.k1 : g.k2;
    const R sgn = seg == 0 ? (R)1 : g.s2;
    // this split's share of the segment, in whole GK steps
    const int steps = (K + GK - 1) / GK;
    const int sb = (int)(((int64_t)steps * split) / gridDim.z), se = (int)(((int64_t)steps * (split + 1)) / gridDim.z);
    for (int k0 = sb * GK; k0 < se * GK; k0 += GK) {
      __syncthreads();
      for (int e = tid; e < GK * GT; e += GNT) {
        // A tile: 64 rows x GK; B tile: GK x 64 cols
        int r, kk;
        const bool a_kfast = (seg == 0 ? (OPA1 == OP_T || OPA1 == OP_C) : (OPA2 == OP_T || OPA2 == OP_C));
        if (a_kfast) { kk = e % GK; r = e / GK; } else { r = e % GT; kk = e / GT; }
        Z va = czero<Z>();
        if (i0 + r < g.m && k0 + kk < K) {
          va = seg == 0 ? load_op<OPA1>(A1, g.lda1, i0 + r, k0 + kk) : load_op<OPA2>(A2, g.lda2, i0 + r, k0 + kk);
          va.x *= sgn; va.y *= sgn;
        }
        sA[0][kk][r] = va.x; sA[1][kk][r] = va.y; sA[2][kk][r] = va.x + va.y;
        int c;
        const bool b_kfast = (seg == 0 ? (OPB1 == OP_N || OPB1 == OP_R) : (OPB2 == OP_N || OPB2 == OP_R));
        if (b_kfast) { kk = e % GK; c = e / GK; } else { c = e % GT; kk = e / GT; }
        Z vb = czero<Z>();
        if (j0 + c < g.n && k0 + kk < K)
          vb = seg == 0 ? load_op<OPB1>(B1, g.ldb1, k0 + kk, j0 + c) : load_op<OPB2>(B2, g.ldb2, k0 + kk, j0 + c);
        sB[0][kk][c] = vb.x; sB[1][kk][c] = vb.y; sB[2][kk][c] = vb.x + vb.y;
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < GK; ++kk) {
        R ar[4], ai[4], as[4], br[4], bi[4], bs[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          ar[q] = sA[0][kk][tr + 16 * q]; ai[q] = sA[1][kk][tr + 16 * q]; as[q] = sA[2][kk][tr + 16 * q];
          br[q] = sB[0][kk][tc + 16 * q]; bi[q] = sB[1][kk][tc + 16 * q]; bs[q] = sB[2][kk][tc + 16 * q];
        }
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = 0; b < 4; ++b) {
            t1[a][b] = fma(ar[a], br[b], t1[a][b]);
            t2[a][b] = fma(ai[a], bi[b], t2[a][b]);
            t3[a][b] = fma(as[a], bs[b], t3[a][b]);
          }
      }
    }
  }
  if (gridDim.z > 1) {
    // raw partial sums; k_zsplit_reduce applies alpha/beta
    Z* P = g.P + (int64_t)split * g.m * g.n;
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      const int i = i0 + tr + 16 * a;
      if (i >= g.m) continue;
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        const int j = j0 + tc + 16 * b;
        if (j >= g.n) continue;
        P[i + (int64_t)j * g.m] = mk(t1[a][b] - t2[a][b], t3[a][b] - t1[a][b] - t2[a][b]);
      }
    }
    return;
  }
  const Z al = g.alpha, be = g.beta;
  const bool use_beta = (be.x != (R)0 || be.y != (R)0);
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const int i = i0 + tr + 16 * a;
    if (i >= g.m) continue;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int j = j0 + tc + 16 * b;
      if (j >= g.n) continue;
      const R re = t1[a][b] - t2[a][b];
      const R im = t3[a][b] - t1[a][b] - t2[a][b];
      Z out = mk(al.x * re - al.y * im, al.x * im + al.y * re);
      const int64_t o = i + (int64_t)j * g.ldc;
      if (use_beta) {
        const Z c = C[o];
        out.x += be.x * c.x - be.y * c.y;
        out.y += be.x * c.y + be.y * c.x;
      }
      C[o] = out;
    }
  }
}

template <typename R>
__global__ void k_zsplit_reduce(ZgemmArgsT<R> g, int splits) {
  using Z = cplx<R>;
  const int64_t total = (int64_t)g.m * g.n;
  const bool use_beta = (g.beta.x != (R)0 || g.beta.y != (R)0);
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    R re = 0, im = 0;
    for (int s = 0; s < splits; ++s) {
      const Z p = g.P[t + (int64_t)s * total];
      re += p.x; im += p.y;
    }
    const int i = (int)(t % g.m), j = (int)(t / g.m);
    Z out = mk(g.alpha.x * re - g.alpha.y * im, g.alpha.x * im + g.alpha.y * re);
    const int64_t o = i + (int64_t)j * g.ldc;
    if (use_beta) {
      const Z c = g.C[o];
      out.x += g.beta.x * c.x - g.beta.y * c.y;
      out.y += g.beta.x * c.y + g.beta.y * c.x;
    }
    g.C[o] = out;
  }
}

// Split the K range over enough CTAs to fill the GPU when the output is small
// (e.g. the 64 x L products of the Q formation); partials go to g.P.
template <typename R>
static int choose_splits(const ZgemmArgsT<R>& g) {
  if (!g.P || g.pcap <= 0) return 1;
  const int tiles = ceil_div(g.m, GT) * ceil_div(g.n, GT);
  const int ksteps = ceil_div(g.k1, GK) + (g.A2 ? ceil_div(g.k2, GK) : 0);
  int s = 1;
  while (tiles * s < 2 * 152 && ksteps / (2 * s) >= 16 && (int64_t)(2 * s) * g.m * g.n <= g.pcap) s *= 2;
  return s;
}

// ----------------------------------------------------------------------------
// FP32 kernels (the refined path's decomposition). The DFMA-shaped kernels
// above leave FP32 bound by shared-memory loads (2 FMA per scalar load); these
// keep the same 64 x 64 output tiles but give each thread an 8 x 8 real or a
// 4 x 8 complex (4M: two accumulators per output) micro-tile read with 16-byte
// shared loads (4 and 5.3 FMA per loaded float), and double-buffer 16-deep K
// stages with cp.async (zero fill outside the matrix).
// ----------------------------------------------------------------------------
constexpr int SK = 16;       // k per stage
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem, bool pred) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(sa), "l"(gmem), "r"(pred ? 4 : 0) : "memory");
}
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem, bool pred) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(sa), "l"(gmem), "r"(pred ? 8 : 0) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// complex, 64 x 64 complex tile, 128 threads (16 x 8), thread (tr, tc) owns rows
// {2tr, 2tr+1, 32+2tr, 33+2tr} and columns {2tc, 2tc+1} + {0, 16, 32, 48}
constexpr int CNT = 128;
template <int OPA, int OPB>
__device__ __forceinline__ void cg_load(float2 (*sA)[GT], float2 (*sB)[GT], const float2* A, int64_t lda,
                                        const float2* B, int64_t ldb, int m, int n, int K, int i0, int j0, int k0) {
  const int tid = threadIdx.x;
#pragma unroll 2
  for (int u = 0; u < SK * GT / CNT; ++u) {
    const int e = tid + CNT * u;
    int r, kk;
    if (OPA == OP_T || OPA == OP_C) { kk = e % SK; r = e / SK; } else { r = e % GT; kk = e / GT; }
    const bool ok = (i0 + r < m) && (k0 + kk < K);
    const float2* src = A;
    if (ok) src = (OPA == OP_T || OPA == OP_C) ? A + (k0 + kk) + (int64_t)(i0 + r) * lda : A + (i0 + r) + (int64_t)(k0 + kk) * lda;
    cp_async8(&sA[kk][r], src, ok);
    int c;
    if (OPB == OP_N || OPB == OP_R) { kk = e % SK; c = e / SK; } else { c = e % GT; kk = e / GT; }
    const bool okb = (j0 + c < n) && (k0 + kk < K);
    const float2* srcb = B;
    if (okb) srcb = (OPB == OP_N || OPB == OP_R) ? B + (k0 + kk) + (int64_t)(j0 + c) * ldb : B + (j0 + c) + (int64_t)(k0 + kk) * ldb;
    cp_async8(&sB[kk][c], srcb, okb);
  }
  cp_commit();
}

template <int OPA, int OPB>
__device__ __forceinline__ void cg_segment(float (&re)[4][8], float (&im)[4][8], float2 (*sA)[SK][GT], float2 (*sB)[SK][GT],
                                           const float2* A, int64_t lda, const float2* B, int64_t ldb, int m, int n,
                                           int K, int i0, int j0, int sb, int se) {
  constexpr bool CA = (OPA == OP_C || OPA == OP_R), CB = (OPB == OP_C || OPB == OP_R);
  const int tr = threadIdx.x & 15, tc = threadIdx.x >> 4;
  if (sb >= se) return;
  cg_load<OPA, OPB>(sA[0], sB[0], A, lda, B, ldb, m, n, K, i0, j0, sb * SK);
  for (int s = sb; s < se; ++s) {
    const int buf = (s - sb) & 1;
    if (s + 1 < se) {
      cg_load<OPA, OPB>(sA[buf ^ 1], sB[buf ^ 1], A, lda, B, ldb, m, n, K, i0, j0, (s + 1) * SK);
      cp_wait<1>();
    } else {
      cp_wait<0>();
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < SK; ++kk) {
      float ar[4], ai[4], br[8], bi[8];
      const float4 a0 = *reinterpret_cast<const float4*>(&sA[buf][kk][2 * tr]);
      const float4 a1 = *reinterpret_cast<const float4*>(&sA[buf][kk][32 + 2 * tr]);
      ar[0] = a0.x; ai[0] = a0.y; ar[1] = a0.z; ai[1] = a0.w; ar[2] = a1.x; ai[2] = a1.y; ar[3] = a1.z; ai[3] = a1.w;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const float4 b = *reinterpret_cast<const float4*>(&sB[buf][kk][16 * q + 2 * tc]);
        br[2 * q] = b.x; bi[2 * q] = b.y; br[2 * q + 1] = b.z; bi[2 * q + 1] = b.w;
      }
#pragma unroll
      for (int x = 0; x < 4; ++x) {
        const float xr = ar[x], xi = CA ? -ai[x] : ai[x];
#pragma unroll
        for (int y = 0; y < 8; ++y) {
          const float yr = br[y], yi = CB ? -bi[y] : bi[y];
          re[x][y] = fmaf(xr, yr, re[x][y]);
          re[x][y] = fmaf(-xi, yi, re[x][y]);
          im[x][y] = fmaf(xr, yi, im[x][y]);
          im[x][y] = fmaf(xi, yr, im[x][y]);
        }
      }
    }
    __syncthreads();  // the next stage's copy overwrites this buffer
  }
}

template <int OPA1, int OPB1, int OPA2, int OPB2>
__global__ void __launch_bounds__(CNT) k_cgemm32(ZgemmArgsT<float> g) {
  __shared__ __align__(16) float2 sA[2][SK][GT];
  __shared__ __align__(16) float2 sB[2][SK][GT];
  const int tr = threadIdx.x & 15, tc = threadIdx.x >> 4;
  const int i0 = blockIdx.x * GT, j0 = blockIdx.y * GT;
  const int split = blockIdx.z;
  float re[4][8], im[4][8];
#pragma unroll
  for (int x = 0; x < 4; ++x)
#pragma unroll
    for (int y = 0; y < 8; ++y) { re[x][y] = 0.f; im[x][y] = 0.f; }
  {
    const int steps = ceil_div(g.k1, SK);
    const int sb = (int)(((int64_t)steps * split) / gridDim.z), se = (int)(((int64_t)steps * (split + 1)) / gridDim.z);
    cg_segment<OPA1, OPB1>(re, im, sA, sB, g.A1, g.lda1, g.B1, g.ldb1, g.m, g.n, g.k1, i0, j0, sb, se);
  }
  if (g.A2 != nullptr) {
    // s2 = +-1: the second product is added (or subtracted, between two negations)
    const bool neg = g.s2 < 0.f;
    if (neg)
#pragma unroll
      for (int x = 0; x < 4; ++x)
#pragma unroll
        for (int y = 0; y < 8; ++y) { re[x][y] = -re[x][y]; im[x][y] = -im[x][y]; }
    const int steps = ceil_div(g.k2, SK);
    const int sb = (int)(((int64_t)steps * split) / gridDim.z), se = (int)(((int64_t)steps * (split + 1)) / gridDim.z);
    cg_segment<OPA2, OPB2>(re, im, sA, sB, g.A2, g.lda2, g.B2, g.ldb2, g.m, g.n, g.k2, i0, j0, sb, se);
    if (neg)
#pragma unroll
      for (int x = 0; x < 4; ++x)
#pragma unroll
        for (int y = 0; y < 8; ++y) { re[x][y] = -re[x][y]; im[x][y] = -im[x][y]; }
  }
  const bool partial = gridDim.z > 1;
  const float2 al = g.alpha, be = g.beta;
  const bool use_beta = (be.x != 0.f || be.y != 0.f);
#pragma unroll
  for (int x = 0; x < 4; ++x) {
    const int i = i0 + ((x < 2) ? 2 * tr + x : 32 + 2 * tr + (x - 2));
    if (i >= g.m) continue;
#pragma unroll
    for (int y = 0; y < 8; ++y) {
      const int j = j0 + 16 * (y >> 1) + 2 * tc + (y & 1);
      if (j >= g.n) continue;
      if (partial) {  // raw partial sums; k_zsplit_reduce applies alpha/beta
        g.P[(int64_t)split * g.m * g.n + i + (int64_t)j * g.m] = make_float2(re[x][y], im[x][y]);
        continue;
      }
      float2 out = make_float2(al.x * re[x][y] - al.y * im[x][y], al.x * im[x][y] + al.y * re[x][y]);
      const int64_t o = i + (int64_t)j * g.ldc;
      if (use_beta) {
        const float2 c = g.C[o];
        out.x += be.x * c.x - be.y * c.y;
        out.y += be.x * c.y + be.y * c.x;
      }
      g.C[o] = out;
    }
  }
}

// real grouped, 64 x 64 tile, 64 threads (8 x 8), thread (tr, tc) owns rows
// {4tr..4tr+3, 32+4tr..} and the same pattern of columns
constexpr int RNT = 64;
__global__ void __launch_bounds__(RNT) k_sgemm_grouped(const DgemmDescT<float>* __restrict__ descs, int count) {
  __shared__ __align__(16) float sA[2][SK][GT];
  __shared__ __align__(16) float sB[2][SK][GT];
  const int t = blockIdx.x;
  int gi = 0;
  {
    int lo = 0, hi = count - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (descs[mid].tile0 <= t) lo = mid; else hi = mid - 1;
    }
    gi = lo;
  }
  const DgemmDescT<float> d = descs[gi];
  const int local = t - d.tile0;
  const int mt = (d.m + GT - 1) / GT;
  const int i0 = (local % mt) * GT, j0 = (local / mt) * GT;
  const int tid = threadIdx.x;
  const int tr = tid & 7, tc = tid >> 3;
  float acc[8][8];
#pragma unroll
  for (int x = 0; x < 8; ++x)
#pragma unroll
    for (int y = 0; y < 8; ++y) acc[x][y] = 0.f;
  // Copy u of this thread (u < 16): with e = tid + 64 u the element is
  // (row tid, k u) of a row-fast operand or (row tid/16 + 4u, k tid%16) of a
  // k-fast one, so address, bounds and shared offset are per-thread constants
  // plus u times a step, computed once per tile.
  const int lo = tid % SK, hi = tid / SK;
  // A: rows i0.., k; ta: k-fast
  const int a_r0 = d.ta ? hi : tid, a_rs = d.ta ? 4 : 0, a_k0 = d.ta ? lo : 0, a_ks = d.ta ? 0 : 1;
  const float* a_base = d.A + (d.ta ? (a_k0 + (int64_t)(i0 + a_r0) * d.lda) : ((i0 + a_r0) + (int64_t)a_k0 * d.lda));
  const int64_t a_kstep = d.ta ? 1 : d.lda, a_ustep = d.ta ? 4 * d.lda : d.lda;
  // B: columns j0.., k; !tb: k-fast
  const int b_c0 = d.tb ? tid : hi, b_cs = d.tb ? 0 : 4, b_k0 = d.tb ? 0 : lo, b_ks = d.tb ? 1 : 0;
  const float* b_base = d.B + (d.tb ? ((j0 + b_c0) + (int64_t)b_k0 * d.ldb) : (b_k0 + (int64_t)(j0 + b_c0) * d.ldb));
  const int64_t b_kstep = d.tb ? d.ldb : 1, b_ustep = d.tb ? d.ldb : 4 * d.ldb;
  auto load = [&](int s, int buf) {
    const int k0 = s * SK;
    const float* pa = a_base + (int64_t)k0 * a_kstep;
    const float* pb = b_base + (int64_t)k0 * b_kstep;
    int ar = a_r0, ak = a_k0 + k0, bc = b_c0, bk = b_k0 + k0;
    float* da = &sA[buf][a_k0][a_r0];
    float* db = &sB[buf][b_k0][b_c0];
#pragma unroll 2
    for (int u = 0; u < SK * GT / RNT; ++u) {
      const bool ok = (i0 + ar < d.m) && (ak < d.k);
      cp_async4(da, ok ? pa : d.A, ok);
      const bool okb = (j0 + bc < d.n) && (bk < d.k);
      cp_async4(db, okb ? pb : d.B, okb);
      pa += a_ustep; ar += a_rs; ak += a_ks; da += a_ks * GT + a_rs;
      pb += b_ustep; bc += b_cs; bk += b_ks; db += b_ks * GT + b_cs;
    }
    cp_commit();
  };
  const int nst = ceil_div(d.k, SK);
  if (nst > 0) load(0, 0);
  for (int s = 0; s < nst; ++s) {
    const int buf = s & 1;
    if (s + 1 < nst) { load(s + 1, buf ^ 1); cp_wait<1>(); } else { cp_wait<0>(); }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < SK; ++kk) {
      const float4 a0 = *reinterpret_cast<const float4*>(&sA[buf][kk][4 * tr]);
      const float4 a1 = *reinterpret_cast<const float4*>(&sA[buf][kk][32 + 4 * tr]);
      const float4 b0 = *reinterpret_cast<const float4*>(&sB[buf][kk][4 * tc]);
      const float4 b1 = *reinterpret_cast<const float4*>(&sB[buf][kk][32 + 4 * tc]);
      const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      const float b[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
      for (int x = 0; x < 8; ++x)
#pragma unroll
        for (int y = 0; y < 8; ++y) acc[x][y] = fmaf(a[x], b[y], acc[x][y]);
    }
    __syncthreads();  // the next stage's copy overwrites this buffer
  }
#pragma unroll
  for (int x = 0; x < 8; ++x) {
    const int i = i0 + ((x < 4) ? 4 * tr + x : 32 + 4 * tr + (x - 4));
    if (i >= d.m) continue;
#pragma unroll
    for (int y = 0; y < 8; ++y) {
      const int j = j0 + ((y < 4) ? 4 * tc + y : 32 + 4 * tc + (y - 4));
      if (j >= d.n) continue;
      const int64_t o = i + (int64_t)j * d.ldc;
      float out = d.alpha * acc[x][y];
      if (d.beta != 0.f) out += d.beta * d.C[o];
      d.C[o] = out;
    }
  }
}

template <typename R, int OPA1, int OPB1, int OPA2, int OPB2>
int zgemm_launch(const ZgemmArgsT<R>& g, int batch, cudaStream_t st) {
  if (g.m <= 0 || g.n <= 0) return ZQ_OK;
  (void)batch;
  const int splits = choose_splits(g);
  dim3 grid(ceil_div(g.m, GT), ceil_div(g.n, GT), splits);
  prof_begin(PC_FORMQ_GEMM, st);
  if constexpr (std::is_same<R, float>::value) {
    if (g.A2 == nullptr || g.s2 == 1.f || g.s2 == -1.f)
      k_cgemm32<OPA1, OPB1, OPA2, OPB2><<<grid, CNT, 0, st>>>(g);
    else
      k_zgemm<R, OPA1, OPB1, OPA2, OPB2><<<grid, GNT, 0, st>>>(g);
  } else {
    k_zgemm<R, OPA1, OPB1, OPA2, OPB2><<<grid, GNT, 0, st>>>(g);
  }
  prof_end(PC_FORMQ_GEMM, st);
  ZQ_LAUNCH_CHECK();
  if (splits > 1) {
    const int64_t total = (int64_t)g.m * g.n;
    const int blocks = (int)((total + 255) / 256 > 4096 ? 4096 : (total + 255) / 256);
    k_zsplit_reduce<R><<<blocks, 256, 0, st>>>(g, splits);
    ZQ_LAUNCH_CHECK();
  }
  return ZQ_OK;
}

template <typename R>
int zgemm(int opa1, int opb1, int opa2, int opb2, const ZgemmArgsT<R>& g, int batch, cudaStream_t st) {
#define ZQ_Z(a, b, c, d) \
  if (opa1 == a && opb1 == b && opa2 == c && opb2 == d) return zgemm_launch<R, a, b, c, d>(g, batch, st);
  // the combinations used by the solver
  ZQ_Z(OP_C, OP_N, OP_C, OP_N)   // Wa^H Xa + Wb^H Xb
  ZQ_Z(OP_T, OP_N, OP_T, OP_N)   // Wa^T Xb - Wb^T Xa
  ZQ_Z(OP_N, OP_N, OP_R, OP_N)   // Wa C - conj(Wb) D
  ZQ_Z(OP_N, OP_N, OP_N, OP_N)
  ZQ_Z(OP_C, OP_N, OP_N, OP_N)
  ZQ_Z(OP_N, OP_C, OP_N, OP_N)
  ZQ_Z(OP_T, OP_N, OP_N, OP_N)
  ZQ_Z(OP_N, OP_R, OP_N, OP_N)   // A conj(B)
#undef ZQ_Z
  return ZQ_ERR_ARG;
}
template int zgemm<double>(int, int, int, int, const ZgemmArgsT<double>&, int, cudaStream_t);
template int zgemm<float>(int, int, int, int, const ZgemmArgsT<float>&, int, cudaStream_t);

// ----------------------------------------------------------------------------
// real grouped GEMM
// ----------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(GNT) k_dgemm_grouped(const DgemmDescT<R>* __restrict__ descs, int count) {
  __shared__ R sA[GKR][GT];
  __shared__ R sB[GKR][GT + 1];
  // locate descriptor (linear search over prefix offsets; count is small)
  const int t = blockIdx.x;
  int gi = 0;
  {
    int lo = 0, hi = count - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (descs[mid].tile0 <= t) lo = mid; else hi = mid - 1;
    }
    gi = lo;
  }
  const DgemmDescT<R> d = descs[gi];
  const int local = t - d.tile0;
  const int mt = (d.m + GT - 1) / GT;
  const int i0 = (local % mt) * GT, j0 = (local / mt) * GT;
  const int tid = threadIdx.x;
  const int tr = tid & 15, tc = tid >> 4;
  R acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = 0;
  for (int k0 = 0; k0 < d.k; k0 += GKR) {
    __syncthreads();
    for (int e = tid; e < GKR * GT; e += GNT) {
      int r, kk;
      if (d.ta) { kk = e % GKR; r = e / GKR; } else { r = e % GT; kk = e / GT; }
      R va = 0;
      if (i0 + r < d.m && k0 + kk < d.k)
        va = d.ta ? d.A[(k0 + kk) + (int64_t)(i0 + r) * d.lda] : d.A[(i0 + r) + (int64_t)(k0 + kk) * d.lda];
      sA[kk][r] = va;
      int c;
      if (!d.tb) { kk = e % GKR; c = e / GKR; } else { c = e % GT; kk = e / GT; }
      R vb = 0;
      if (j0 + c < d.n && k0 + kk < d.k)
        vb = d.tb ? d.B[(j0 + c) + (int64_t)(k0 + kk) * d.ldb] : d.B[(k0 + kk) + (int64_t)(j0 + c) * d.ldb];
      sB[kk][c] = vb;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GKR; ++kk) {
      R a[4], b[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) { a[q] = sA[kk][tr + 16 * q]; b[q] = sB[kk][tc + 16 * q]; }
#pragma unroll
      for (int x = 0; x < 4; ++x)
#pragma unroll
        for (int y = 0; y < 4; ++y) acc[x][y] = fma(a[x], b[y], acc[x][y]);
    }
  }
#pragma unroll
  for (int x = 0; x < 4; ++x) {
    const int i = i0 + tr + 16 * x;
    if (i >= d.m) continue;
#pragma unroll
    for (int y = 0; y < 4; ++y) {
      const int j = j0 + tc + 16 * y;
      if (j >= d.n) continue;
      const int64_t o = i + (int64_t)j * d.ldc;
      R out = d.alpha * acc[x][y];
      if (d.beta != (R)0) out += d.beta * d.C[o];
      d.C[o] = out;
    }
  }
}

template <typename R>
void grouped_launch(const DgemmDescT<R>* dev_descs, int count, int tiles, cudaStream_t st) {
  if (tiles <= 0 || count <= 0) return;
  if constexpr (std::is_same<R, float>::value)
    k_sgemm_grouped<<<tiles, RNT, 0, st>>>(dev_descs, count);
  else
    k_dgemm_grouped<R><<<tiles, GNT, 0, st>>>(dev_descs, count);
}
template void grouped_launch<double>(const DgemmDescT<double>*, int, int, cudaStream_t);
template void grouped_launch<float>(const DgemmDescT<float>*, int, int, cudaStream_t);

int dgemm_tiles(int m, int n) { return ceil_div(m, GT) * ceil_div(n, GT); }

template <typename R>
int dgemm_grouped(DgemmDescT<R>* host_descs, int count, DgemmDescT<R>* dev_descs, cudaStream_t st) {
  int tiles = 0;
  int used = 0;
  for (int i = 0; i < count; ++i) {
    DgemmDescT<R>& d = host_descs[i];
    if (d.m <= 0 || d.n <= 0) continue;
    d.tile0 = tiles;
    tiles += ceil_div(d.m, GT) * ceil_div(d.n, GT);
    host_descs[used++] = d;
  }
  if (used == 0) return ZQ_OK;
  ZQ_CUDA(cudaMemcpyAsync(dev_descs, host_descs, sizeof(DgemmDescT<R>) * used, cudaMemcpyHostToDevice, st));
  grouped_launch<R>(dev_descs, used, tiles, st);
  ZQ_LAUNCH_CHECK();
  return ZQ_OK;
}
template int dgemm_grouped<double>(DgemmDescT<double>*, int, DgemmDescT<double>*, cudaStream_t);
template int dgemm_grouped<float>(DgemmDescT<float>*, int, DgemmDescT<float>*, cudaStream_t);

}  // namespace zq
