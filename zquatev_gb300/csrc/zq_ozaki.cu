// FP64-accurate complex matrix products on the bf16 tensor cores (Ozaki
// scheme I, error-free slicing), used by the refinement products G = X^H X,
// H X and S = X^H (H X) of zq_refine.cu.
//
// Scheme (Ozaki, Ogita, Oishi & Rump, Numer. Algorithms 59 (2012) 95-118;
// the bf16 / FP32-accumulate variant with exact chunked accumulation):
//   * the complex product C = op(A1) op(B1) + s2 op(A2) op(B2) is written as two
//     real products with the K dimension concatenated:
//       Re C = Ahat . Bre,  Im C = Ahat . Bim,
//       Ahat = [ar1 | ai1 | s2 ar2 | s2 ai2],  Bre = [br1 | -bi1 | br2 | -bi2],
//       Bim  = [bi1 | br1 | bi2 | br2];
//   * every row of Ahat is scaled by a power of two sigma_i >= its max |entry|
//     (every column of B by tau_j) and cut into S slices of BETA = 7 bits:
//     integers in [-128, 128], exact in bf16;
//   * slice products are integers <= 2^14; FP32 accumulation of up to 256 of
//     them is exact (< 2^22), so the tensor-core accumulator is emptied into an
//     int32 accumulator every 256 terms (exact), and each (level, super-chunk)
//     writes its int32 result; level l = t + u collects the slice pairs (t, u)
//     with t + u = l, l < S (the triangular truncation);
//   * at the end of each (level, super-chunk) the owning CTA adds
//     sigma_i tau_j 2^(-BETA (l + 2)) I into the FP64 output.
// With S = 7 the dropped terms are below 2^-49 of sigma_i tau_j per product,
// i.e. FP64-level accuracy for the refinement's sums.
//
// Two product kernels with the same arithmetic: k_oz_umma (zq_ozaki_umma.cu,
// tcgen05 MMAs into TMEM fed by TMA; the default) and k_oz_gemm below, a bf16
// mma.sync (m16n8k16) tiled GEMM: 64x64 CTA tile, four 32x32 warp tiles
// computing the real and imaginary outputs from one staged A tile and two B
// tiles, cp.async double buffering.
#include "zq_common.cuh"
#include "zq_kernels.h"

#include <atomic>
#include <cstdlib>
#include <cstring>
#include <cuda_bf16.h>
#include <vector>

namespace zq {

constexpr int OZ_BETA = 7;
constexpr int OZ_SMAX = 8;              // most slices per operand (56 bits)
constexpr int OZ_CHUNK = 256;            // exact FP32 accumulation length
constexpr int OZ_SUPER = 64 * 1024;      // terms per int32 partial (64 * 1024 * 2^14 < 2^31)
constexpr int OZ_TM = 64, OZ_TN = 64, OZ_TK = 64;
constexpr int OZ_LDS = OZ_TK + 8;        // padded shared row (bf16), 144 bytes
constexpr int OZ_THREADS = 128;
constexpr int OZ_PAD = 128;             // slice rows padded for either product kernel

// element (r, c) of op(X)
__device__ __forceinline__ double2 oz_op(const double2* X, int64_t ld, int op, int r, int c) {
  double2 v;
  if (op == OP_N || op == OP_R) v = X[r + (int64_t)c * ld];
  else v = X[c + (int64_t)r * ld];
  if (op == OP_R || op == OP_C) v.y = -v.y;
  return v;
}

struct OzSide {
  const double2* X1; int64_t ld1; int op1; int K1;
  const double2* X2; int64_t ld2; int op2; int K2;
  double s2;
};

// value of Ahat[i][k'] (rows of op(A)) or of Bre/Bim[j][k'] (columns of op(B))
__device__ __forceinline__ void oz_entry(const OzSide& s, bool is_a, int idx, int kp, double& v_re_form, double& v_im_form) {
  int seg = 0, k = kp;
  if (k >= 2 * s.K1) { seg = 1; k -= 2 * s.K1; }
  const int K = seg ? s.K2 : s.K1;
  if (k >= 2 * K) { v_re_form = 0.0; v_im_form = 0.0; return; }  // padding
  const bool imag_half = k >= K;
  const int kk = imag_half ? k - K : k;
  double2 x;
  if (is_a) x = seg ? oz_op(s.X2, s.ld2, s.op2, idx, kk) : oz_op(s.X1, s.ld1, s.op1, idx, kk);
  else x = seg ? oz_op(s.X2, s.ld2, s.op2, kk, idx) : oz_op(s.X1, s.ld1, s.op1, kk, idx);
  if (is_a) {
    const double sg = seg ? s.s2 : 1.0;
    v_re_form = sg * (imag_half ? x.y : x.x);
    v_im_form = v_re_form;
  } else {
    v_re_form = imag_half ? -x.y : x.x;  // Bre = [br | -bi]
    v_im_form = imag_half ? x.x : x.y;   // Bim = [bi | br]
  }
}

// exponent e with 2^e >= max |entry| of row/column idx (e = -1100 for a zero row)
__global__ void k_oz_exp(OzSide s, bool is_a, int count, int parts, int* __restrict__ exps) {
  // The entries of row/column idx over k' are Re x and Im x of each complex x
  // of the row (times s2 in A's second segment), so the maximum is taken over
  // max(|Re x|, |Im x|) with eight loads in flight per lane. One warp per
  // (row/column, part): part p takes the chunks p, p + parts, ... of 256
  // entries of each segment, so that enough warps are resident to cover the
  // load latency. The frexp exponent is monotone in the value, so the largest
  // part exponent (atomicMax into exps, preset to -1100: a zero row) is the
  // exponent of the maximum.
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (gw >= count * parts) return;
  const int warp = gw / parts, part = gw - warp * parts;
  double mx = 0.0;
  const int nseg = (s.X2 != nullptr && s.K2 > 0) ? 2 : 1;
  for (int seg = 0; seg < nseg; ++seg) {
    const double2* X = seg ? s.X2 : s.X1;
    const int64_t ld = seg ? s.ld2 : s.ld1;
    const int op = seg ? s.op2 : s.op1;
    const int K = seg ? s.K2 : s.K1;
    unsigned long long m2 = 0;  // max |entry| as bits (sign cleared): same order as the values
    if (K <= 0) continue;
    // element (idx, k) of op(X) (A) or (k, idx) (B) lies at X[a + k * sk]: one
    // branch-free address per load, so the eight loads are in flight together
    // (loads past K read element K - 1 and are masked)
    const bool colmaj = (op == OP_N || op == OP_R);  // op(X)(r, c) = X[r + c ld]
    const int64_t sk = (is_a == colmaj) ? ld : 1;    // stride along k
    const int64_t a = (is_a == colmaj) ? (int64_t)warp : (int64_t)warp * ld;
    for (int k0 = part * 256; k0 < K; k0 += parts * 256) {
      double2 x[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int k = k0 + lane + 32 * u;
        x[u] = __ldg(X + a + (int64_t)(k < K ? k : K - 1) * sk);
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const bool in = k0 + lane + 32 * u < K;
        m2 = max(m2, in ? absmax_bits(x[u]) : 0ull);
      }
    }
    // rounding is monotone: max |s2 x| = |s2| max |x| exactly
    const double m2d = bits_to_double(m2);
    mx = fmax(mx, (is_a && seg) ? fabs(s.s2) * m2d : m2d);
  }
  mx = warp_max(mx);
  if (lane == 0 && mx > 0.0) {
    int ex;
    frexp(mx, &ex);  // mx = f 2^ex, f in [0.5, 1): 2^ex > mx
    atomicMax(exps + warp, ex);
  }
}

// bf16 pair from its bit pattern (low half: first element)
__device__ __forceinline__ __nv_bfloat162 oz_bf2(unsigned u) {
  __nv_bfloat162 r;
  *reinterpret_cast<unsigned*>(&r) = u;
  return r;
}
// sign factors of a digit pair: (s0, s1) = (+-1, +-1) and (-128 s0, -128 s1)
__device__ __forceinline__ void oz_sign_pair(bool neg0, bool neg1, __nv_bfloat162& sg, __nv_bfloat162& off) {
  sg = oz_bf2((neg0 ? 0xBF80u : 0x3F80u) | ((neg1 ? 0xBF80u : 0x3F80u) << 16));
  off = oz_bf2((neg0 ? 0x4300u : 0xC300u) | ((neg1 ? 0x4300u : 0xC300u) << 16));
}
// bf16 bits of the signed digits (s0 d0, s1 d1), d in [0, 127], without a
// conversion instruction: the bit pattern 0x4300 | d is the bf16 value 128 + d
// (exponent 2^7, mantissa d), and one bf16x2 FMA gives s (128 + d) - 128 s =
// s d exactly (a zero digit gives +0)
__device__ __forceinline__ unsigned oz_digit_pair(unsigned d0, unsigned d1, __nv_bfloat162 sg, __nv_bfloat162 off) {
  const __nv_bfloat162 r = __hfma2(oz_bf2(0x43004300u | d0 | (d1 << 16)), sg, off);
  return *reinterpret_cast<const unsigned*>(&r);
}

// base-128 digits of floor(|v| / 2^e * 2^(7 S)) (integer arithmetic on the
// 53-bit significand: exact truncation), most significant first, and the sign
__device__ __forceinline__ unsigned long long oz_fixed(double v, int e, int F, bool& neg) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
  neg = (bits >> 63) != 0;
  const int ex = (int)((bits >> 52) & 0x7ff);
  unsigned long long mant = bits & ((1ull << 52) - 1);
  int ebits = ex;
  if (ex == 0) ebits = 1; else mant |= (1ull << 52);
  // |v| = mant * 2^(ebits - 1075);  V = floor(|v| 2^(F - e))
  const int sh = ebits - 1075 - e + F;
  if (mant == 0 || e < -1000) return 0;
  if (sh >= 0) return (sh >= 64) ? 0 : (mant << sh);
  return (-sh >= 64) ? 0 : (mant >> (-sh));
}

// S slices of one operand: out[t][idx][kp] (bf16), idx < padded count (zero rows above count).
// The slices are the base-128 digits of floor(|v| / 2^e * 2^(7 S)) (integer
// arithmetic on the 53-bit significand), with the sign of v: exact truncation.
__global__ void __launch_bounds__(256, 4)
    k_oz_slice(OzSide s, bool is_a, int count, int count_pad, int Kp, const int* __restrict__ exps, int nsl,
               __nv_bfloat16* __restrict__ out_re, __nv_bfloat16* __restrict__ out_im, int64_t slice_stride) {
  // eight consecutive k' of one row per thread (Kp is a multiple of 64), each
  // slice written as one 16-byte store
  const int64_t total8 = (int64_t)count_pad * Kp / 8;
  const int F = OZ_BETA * nsl;
  for (int64_t t8 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t8 < total8; t8 += (int64_t)gridDim.x * blockDim.x) {
    const int64_t t = t8 * 8;
    const int idx = (int)(t / Kp), kp0 = (int)(t % Kp);
    const bool live = idx < count;
    const int e = live ? exps[idx] : 0;
    double va[8], vb[8];
    // the eight k' lie in one half (Re or Im part) of one segment in all but
    // the groups that straddle a boundary or the padding: there the eight
    // loads use one base and one stride and are issued together
    int seg = 0, k = kp0;
    if (k >= 2 * s.K1) { seg = 1; k -= 2 * s.K1; }
    const int K = seg ? s.K2 : s.K1;
    const bool imag_half = k >= K;
    const int kk0 = imag_half ? k - K : k;
    if (live && kk0 + 7 < K) {
      const double2* X = seg ? s.X2 : s.X1;
      const int64_t ld = seg ? s.ld2 : s.ld1;
      const int op = seg ? s.op2 : s.op1;
      const bool colmaj = (op == OP_N || op == OP_R);
      const int64_t sk = (is_a == colmaj) ? ld : 1;
      const double2* p = X + ((is_a == colmaj) ? (int64_t)idx : (int64_t)idx * ld) + (int64_t)kk0 * sk;
      const double cs = (op == OP_R || op == OP_C) ? -1.0 : 1.0;  // sign of the imaginary part of op(X)
      double2 x[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) x[u] = __ldg(p + u * sk);
      if (is_a) {
        const double sg = seg ? s.s2 : 1.0;
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          va[u] = imag_half ? (sg * cs) * x[u].y : sg * x[u].x;
          vb[u] = 0.0;
        }
      } else {
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const double y = cs * x[u].y;
          va[u] = imag_half ? -y : x[u].x;  // Bre = [br | -bi]
          vb[u] = imag_half ? x[u].x : y;   // Bim = [bi | br]
        }
      }
    } else {
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        va[u] = 0.0;
        vb[u] = 0.0;
        if (live) oz_entry(s, is_a, idx, kp0 + u, va[u], vb[u]);
      }
    }
    unsigned long long V0[8], V1[8];
    unsigned n0 = 0, n1 = 0;  // sign bits
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      bool ng0, ng1;
      V0[u] = oz_fixed(va[u], e, F, ng0);
      V1[u] = oz_fixed(vb[u], e, F, ng1);
      n0 |= (unsigned)ng0 << u;
      n1 |= (unsigned)ng1 << u;
    }
    __nv_bfloat162 sg0[4], of0[4], sg1[4], of1[4];
#pragma unroll
    for (int h = 0; h < 4; ++h) {
      oz_sign_pair((n0 >> (2 * h)) & 1, (n0 >> (2 * h + 1)) & 1, sg0[h], of0[h]);
      oz_sign_pair((n1 >> (2 * h)) & 1, (n1 >> (2 * h + 1)) & 1, sg1[h], of1[h]);
    }
    for (int q = 0; q < nsl; ++q) {
      const int shift = F - OZ_BETA * (q + 1);
      unsigned pr[4], pi[4];
#pragma unroll
      for (int h = 0; h < 4; ++h) {
        pr[h] = oz_digit_pair((unsigned)(V0[2 * h] >> shift) & 127u, (unsigned)(V0[2 * h + 1] >> shift) & 127u, sg0[h],
                              of0[h]);
        pi[h] = oz_digit_pair((unsigned)(V1[2 * h] >> shift) & 127u, (unsigned)(V1[2 * h + 1] >> shift) & 127u, sg1[h],
                              of1[h]);
      }
      *reinterpret_cast<uint4*>(out_re + q * slice_stride + t) = make_uint4(pr[0], pr[1], pr[2], pr[3]);
      if (out_im) *reinterpret_cast<uint4*>(out_im + q * slice_stride + t) = make_uint4(pi[0], pi[1], pi[2], pi[3]);
    }
  }
}

// Column-major A operands (op N or R: a row of op(A) is strided in memory):
// the exponent pass and the slicing read 32 consecutive rows per warp.
__global__ void k_oz_exp_init(int* __restrict__ exps, int count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) exps[i] = -1100;
}
// block (32, 8): 32 rows x 256 K terms; the per-row maximum exponent via atomicMax (order-free)
__global__ void k_oz_exp_cm(OzSide s, int count, int Kc, int* __restrict__ exps) {
  // rows of a column-major op(A) (OP_N / OP_R): 32 rows x 256 complex columns
  // per CTA, rows on the lanes (coalesced); the maximum of max(|Re x|, |Im x|)
  // (times |s2| in the second segment) over each complex column once, eight
  // loads in flight per thread; its exponent equals the largest digit
  // exponent of the row's entries (frexp is monotone in |a|)
  __shared__ double s_m[8][32];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int row = blockIdx.x * 32 + tx;
  const int kb = blockIdx.y * 256;
  double mx = 0.0;
  if (row < count) {
    // this CTA's columns [kb, kb + 256) of each segment: X[row + k ld], one
    // base and stride per segment, eight loads in flight per thread (loads
    // past the range read its last column and are masked)
    for (int seg = 0; seg < 2; ++seg) {
      const double2* X = seg ? s.X2 : s.X1;
      const int K = seg ? s.K2 : s.K1;
      const int koff = seg ? s.K1 : 0;
      const int lo = max(kb, koff) - koff, hi = min(min(kb + 256, Kc), koff + K) - koff;
      if (X == nullptr || lo >= hi) continue;
      const int64_t ld = seg ? s.ld2 : s.ld1;
      const double2* p = X + row;
      unsigned long long m2 = 0;
      for (int q0 = lo + ty; q0 < hi; q0 += 8 * 8) {
        double2 x[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) x[u] = __ldg(p + (int64_t)min(q0 + 8 * u, hi - 1) * ld);
#pragma unroll
        for (int u = 0; u < 8; ++u) m2 = max(m2, q0 + 8 * u < hi ? absmax_bits(x[u]) : 0ull);
      }
      // rounding is monotone: max |s2 x| = |s2| max |x| exactly
      const double m2d = bits_to_double(m2);
      mx = fmax(mx, seg ? fabs(s.s2) * m2d : m2d);
    }
  }
  s_m[ty][tx] = mx;
  __syncthreads();
  if (ty == 0 && row < count) {
    double m = s_m[0][tx];
    for (int r = 1; r < 8; ++r) m = fmax(m, s_m[r][tx]);
    if (m > 0.0) {
      int ex;
      frexp(m, &ex);  // 2^ex > m
      atomicMax(exps + row, ex);
    }
  }
}
// block (32, 8): a 32-row x 32-K tile, digits staged in shared memory, stored along K
__global__ void k_oz_slice_cm(OzSide s, int count, int Kp, const int* __restrict__ exps, int nsl,
                              __nv_bfloat16* __restrict__ out, int64_t slice_stride) {
  __shared__ __nv_bfloat16 s_d[OZ_SMAX][32][33];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int i0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  const int F = OZ_BETA * nsl;
  const int row = i0 + tx;
  const int e = row < count ? exps[row] : 0;
  for (int kk = ty; kk < 32; kk += 8) {
    const int kp = k0 + kk;
    double v = 0.0, dummy;
    if (row < count && kp < Kp) oz_entry(s, true, row, kp, v, dummy);
    bool neg;
    const unsigned long long V = oz_fixed(v, e, F, neg);
    for (int q = 0; q < nsl; ++q) {
      const int d = (int)((V >> (F - OZ_BETA * (q + 1))) & 127);
      s_d[q][kk][tx] = __int2bfloat16_rn(neg ? -d : d);
    }
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const int kp = k0 + tx;
    if (kp >= Kp) continue;
    const int64_t o = (int64_t)(i0 + r) * Kp + kp;
    for (int q = 0; q < nsl; ++q) out[q * slice_stride + o] = s_d[q][tx][r];
  }
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::); }
__device__ __forceinline__ void cp_async_wait_one() { asm volatile("cp.async.wait_group 1;\n" ::); }

__device__ __forceinline__ void ldsm_x4(unsigned (&r)[4], const void* smem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(s));
}
__device__ __forceinline__ void mma_bf16(float (&d)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

struct OzGemmArgs {
  const __nv_bfloat16* A;    // [S][mp][Kp]
  const __nv_bfloat16* Bre;  // [S][np][Kp]
  const __nv_bfloat16* Bim;
  int64_t sa, sb;            // slice strides (elements)
  int mp, np, Kp;
  int m, n;                  // true output size
  const int* ea;             // row exponents of A
  const int* eb;             // column exponents of B
  double2* C;                // FP64 output, column-major
  int64_t ldc;
  int nsl;                   // slices per operand
  int lower;                 // 1: only tiles with I >= J (square structured outputs)
};

// 2^E as a double (E within the normal range), built from the exponent bits
__device__ __forceinline__ double pow2i(int E) {
  if (E < -1022) return 0.0;
  return __longlong_as_double((long long)(1023 + E) << 52);
}

// One CTA per 64x64 tile; loops over all levels and super-chunks.
__global__ void __launch_bounds__(OZ_THREADS, 3) k_oz_gemm(OzGemmArgs g) {
  extern __shared__ __align__(16) unsigned char oz_smem[];
  __nv_bfloat16* sm = reinterpret_cast<__nv_bfloat16*>(oz_smem);
  // stage layout: A [64][LDS], Bre [64][LDS], Bim [64][LDS]; two stages
  const int stage_elems = 3 * OZ_TM * OZ_LDS;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp >> 1, wn = warp & 1;
  int bi = blockIdx.x, bj = blockIdx.y;
  if (g.lower) {
    const int t = blockIdx.x;
    tri_tile(t, bi, bj);
  }
  const int i0 = bi * OZ_TM, j0 = bj * OZ_TN;
  int sc = 0;
  for (int lev = 0; lev < g.nsl; ++lev) {
    const int64_t total_k = (int64_t)(lev + 1) * g.Kp;
    for (int64_t kbeg = 0; kbeg < total_k; kbeg += OZ_SUPER) {
      const int64_t kend = (kbeg + OZ_SUPER < total_k) ? kbeg + OZ_SUPER : total_k;
      const int ntiles = (int)((kend - kbeg) / OZ_TK);
      float fr[2][4][4], fi[2][4][4];
      int ir[2][4][4], ii[2][4][4];
#pragma unroll
      for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b)
#pragma unroll
          for (int c = 0; c < 4; ++c) { fr[a][b][c] = 0.f; fi[a][b][c] = 0.f; ir[a][b][c] = 0; ii[a][b][c] = 0; }

      auto load_stage = [&](int st, int tile) {
        const int64_t kg = kbeg + (int64_t)tile * OZ_TK;
        const int t = (int)(kg / g.Kp);
        const int kk = (int)(kg % g.Kp);
        const int u = lev - t;
        const __nv_bfloat16* Ab = g.A + t * g.sa + (int64_t)i0 * g.Kp + kk;
        const __nv_bfloat16* Brb = g.Bre + u * g.sb + (int64_t)j0 * g.Kp + kk;
        const __nv_bfloat16* Bib = g.Bim + u * g.sb + (int64_t)j0 * g.Kp + kk;
        __nv_bfloat16* s = sm + st * stage_elems;
        // 64 rows x 8 chunks of 16 B per operand
        for (int c = tid; c < 64 * 8; c += OZ_THREADS) {
          const int row = c >> 3, ch = c & 7;
          cp_async16(s + row * OZ_LDS + ch * 8, Ab + (int64_t)row * g.Kp + ch * 8);
          cp_async16(s + OZ_TM * OZ_LDS + row * OZ_LDS + ch * 8, Brb + (int64_t)row * g.Kp + ch * 8);
          cp_async16(s + 2 * OZ_TM * OZ_LDS + row * OZ_LDS + ch * 8, Bib + (int64_t)row * g.Kp + ch * 8);
        }
        cp_async_commit();
      };

      load_stage(0, 0);
      for (int tile = 0; tile < ntiles; ++tile) {
        const int st = tile & 1;
        if (tile + 1 < ntiles) {
          load_stage(st ^ 1, tile + 1);
          cp_async_wait_one();
        } else {
          cp_async_wait_all();
        }
        __syncthreads();
        const __nv_bfloat16* sA = sm + st * stage_elems;
        const __nv_bfloat16* sBr = sA + OZ_TM * OZ_LDS;
        const __nv_bfloat16* sBi = sBr + OZ_TM * OZ_LDS;
#pragma unroll
        for (int ks = 0; ks < OZ_TK / 16; ++ks) {
          unsigned af[2][4];
#pragma unroll
          for (int mt = 0; mt < 2; ++mt) {
            const int q = lane >> 3;
            const int row = wm * 32 + mt * 16 + (q & 1) * 8 + (lane & 7);
            const int col = ks * 16 + (q >> 1) * 8;
            ldsm_x4(af[mt], sA + row * OZ_LDS + col);
          }
          unsigned br[4][2], bi[4][2];
#pragma unroll
          for (int pr = 0; pr < 2; ++pr) {
            const int q = lane >> 3;
            const int row = wn * 32 + pr * 16 + (q >> 1) * 8 + (lane & 7);
            const int col = ks * 16 + (q & 1) * 8;
            unsigned r[4];
            ldsm_x4(r, sBr + row * OZ_LDS + col);
            br[2 * pr][0] = r[0]; br[2 * pr][1] = r[1]; br[2 * pr + 1][0] = r[2]; br[2 * pr + 1][1] = r[3];
            ldsm_x4(r, sBi + row * OZ_LDS + col);
            bi[2 * pr][0] = r[0]; bi[2 * pr][1] = r[1]; bi[2 * pr + 1][0] = r[2]; bi[2 * pr + 1][1] = r[3];
          }
#pragma unroll
          for (int mt = 0; mt < 2; ++mt)
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
              mma_bf16(fr[mt][nt], af[mt], br[nt][0], br[nt][1]);
              mma_bf16(fi[mt][nt], af[mt], bi[nt][0], bi[nt][1]);
            }
        }
        __syncthreads();
        // empty the FP32 accumulators every OZ_CHUNK terms (exact integers)
        if (((tile + 1) * OZ_TK) % OZ_CHUNK == 0 || tile + 1 == ntiles) {
#pragma unroll
          for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b)
#pragma unroll
              for (int c = 0; c < 4; ++c) {
                ir[a][b][c] += __float2int_rz(fr[a][b][c]); fr[a][b][c] = 0.f;
                ii[a][b][c] += __float2int_rz(fi[a][b][c]); fi[a][b][c] = 0.f;
              }
        }
      }
      // add this (level, super-chunk) exact result into the FP64 output:
      //   C += 2^(ea_i + eb_j - BETA (lev + 2)) (ir + i ii)
#pragma unroll
      for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 4; ++nt)
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int r = i0 + wm * 32 + mt * 16 + (lane >> 2) + ((q & 2) ? 8 : 0);
            const int c = j0 + wn * 32 + nt * 8 + 2 * (lane & 3) + (q & 1);
            if (r >= g.m || c >= g.n) continue;
            const int e0 = g.ea[r], e1 = g.eb[c];
            const double sc_ = (e0 > -1000 && e1 > -1000) ? pow2i(e0 + e1 - OZ_BETA * (lev + 2)) : 0.0;
            double2* cp = g.C + r + (int64_t)c * g.ldc;
            const double vr = sc_ * (double)ir[mt][nt][q], vi = sc_ * (double)ii[mt][nt][q];
            if (sc == 0) *cp = make_double2(vr, vi);
            else { double2 cur = *cp; cur.x += vr; cur.y += vi; *cp = cur; }
          }
      ++sc;
    }
  }
}

static int64_t rup(int64_t a, int64_t b) { return (a + b - 1) / b * b; }

// product kernel: 0 mma.sync (k_oz_gemm), 1 tcgen05 (k_oz_umma, one CTA per
// tile), 2 tcgen05 in two-CTA clusters sharing B by multicast, 3 tcgen05 2-SM
// MMAs on two-CTA clusters (the default: n2 = 8192 solve 422 ms against 430
// ms with one CTA per tile and 440 ms with multicast)
static std::atomic<int> g_oz_kernel{3};
int ozaki_kernel() {
  if (const char* s = getenv("ZQ_OZAKI")) {
    if (!strcmp(s, "mma")) return 0;
    if (!strcmp(s, "umma")) return 1;
    if (!strcmp(s, "umma_mc")) return 2;
    if (!strcmp(s, "umma_2sm")) return 3;
  }
  return g_oz_kernel.load();
}
int set_ozaki_kernel(int k) {
  if (k < 0 || k > 3) return ZQ_ERR_ARG;
  g_oz_kernel.store(k);
  return ZQ_OK;
}
int oz_umma_gemm(const __nv_bfloat16* As, const __nv_bfloat16* Brs, const __nv_bfloat16* Bis, int mp, int np, int Kp,
                 int m, int n, int nsl, int lower, const int* ea, const int* eb, double2* C, int64_t ldc, int* err,
                 cudaStream_t st, int variant);

// workspace for products with m, n <= 2 * nq and Kp <= 4 * nq + 64
size_t ozaki_workspace_bytes(int nq) {
  const int64_t mp = rup(2 * (int64_t)nq, OZ_PAD), np = rup(2 * (int64_t)nq, OZ_PAD), Kp = rup(4 * (int64_t)nq, 64);
  size_t b = 0;
  b += sizeof(__nv_bfloat16) * (size_t)OZ_SMAX * mp * Kp;       // A slices
  b += sizeof(__nv_bfloat16) * (size_t)OZ_SMAX * np * Kp * 2;   // B slices (re / im forms)
  b += sizeof(int) * (size_t)(mp + np + 64);
  return b + 9 * 256;
}

// structured square outputs: fill the upper triangle from the lower one
// (sym = +1 Hermitian, -1 complex antisymmetric); diagonal 64-tiles averaged
// 32 x 32 tiles: the block of tile pair (ti >= tj) reads the lower tile and,
// inside the diagonal 64 x 64 blocks (computed in full by the product), the
// mirrored upper tile, and writes both, all with coalesced rows; the mirror
// is transposed through shared memory.
constexpr int SF_T = 32;
__global__ void __launch_bounds__(256) k_oz_symfill(double2* __restrict__ C, int64_t ldc, int n, int sym) {
  const int ti = blockIdx.x, tj = blockIdx.y;
  if (tj > ti) return;
  __shared__ double2 sl[SF_T][SF_T + 1];  // sl[r][c] = C(i0 + r, j0 + c)
  __shared__ double2 su[SF_T][SF_T + 1];  // su[r][c] = C(j0 + r, i0 + c)
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int i0 = ti * SF_T, j0 = tj * SF_T;
  const bool diag64 = (ti >> 1) == (tj >> 1);  // the tile pair lies in a diagonal 64 x 64 block
#pragma unroll
  for (int k = 0; k < SF_T / 8; ++k) {
    const int c = ty + 8 * k;
    if (i0 + tx < n && j0 + c < n) sl[tx][c] = C[(i0 + tx) + (int64_t)(j0 + c) * ldc];
    if (diag64 && j0 + tx < n && i0 + c < n) su[tx][c] = C[(j0 + tx) + (int64_t)(i0 + c) * ldc];
  }
  __syncthreads();
  // entry (i, j) = (i0 + r, j0 + c), i >= j: its value, written back below, and
  // its mirror, staged for the upper tile (threads own distinct (r, c), so the
  // writes to su go to entries no other thread reads)
  double2 mir[SF_T / 8];
#pragma unroll
  for (int k = 0; k < SF_T / 8; ++k) {
    const int r = tx, c = ty + 8 * k;
    const int i = i0 + r, j = j0 + c;
    mir[k] = make_double2(0.0, 0.0);
    if (i >= n || j >= n || i < j) continue;
    double2 a = sl[r][c];
    if (diag64) {
      const double2 b = su[c][r];  // C(j, i)
      if (sym > 0) a = make_double2(0.5 * (a.x + b.x), 0.5 * (a.y - b.y));
      else a = make_double2(0.5 * (a.x - b.x), 0.5 * (a.y - b.y));
    }
    if (i == j) {
      if (sym > 0) a.y = 0.0; else a = make_double2(0.0, 0.0);
    }
    C[i + (int64_t)j * ldc] = a;
    mir[k] = (sym > 0) ? make_double2(a.x, -a.y) : make_double2(-a.x, -a.y);
  }
  __syncthreads();  // every read of su is done
#pragma unroll
  for (int k = 0; k < SF_T / 8; ++k) {
    const int r = tx, c = ty + 8 * k;
    su[c][r] = mir[k];
  }
  __syncthreads();
  // upper tile: C(j0 + r, i0 + c) for i0 + c > j0 + r
#pragma unroll
  for (int k = 0; k < SF_T / 8; ++k) {
    const int r = tx, c = ty + 8 * k;
    const int row = j0 + r, col = i0 + c;
    if (row < n && col < n && col > row) C[row + (int64_t)col * ldc] = su[r][c];
  }
}

int structured_fill(double2* C, int64_t ldc, int n, int sym, cudaStream_t st) {
  if (n <= 0) return ZQ_OK;
  const unsigned nt = (unsigned)ceil_div(n, SF_T);
  k_oz_symfill<<<dim3(nt, nt), dim3(SF_T, 8), 0, st>>>(C, ldc, n, sym);
  ZQ_LAUNCH_CHECK();
  return ZQ_OK;
}

// warps per row/column of k_oz_exp: enough for about 48 resident warps per
// SM (152 SMs), at most 8, and at least two 256-entry chunks per warp
static int oz_exp_parts(int count, const OzSide& s) {
  const int kmax = s.K1 > s.K2 ? s.K1 : s.K2;
  int parts = 1;
  while (parts < 8 && (int64_t)count * parts < 152 * 48 && kmax >= 2 * 256 * parts) parts *= 2;
  return parts;
}

int zgemm_ozaki(int opa1, int opb1, int opa2, int opb2, const ZgemmArgs& g, void* ws, size_t ws_bytes, cudaStream_t st,
                const OzOpts& opt) {
  const int m = g.m, n = g.n;
  if (m <= 0 || n <= 0) return ZQ_OK;
  const int nsl = (opt.slices >= 2 && opt.slices <= OZ_SMAX) ? opt.slices : 7;
  const bool two = g.A2 != nullptr;
  OzSide a{}, b{};
  a.X1 = g.A1; a.ld1 = g.lda1; a.op1 = opa1; a.K1 = g.k1;
  a.X2 = two ? g.A2 : nullptr; a.ld2 = g.lda2; a.op2 = opa2; a.K2 = two ? g.k2 : 0; a.s2 = two ? g.s2 : 0.0;
  b.X1 = g.B1; b.ld1 = g.ldb1; b.op1 = opb1; b.K1 = g.k1;
  b.X2 = two ? g.B2 : nullptr; b.ld2 = g.ldb2; b.op2 = opb2; b.K2 = two ? g.k2 : 0; b.s2 = 1.0;
  const int64_t Kp = rup(2 * ((int64_t)g.k1 + (two ? g.k2 : 0)), OZ_TK);
  const int64_t mp = rup(m, OZ_PAD), np = rup(n, OZ_PAD);
  size_t need = sizeof(__nv_bfloat16) * ((size_t)OZ_SMAX * mp * Kp + 2 * (size_t)OZ_SMAX * np * Kp) +
                sizeof(int) * (size_t)(mp + np + 64) + 9 * 256;
  if (need > ws_bytes) { set_error_message("zgemm_ozaki: workspace too small"); return ZQ_ERR_LIMIT; }
  if (g.alpha.x != 1.0 || g.alpha.y != 0.0 || g.beta.x != 0.0 || g.beta.y != 0.0) {
    set_error_message("zgemm_ozaki: only C = op(A) op(B) (alpha 1, beta 0)");
    return ZQ_ERR_ARG;
  }
  if (opt.structured != 0 && m != n) { set_error_message("zgemm_ozaki: structured output must be square"); return ZQ_ERR_ARG; }
  char* p = reinterpret_cast<char*>(ws);
  auto take = [&](size_t bytes) { char* q = p; p += (bytes + 255) & ~(size_t)255; return q; };
  // fixed carve-up (sized for the largest shapes) so the A slices of one call can be reused by the next
  const int64_t cap = (int64_t)(ws_bytes / 8);
  (void)cap;
  __nv_bfloat16* As = reinterpret_cast<__nv_bfloat16*>(take(sizeof(__nv_bfloat16) * OZ_SMAX * mp * Kp));
  __nv_bfloat16* Brs = reinterpret_cast<__nv_bfloat16*>(take(sizeof(__nv_bfloat16) * OZ_SMAX * np * Kp));
  __nv_bfloat16* Bis = reinterpret_cast<__nv_bfloat16*>(take(sizeof(__nv_bfloat16) * OZ_SMAX * np * Kp));
  int* ea = reinterpret_cast<int*>(take(sizeof(int) * mp));
  int* eb = reinterpret_cast<int*>(take(sizeof(int) * np));
  int* errf = reinterpret_cast<int*>(take(sizeof(int) * 4));
  auto grid = [](int64_t total) { int64_t x = (total + 255) / 256; return (int)(x > 16384 ? 16384 : x); };
  if (!opt.reuse_a) {
    const bool cm = (opa1 == OP_N || opa1 == OP_R) && (!two || opa2 == OP_N || opa2 == OP_R);
    if (cm) {
      // rows of op(A) are strided: column-wise passes (coalesced reads)
      k_oz_exp_init<<<ceil_div(m, 256), 256, 0, st>>>(ea, m);
      ZQ_LAUNCH_CHECK();
      const int Kc = g.k1 + (two ? g.k2 : 0);  // complex columns of op(A)
      k_oz_exp_cm<<<dim3((unsigned)ceil_div(m, 32), (unsigned)ceil_div(Kc, 256)), dim3(32, 8), 0, st>>>(a, m, Kc, ea);
      ZQ_LAUNCH_CHECK();
      k_oz_slice_cm<<<dim3((unsigned)(mp / 32), (unsigned)ceil_div((int)Kp, 32)), dim3(32, 8), 0, st>>>(a, m, (int)Kp, ea,
                                                                                                        nsl, As, mp * Kp);
      ZQ_LAUNCH_CHECK();
    } else {
      const int parts = oz_exp_parts(m, a);
      k_oz_exp_init<<<ceil_div(m, 256), 256, 0, st>>>(ea, m);
      ZQ_LAUNCH_CHECK();
      k_oz_exp<<<ceil_div(m * parts * 32, 256), 256, 0, st>>>(a, true, m, parts, ea);
      ZQ_LAUNCH_CHECK();
      k_oz_slice<<<grid(mp * Kp / 8), 256, 0, st>>>(a, true, m, (int)mp, (int)Kp, ea, nsl, As, nullptr, mp * Kp);
      ZQ_LAUNCH_CHECK();
    }
  }
  {
    const int parts = oz_exp_parts(n, b);
    k_oz_exp_init<<<ceil_div(n, 256), 256, 0, st>>>(eb, n);
    ZQ_LAUNCH_CHECK();
    k_oz_exp<<<ceil_div(n * parts * 32, 256), 256, 0, st>>>(b, false, n, parts, eb);
    ZQ_LAUNCH_CHECK();
  }
  k_oz_slice<<<grid(np * Kp / 8), 256, 0, st>>>(b, false, n, (int)np, (int)Kp, eb, nsl, Brs, Bis, np * Kp);
  ZQ_LAUNCH_CHECK();
  OzGemmArgs og{};
  og.A = As; og.Bre = Brs; og.Bim = Bis; og.sa = mp * Kp; og.sb = np * Kp;
  og.mp = (int)mp; og.np = (int)np; og.Kp = (int)Kp;
  og.m = m; og.n = n; og.ea = ea; og.eb = eb; og.C = g.C; og.ldc = g.ldc;
  og.nsl = nsl; og.lower = opt.structured != 0 ? 1 : 0;
  const bool lower = og.lower != 0;
  if (ozaki_kernel() >= 1) {
    // tcgen05 / TMEM / TMA product (zq_ozaki_umma.cu), 128 x 128 tiles
    const int tm = (int)(mp / 128), tn = (int)(np / 128);
    const double pairs = (double)nsl * (nsl + 1) / 2.0;
    const double tiles = lower ? (double)tm * (tm + 1) / 2.0 : (double)tm * tn;
    prof_add_flops(PC_OZAKI, pairs * 2.0 * tiles * 128.0 * 128.0 * (double)Kp * 2.0);
    prof_begin(PC_OZAKI, st);
    if (int rc = oz_umma_gemm(As, Brs, Bis, (int)mp, (int)np, (int)Kp, m, n, nsl, lower ? 1 : 0, ea, eb, g.C, g.ldc, errf,
                              st, ozaki_kernel() - 1))
      return rc;
    prof_end(PC_OZAKI, st);
    int herr = 0;
    ZQ_CUDA(cudaMemcpyAsync(&herr, errf, sizeof(int), cudaMemcpyDeviceToHost, st));
    ZQ_CUDA(cudaStreamSynchronize(st));
    if (herr) {
      set_error_message("k_oz_umma: a pipeline wait ran out of time (kernel stopped)");
      return ZQ_ERR_TIMEOUT;
    }
  } else {
    const int smem = 2 * 3 * OZ_TM * OZ_LDS * (int)sizeof(__nv_bfloat16);
    {
      // the shared-memory opt-in is per device; set once for each
      static std::atomic<unsigned long long> attr_set{0};
      int dev = 0;
      ZQ_CUDA(cudaGetDevice(&dev));
      const unsigned long long bit = 1ull << (dev & 63);
      if (!(attr_set.load() & bit)) {
        ZQ_CUDA(cudaFuncSetAttribute(k_oz_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        attr_set.fetch_or(bit);
      }
    }
    const int tm = (int)((m + OZ_TM - 1) / OZ_TM), tn = (int)((n + OZ_TN - 1) / OZ_TN);
    dim3 gg = og.lower ? dim3((unsigned)(tm * (tm + 1) / 2), 1) : dim3((unsigned)tm, (unsigned)tn);
    {
      // executed tensor-core flops: slice pairs x (Re, Im) x tiles x 64 x 64 x Kp x 2
      const double pairs = (double)nsl * (nsl + 1) / 2.0;
      const double tiles = og.lower ? (double)tm * (tm + 1) / 2.0 : (double)tm * tn;
      prof_add_flops(PC_OZAKI, pairs * 2.0 * tiles * OZ_TM * OZ_TN * (double)Kp * 2.0);
    }
    prof_begin(PC_OZAKI, st);
    k_oz_gemm<<<gg, OZ_THREADS, smem, st>>>(og);
    prof_end(PC_OZAKI, st);
    ZQ_LAUNCH_CHECK();
  }
  if (opt.structured != 0 && !opt.nofill) {
    if (int rc = structured_fill(g.C, g.ldc, m, opt.structured, st)) return rc;
  }
  return ZQ_OK;
}

}  // namespace zq

extern "C" int zq_set_ozaki_kernel(int which) {
  if (zq::set_ozaki_kernel(which)) {
    zq::set_error_message(
        "kernel must be 0 (mma.sync), 1 (tcgen05), 2 (tcgen05, cluster-multicast B) or 3 (tcgen05 2-SM MMA)");
    return zq::ZQ_ERR_ARG;
  }
  return zq::ZQ_OK;
}
extern "C" int zq_get_ozaki_kernel(void) { return zq::ozaki_kernel(); }

// Public utility: FP64-accurate complex product on the tensor cores.
//   C = op(A) op(B) (m x n, K inner), op codes 0 N, 1 T, 2 C (conj-transpose), 3 R (conj)
extern "C" int zq_zgemm_accurate(int opa, int opb, int m, int n, int k, const double* A, int lda, const double* B,
                                 int ldb, double* C, int ldc, void* stream) {
  using namespace zq;
  if (m < 0 || n < 0 || k < 0 || opa < 0 || opa > 3 || opb < 0 || opb > 3) return ZQ_ERR_ARG;
  if (m == 0 || n == 0) return ZQ_OK;
  const int q = (m > n ? m : n) / 2 + 1 > (k + 1) / 2 + 16 ? (m > n ? m : n) / 2 + 1 : (k + 1) / 2 + 16;
  const size_t bytes = ozaki_workspace_bytes(q);
  void* ws = nullptr;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  ZQ_CUDA(cudaMallocAsync(&ws, bytes, st));
  ZgemmArgs g{};
  g.m = m; g.n = n; g.k1 = k;
  g.A1 = reinterpret_cast<const double2*>(A); g.lda1 = lda;
  g.B1 = reinterpret_cast<const double2*>(B); g.ldb1 = ldb;
  g.alpha = make_double2(1.0, 0.0); g.beta = make_double2(0.0, 0.0);
  g.C = reinterpret_cast<double2*>(C); g.ldc = ldc;
  OzOpts opt{};
  opt.slices = 8;
  const int rc = zgemm_ozaki(opa, opb, OP_N, OP_N, g, ws, bytes, st, opt);
  cudaFreeAsync(ws, st);
  return rc;
}
