// FP32-accurate products on the 5th-generation tensor cores (tcgen05.mma
// kind::tf32, three passes) for the refined path's FP32 decomposition: the
// trailing update of the reduction (reference blocked.cc:416-475), the Q
// formation (blocked.cc:477-544), the back-transform X Z (zquatev.cc:86-90)
// and the large merges of the divide and conquer.
//
// Each FP32 operand x is split into two TF32 values, hi = rna(x) and
// lo = rna(x - hi) (11 + 11 significant bits: x is represented to ~2^-22),
// and the product is formed as hi*hi + hi*lo + lo*hi with FP32 accumulation
// in tensor memory, at the TF32 tensor rate. The accumulation in tensor memory
// loses more than FP32 fused multiply-adds as K grows (measured: 7.8e-7 of
// sum |a||b| at K = 64, 2.1e-6 at 1024, 4.6e-6 at 4096, against 2.4e-7, 6e-8
// and 6e-8 for an FP32 GEMM), so the refined path uses it only where that stays
// below what the refinement removes (fp32_products_on_tensor_cores).
//
// Throughput: 4096^3 real in 1.83 ms (225 TFLOP/s of TF32 passes; 0.70 ms with
// the loads replaced by constants, so the producers' global loads still bound
// it), the n2 = 8192 back-transform in 5.9 ms against 17 ms with FP32
// multiply-adds. The producers' loads are unconditional and their values are
// not touched before the stores (see ld_chunk): with per-element arithmetic
// and bounds branches around them every load waited for the previous one
// (4.35 ms for the same product).
//
// A CTA owns a 128-row output tile: 128 complex columns (real and imaginary
// parts: 256 accumulator columns) or 256 real columns. Complex operands are
// expanded to real ones along K: row i of A carries (Re a_ik, Im a_ik) for
// consecutive k; output column j has two B rows, (Re b_kj, -Im b_kj) for the
// real part and (Im b_kj, Re b_kj) for the imaginary part.
//
// Roles (288 threads, one CTA per SM by its shared memory):
//   warp 0      allocates 256 TMEM columns; one thread issues the MMAs (12 per
//               32-term K block: 4 K steps x 3 passes) and the commits;
//   warps 1..8  producers: load their share of the next K block from global
//               memory (any layout: row- or K-contiguous, conjugated, signed,
//               two column sources, zero outside the matrix), split it into
//               hi/lo TF32 and store it in the 128-byte-swizzled K-major layout
//               the MMA reads (2 stages of 96 KB); after the last block they
//               drain the accumulator (tcgen05.ld) and write the output.
// Every mbarrier wait is bounded (zq_set_pipeline_wait); a wait that runs out
// raises a device flag the host reads once per solve, and the kernel stops,
// waits for the MMAs it issued, frees its TMEM and returns.
#include "zq_common.cuh"
#include "zq_kernels.h"
#include "zq_tc32.h"

#include <string>

#include <atomic>
#include <cstdlib>
#include <cstring>

namespace zq {
namespace {

constexpr int TC_BM = 128;
constexpr int TC_THREADS = 288;
constexpr int TC_STAGES = 2;
constexpr uint32_t TC_A_BYTES = 128 * 128;                   // 128 rows x 32 tf32
constexpr uint32_t TC_B_BYTES = 256 * 128;                   // 256 rows x 32 tf32
constexpr uint32_t TC_STAGE_BYTES = 2 * TC_A_BYTES + 2 * TC_B_BYTES;  // hi and lo of A and B: 96 KB
constexpr int TC_SMEM = 1024 + TC_STAGES * TC_STAGE_BYTES + 256;
constexpr uint32_t TC_TMEM_COLS = 256;
constexpr long long TC_DRAIN_CYCLES = 4000000000LL;
// kind::tf32 instruction descriptor: D f32, A and B tf32, both K-major, N = 256, M = 128
constexpr uint32_t TC_IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((256u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* abort, long long limit) {
  const long long t0 = clock64();
  while (!mbar_try(bar, parity)) {
    if (*abort) return false;
    if (clock64() - t0 > limit) { *abort = 1; return false; }
  }
  return true;
}
__device__ __forceinline__ void mbar_drain(uint32_t bar, uint32_t parity) {
  const long long t0 = clock64();
  while (!mbar_try(bar, parity) && clock64() - t0 <= TC_DRAIN_CYCLES) {
  }
}
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) | ((uint64_t)1 << 46) |
         ((uint64_t)2 << 61);
}
__device__ __forceinline__ void umma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(TC_IDESC), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ uint32_t tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}
// hi = rna(x), lo = rna(x - hi) for four values, stored as two 16-byte chunks
__device__ __forceinline__ void split_store(uint32_t dst_hi, uint32_t dst_lo, float a, float b, float c, float d) {
  const uint32_t h0 = tf32_rna(a), h1 = tf32_rna(b), h2 = tf32_rna(c), h3 = tf32_rna(d);
  const uint32_t l0 = tf32_rna(a - __uint_as_float(h0)), l1 = tf32_rna(b - __uint_as_float(h1));
  const uint32_t l2 = tf32_rna(c - __uint_as_float(h2)), l3 = tf32_rna(d - __uint_as_float(h3));
  asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(dst_hi), "r"(h0), "r"(h1), "r"(h2), "r"(h3) : "memory");
  asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(dst_lo), "r"(l0), "r"(l1), "r"(l2), "r"(l3) : "memory");
}
// byte offset of 16-byte chunk c (0..7) of row r in a 128-byte-swizzled K-major tile
__device__ __forceinline__ uint32_t swz(int r, int c) {
  return (uint32_t)((r >> 3) * 1024 + (r & 7) * 128 + ((c ^ (r & 7)) << 4));
}

// Raw loads of one 16-byte chunk (four floats: two complex or four real
// elements along K) of one operand row. The loads are unconditional and their
// values untouched here: an element outside [0, rows) x [0, kdim) reads the
// operand's base address instead and is cleared by its mask bit later, and
// signs / conjugation are applied when the chunk is stored. So all of a
// thread's loads of a K block are in flight together; an arithmetic use right
// after each load (or a branch around it) would make every load wait for the
// previous one.
__device__ __forceinline__ uint32_t ld_chunk(const Tc32Src& s, bool cplx, int r, int rows, int k, int kdim, float (&v)[4]) {
  const int per = cplx ? 2 : 4;        // elements in the chunk
  const bool row_ok = r < rows;
  if (s.vec && row_ok && k + per - 1 < kdim) {
    const int64_t off = cplx ? 2 * (k + (int64_t)r * s.ld) : (k + (int64_t)r * s.ld);
    const float4 q = __ldg(reinterpret_cast<const float4*>(s.p + off));
    v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
    return 0xFu;
  }
  uint32_t mask = 0;
  if (cplx) {
    const float2* p = reinterpret_cast<const float2*>(s.p);
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const bool ok = row_ok && k + e < kdim;
      const float2* a = ok ? (s.kfast ? p + (k + e) + (int64_t)r * s.ld : p + r + (int64_t)(k + e) * s.ld) : p;
      const float2 x = __ldg(a);
      v[2 * e] = x.x; v[2 * e + 1] = x.y;
      mask |= ok ? (3u << (2 * e)) : 0u;
    }
  } else {
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const bool ok = row_ok && k + e < kdim;
      const float* a = ok ? (s.kfast ? s.p + (k + e) + (int64_t)r * s.ld : s.p + r + (int64_t)(k + e) * s.ld) : s.p;
      v[e] = __ldg(a);
      mask |= ok ? (1u << e) : 0u;
    }
  }
  return mask;
}
// the chunk's values as the product uses them: masked, signed, conjugated
__device__ __forceinline__ void fix_chunk(const Tc32Src& s, bool cplx, uint32_t mask, const float (&v)[4], float (&o)[4]) {
  const float si = (cplx && s.conj) ? -s.sign : s.sign;
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const float sg = (cplx && (e & 1)) ? si : s.sign;
    o[e] = ((mask >> e) & 1u) ? v[e] * sg : 0.f;
  }
}

// One producer thread's share of one K block, held in registers between its
// global loads and its shared-memory stores (complex: 4 A and 4 B chunks;
// real: 4 A and 8 B chunks), with the chunks' mask bits.
template <bool CPLX>
struct TcStage {
  float a[4][4];
  float b[CPLX ? 4 : 8][4];
  uint32_t am, bm;
};

// unit q of thread t -> (row, 16-byte chunk): K-contiguous sources put eight
// consecutive threads on one row, row-contiguous ones 32 threads on
// consecutive rows (both coalesced)
__device__ __forceinline__ void unit_a(const Tc32Src& s, int t, int q, int& r, int& c) {
  if (s.kfast) { c = t & 7; r = (t >> 3) + 32 * q; } else { r = t & 127; c = (t >> 7) + 2 * q; }
}
__device__ __forceinline__ void unit_b(const Tc32Src& s, bool cplx, int t, int q, int& r, int& c) {
  if (cplx || s.kfast) unit_a(s, t, q, r, c);
  else { r = t; c = q; }
}
__device__ __forceinline__ int seg_of(const Tc32Args& g, int kbg) {
  int s = 0;
  while (s + 1 < g.nseg && kbg >= g.kb_first[s + 1]) ++s;
  return s;
}
// the segment's descriptors copied into registers: each field read at a
// constant parameter offset, not through a run-time index into parameter space
__device__ __forceinline__ Tc32Seg seg_copy(const Tc32Args& g, int s) {
  switch (s) {
    case 0: return g.seg[0];
    case 1: return g.seg[1];
    case 2: return g.seg[2];
    default: return g.seg[3];
  }
}
// the B source of output column col (the second source past nsplit)
__device__ __forceinline__ void b_source(const Tc32Seg& sg, int n, int col, Tc32Src& bs, int& bc, int& bcols) {
  const bool second = sg.b2.p != nullptr && col >= sg.nsplit;
  bs = second ? sg.b2 : sg.b;
  bc = second ? col - sg.nsplit : col;
  bcols = second ? n - sg.nsplit : (sg.b2.p != nullptr ? sg.nsplit : n);
}

template <bool CPLX>
__device__ __forceinline__ void stage_load(const Tc32Args& g, int kbg, int i0, int j0, int t, TcStage<CPLX>& st) {
  const int s = seg_of(g, kbg);
  const Tc32Seg sg = seg_copy(g, s);
  const int k0 = (kbg - g.kb_first[s]) * (CPLX ? 16 : 32);
  const int kw = CPLX ? 2 : 4;  // K elements per chunk
  st.am = 0; st.bm = 0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    int r, c;
    unit_a(sg.a, t, q, r, c);
    st.am |= ld_chunk(sg.a, CPLX, i0 + r, g.m, k0 + kw * c, sg.k, st.a[q]) << (4 * q);
  }
#pragma unroll
  for (int q = 0; q < (CPLX ? 4 : 8); ++q) {
    int r, c;
    unit_b(sg.b, CPLX, t, q, r, c);
    Tc32Src bs;
    int bc, bcols;
    b_source(sg, g.n, j0 + r, bs, bc, bcols);
    st.bm |= ld_chunk(bs, CPLX, bc, bcols, k0 + kw * c, sg.k, st.b[q]) << (4 * q);
  }
}

template <bool CPLX>
__device__ __forceinline__ void stage_store(const Tc32Args& g, int kbg, int j0, int t, uint32_t sa,
                                            const TcStage<CPLX>& st) {
  const Tc32Seg sg = seg_copy(g, seg_of(g, kbg));
  const uint32_t sah = sa, sal = sa + TC_A_BYTES, sbh = sa + 2 * TC_A_BYTES, sbl = sbh + TC_B_BYTES;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    int r, c;
    unit_a(sg.a, t, q, r, c);
    float v[4];
    fix_chunk(sg.a, CPLX, (st.am >> (4 * q)) & 0xFu, st.a[q], v);
    const uint32_t o = swz(r, c);
    split_store(sah + o, sal + o, v[0], v[1], v[2], v[3]);
  }
#pragma unroll
  for (int q = 0; q < (CPLX ? 4 : 8); ++q) {
    int r, c;
    unit_b(sg.b, CPLX, t, q, r, c);
    Tc32Src bs;
    int bc, bcols;
    b_source(sg, g.n, j0 + r, bs, bc, bcols);
    float b[4];
    fix_chunk(bs, CPLX, (st.bm >> (4 * q)) & 0xFu, st.b[q], b);
    if (CPLX) {  // (re0, im0, re1, im1) -> real-part row (re, -im), imaginary-part row (im, re)
      const uint32_t ore = swz(r, c), oim = swz(128 + r, c);
      split_store(sbh + ore, sbl + ore, b[0], -b[1], b[2], -b[3]);
      split_store(sbh + oim, sbl + oim, b[1], b[0], b[3], b[2]);
    } else {
      const uint32_t o = swz(r, c);
      split_store(sbh + o, sbl + o, b[0], b[1], b[2], b[3]);
    }
  }
}

template <bool CPLX>
__global__ void __launch_bounds__(TC_THREADS, 1) k_tc32(const __grid_constant__ Tc32Args g) {
  extern __shared__ __align__(1024) unsigned char tc_smem_raw[];
  const uint32_t raw = su32(tc_smem_raw);
  const uint32_t ring = (raw + 1023u) & ~1023u;
  const uint32_t bars = ring + TC_STAGES * TC_STAGE_BYTES;  // full[2], empty[2], accf, done
  const uint32_t full0 = bars, empty0 = bars + 8 * TC_STAGES, accf = empty0 + 8 * TC_STAGES, done_bar = accf + 8;
  __shared__ uint32_t s_tmem;
  __shared__ int s_abort;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < TC_STAGES; ++s) {
      mbar_init(full0 + 8 * s, 8);  // one arrival per producer warp
      mbar_init(empty0 + 8 * s, 1);
    }
    mbar_init(accf, 1);
    mbar_init(done_bar, 1);
    s_abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&s_tmem)),
                 "r"(TC_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = s_tmem;
  volatile int* abort = &s_abort;

  // output tile
  const int bn = CPLX ? 128 : 256;
  int bi, bj;
  if (g.tri) {
    tri_tile((int)blockIdx.x, bi, bj);
  } else {
    const int tm = ceil_div(g.m, TC_BM);
    bi = (int)blockIdx.x % tm;
    bj = (int)blockIdx.x / tm;
  }
  const int i0 = bi * TC_BM, j0 = bj * bn;
  // this split's K blocks
  const int z = (int)blockIdx.z;
  const int kb0 = (int)(((int64_t)g.kb_total * z) / g.splits), kb1 = (int)(((int64_t)g.kb_total * (z + 1)) / g.splits);
  const int nblk = kb1 - kb0;

  if (warp == 0) {
    // ------------------------------------------------------------ MMA issuer
    if (lane == 0) {
      bool ok = true;
      for (int it = 0; it < nblk; ++it) {
        const int stage = it % TC_STAGES, round = it / TC_STAGES;
        if (!mbar_wait(full0 + 8 * stage, round & 1, abort, g.wait)) { ok = false; break; }
        tc_fence_after();
        const uint32_t sa = ring + stage * TC_STAGE_BYTES;
        const uint64_t ah = sw128_desc(sa), al = sw128_desc(sa + TC_A_BYTES);
        const uint64_t bh = sw128_desc(sa + 2 * TC_A_BYTES), bl = sw128_desc(sa + 2 * TC_A_BYTES + TC_B_BYTES);
#pragma unroll
        for (int k = 0; k < 4; ++k) {  // 8 tf32 = 32 bytes along the swizzled row
          umma_tf32(tmem, ah + 2 * k, bh + 2 * k, (it > 0 || k > 0) ? 1u : 0u);
          umma_tf32(tmem, ah + 2 * k, bl + 2 * k, 1u);
          umma_tf32(tmem, al + 2 * k, bh + 2 * k, 1u);
        }
        umma_commit(empty0 + 8 * stage);
      }
      if (ok) umma_commit(accf);
      umma_commit(done_bar);
      mbar_drain(done_bar, 0);
    }
  } else {
    // ------------------------------------------------------------ producers
    // software-pipelined: the global loads of block it + 1 are in flight while
    // block it is split and stored
    const int t = threadIdx.x - 32;  // 0..255
    TcStage<CPLX> sx, sy;
    bool go = true;
    auto step = [&](int it, TcStage<CPLX>& cur, TcStage<CPLX>& nxt) {
      if (it + 1 < nblk) stage_load<CPLX>(g, kb0 + it + 1, i0, j0, t, nxt);
      const int stage = it % TC_STAGES, round = it / TC_STAGES;
      if (!__all_sync(0xffffffffu, mbar_wait(empty0 + 8 * stage, (round & 1) ^ 1, abort, g.wait))) { go = false; return; }
      stage_store<CPLX>(g, kb0 + it, j0, t, ring + stage * TC_STAGE_BYTES, cur);
      // generic-proxy stores become visible to the tensor core (async proxy)
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(full0 + 8 * stage);
    };
    if (nblk > 0) stage_load<CPLX>(g, kb0, i0, j0, t, sx);
    for (int it = 0; it < nblk && go; it += 2) {
      step(it, sx, sy);
      if (go && it + 1 < nblk) step(it + 1, sy, sx);
    }

    // ------------------------------------------------------------ epilogue
    const int q = warp & 3;             // TMEM lane quarter of this warp
    const int h = (warp - 1) >> 2;      // column half
    const int row = i0 + 32 * q + lane;
    const uint32_t lane_base = tmem + ((uint32_t)(32 * q) << 16);
    const bool partial = g.splits > 1;
    const bool use_beta = !partial && (g.beta.x != 0.f || g.beta.y != 0.f);
    const int64_t ldc = partial ? g.m : g.ldc;
    const int ctr = partial ? 0 : g.ctrans;
    auto masked = [&](int col) { return col >= g.n || (g.tri && (row < col || (g.tri == 2 && row == col))); };
    auto cidx = [&](int col) { return ctr ? (col + (int64_t)row * ldc) : (row + (int64_t)col * ldc); };
    constexpr int NG = CPLX ? 4 : 8;    // 16-column groups of this thread's half
    const int cw = CPLX ? 64 : 128;     // columns per half
    // beta != 0: the C values of a group are loaded one group ahead (the first
    // while the last MMAs run), so the reads overlap instead of each waiting
    float2 cpre[16];
    float rpre[16];
    auto prefetch = [&](int gq) {
      if (!use_beta || row >= g.m) return;
#pragma unroll
      for (int c = 0; c < 16; ++c) {
        const int col = j0 + cw * h + 16 * gq + c;
        if (CPLX) cpre[c] = masked(col) ? make_float2(0.f, 0.f) : reinterpret_cast<const float2*>(g.C)[cidx(col)];
        else rpre[c] = masked(col) ? 0.f : g.C[cidx(col)];
      }
    };
    prefetch(0);
    bool have = nblk > 0 && go;
    if (have) {
      const bool got = __all_sync(0xffffffffu, mbar_wait(accf, 0, abort, g.wait));
      if (!got) have = false;
      tc_fence_after();
    }
    if (!*abort) {
#pragma unroll 1
      for (int gq = 0; gq < NG; ++gq) {
        float2 cv[16];
        float rv[16];
#pragma unroll
        for (int c = 0; c < 16; ++c) { cv[c] = cpre[c]; rv[c] = rpre[c]; }
        if (gq + 1 < NG) prefetch(gq + 1);
        const int c0 = cw * h + 16 * gq;
        uint32_t re[16], im[16];
        if (have) {
          tmem_ld16(lane_base + (uint32_t)c0, re);
          if (CPLX) tmem_ld16(lane_base + (uint32_t)(128 + c0), im);
          tmem_wait_ld();
        } else {
#pragma unroll
          for (int c = 0; c < 16; ++c) { re[c] = 0u; im[c] = 0u; }
        }
        if (row >= g.m) continue;
#pragma unroll
        for (int c = 0; c < 16; ++c) {
          const int col = j0 + c0 + c;
          if (masked(col)) continue;
          const int64_t o = cidx(col);
          if (CPLX) {
            float2* C = reinterpret_cast<float2*>(partial ? g.P + (int64_t)2 * z * g.m * g.n : g.C);
            const float xr = __uint_as_float(re[c]), xi = __uint_as_float(im[c]);
            if (partial) { C[o] = make_float2(xr, xi); continue; }
            float2 out = make_float2(g.alpha.x * xr - g.alpha.y * xi, g.alpha.x * xi + g.alpha.y * xr);
            if (use_beta) {
              out.x += g.beta.x * cv[c].x - g.beta.y * cv[c].y;
              out.y += g.beta.x * cv[c].y + g.beta.y * cv[c].x;
            }
            C[o] = out;
          } else {
            float* C = partial ? g.P + (int64_t)z * g.m * g.n : g.C;
            const float x = __uint_as_float(re[c]);
            if (partial) { C[o] = x; continue; }
            float out = g.alpha.x * x;
            if (use_beta) out += g.beta.x * rv[c];
            C[o] = out;
          }
        }
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_TMEM_COLS) : "memory");
  if (threadIdx.x == 0 && s_abort && g.err) atomicExch(g.err, 1);
}

// C = alpha * sum_z P_z + beta * C (partials column-major m x n)
__global__ void k_tc32_reduce(const __grid_constant__ Tc32Args g) {
  const int64_t total = (int64_t)g.m * g.n;
  const bool use_beta = (g.beta.x != 0.f || g.beta.y != 0.f);
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % g.m), j = (int)(t / g.m);
    const int64_t o = g.ctrans ? (j + (int64_t)i * g.ldc) : (i + (int64_t)j * g.ldc);
    if (g.cplx) {
      const float2* P = reinterpret_cast<const float2*>(g.P);
      float re = 0.f, im = 0.f;
      for (int s = 0; s < g.splits; ++s) { const float2 p = P[t + s * total]; re += p.x; im += p.y; }
      float2* C = reinterpret_cast<float2*>(g.C);
      float2 out = make_float2(g.alpha.x * re - g.alpha.y * im, g.alpha.x * im + g.alpha.y * re);
      if (use_beta) {
        const float2 c = C[o];
        out.x += g.beta.x * c.x - g.beta.y * c.y;
        out.y += g.beta.x * c.y + g.beta.y * c.x;
      }
      C[o] = out;
    } else {
      float acc = 0.f;
      for (int s = 0; s < g.splits; ++s) acc += g.P[t + s * total];
      float out = g.alpha.x * acc;
      if (use_beta) out += g.beta.x * g.C[o];
      g.C[o] = out;
    }
  }
}

}  // namespace

int tc32_smem_bytes() { return TC_SMEM; }

bool fp32_products_on_tensor_cores(int use) {
  // default: the back-transform X Z and both kinds of Q-formation products.
  // The tensor cores' FP32 accumulation truncates, so a long inner dimension
  // loses accuracy: the W^H X products (inner L) are split along K into
  // accumulations of at most 8 K blocks (128 terms), summed in FP32 by the
  // split reduce. Measured at n2 = 8192 (a refinement step ends the solve when
  // its correction is <= 1e-7): with these the second step's correction is
  // 6.2e-8 (5.9e-8 with FP32 multiply-adds) and the solve takes two steps,
  // 30 ms faster; with the W^H X products in one accumulation per output it is
  // 2.6e-7 and a third step (~117 ms) is needed. With the divide-and-conquer
  // merges on this kernel the refinement needs four steps; with the trailing
  // update it does not converge from n = 1500 (its errors enter the
  // tridiagonal itself).
  // ZQ_FP32_PRODUCTS=cuda: none; ZQ_TC32_USES: comma list of trail, formq
  // (both kinds of Q-formation products), formq_w (the W^H X products),
  // formq_x (the X updates), applyz, dc, none.
  static const unsigned mask = [] {
    const char* e = getenv("ZQ_FP32_PRODUCTS");
    if (e && !strcmp(e, "cuda")) return 0u;
    const char* u = getenv("ZQ_TC32_USES");
    if (!u) return (1u << TC_USE_APPLYZ) | (1u << TC_USE_FORMQ) | (1u << TC_USE_FORMQ_X);
    unsigned m = 0;
    std::string list(u);
    size_t pos = 0;
    while (pos <= list.size()) {
      const size_t end = list.find(',', pos) == std::string::npos ? list.size() : list.find(',', pos);
      const std::string tok = list.substr(pos, end - pos);
      if (tok == "trail") m |= 1u << TC_USE_TRAIL;
      else if (tok == "formq") m |= (1u << TC_USE_FORMQ) | (1u << TC_USE_FORMQ_X);
      else if (tok == "formq_w") m |= 1u << TC_USE_FORMQ;
      else if (tok == "formq_x") m |= 1u << TC_USE_FORMQ_X;
      else if (tok == "applyz") m |= 1u << TC_USE_APPLYZ;
      else if (tok == "dc") m |= 1u << TC_USE_DC;
      pos = end + 1;
    }
    return m;
  }();
  return (mask >> use) & 1u;
}

int tc32_gemm(const Tc32Args& in, cudaStream_t st) {
  Tc32Args g = in;
  if (g.m <= 0 || g.n <= 0) return ZQ_OK;
  if (g.nseg < 1 || g.nseg > 4) { set_error_message("tc32_gemm: 1..4 segments"); return ZQ_ERR_ARG; }
  const int per = g.cplx ? 16 : 32;
  int kb = 0;
  for (int s = 0; s < g.nseg; ++s) {
    g.kb_first[s] = kb;
    kb += ceil_div(g.seg[s].k > 0 ? g.seg[s].k : 0, per);
  }
  g.kb_first[g.nseg] = kb;
  g.kb_total = kb;
  if (g.splits < 1) g.splits = 1;
  if (g.splits > kb && kb > 0) g.splits = kb;
  if (g.splits > 1 && (g.P == nullptr || g.tri)) { set_error_message("tc32_gemm: split K needs P and full tiles"); return ZQ_ERR_ARG; }
  if (g.tri && ceil_div(g.m, TC_BM) != ceil_div(g.n, g.cplx ? 128 : 256)) {
    set_error_message("tc32_gemm: triangular output needs a square tile grid");
    return ZQ_ERR_ARG;
  }
  g.wait = pipeline_wait_cycles();
  // 16-byte loads where a source is K-contiguous, 16-byte aligned and its rows
  // start on 16-byte boundaries
  auto vec_ok = [&](Tc32Src& x) {
    x.vec = (x.p != nullptr && x.kfast && (reinterpret_cast<uintptr_t>(x.p) % 16) == 0 &&
             (g.cplx ? (x.ld % 2) == 0 : (x.ld % 4) == 0)) ? 1 : 0;
  };
  for (int s = 0; s < g.nseg; ++s) { vec_ok(g.seg[s].a); vec_ok(g.seg[s].b); vec_ok(g.seg[s].b2); }
  {
    static std::atomic<unsigned long long> attr_set{0};
    int dev = 0;
    ZQ_CUDA(cudaGetDevice(&dev));
    const unsigned long long bit = 1ull << (dev & 63);
    if (!(attr_set.load() & bit)) {
      ZQ_CUDA(cudaFuncSetAttribute(k_tc32<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM));
      ZQ_CUDA(cudaFuncSetAttribute(k_tc32<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM));
      attr_set.fetch_or(bit);
    }
  }
  const int tm = ceil_div(g.m, TC_BM), tn = ceil_div(g.n, g.cplx ? 128 : 256);
  const dim3 grid(g.tri ? (unsigned)(tm * (tm + 1) / 2) : (unsigned)(tm * tn), 1, (unsigned)g.splits);
  if (g.cplx) k_tc32<true><<<grid, TC_THREADS, TC_SMEM, st>>>(g);
  else k_tc32<false><<<grid, TC_THREADS, TC_SMEM, st>>>(g);
  ZQ_LAUNCH_CHECK();
  if (g.splits > 1) {
    const int64_t total = (int64_t)g.m * g.n;
    const int blocks = (int)((total + 255) / 256 > 4096 ? 4096 : (total + 255) / 256);
    k_tc32_reduce<<<blocks, 256, 0, st>>>(g);
    ZQ_LAUNCH_CHECK();
  }
  return ZQ_OK;
}

}  // namespace zq

// C = op(A) op(B) in FP32-accurate tensor-core arithmetic (see zq_tc32.cu's
// header); all pointers in device memory, ordered after `stream`, waits for it.
extern "C" int zq_gemm_tf32x3(int cplx, int opa, int opb, int m, int n, int k, const float* A, int lda,
                              const float* B, int ldb, float* C, int ldc, int splits, void* stream) {
  using namespace zq;
  if (m < 0 || n < 0 || k < 0 || opa < 0 || opa > 3 || opb < 0 || opb > 3 || splits < 1 || splits > 64) return ZQ_ERR_ARG;
  if (!cplx && (opa > 1 || opb > 1)) return ZQ_ERR_ARG;
  const bool a_rows = (opa == OP_N || opa == OP_R), b_kfirst = (opb == OP_N || opb == OP_R);
  if (lda < 1 || ldb < 1 || ldc < 1 || lda < (a_rows ? m : k) || ldb < (b_kfirst ? k : n) || ldc < m) {
    set_error_message("zq_gemm_tf32x3: leading dimension too small");
    return ZQ_ERR_ARG;
  }
  if (m == 0 || n == 0) return ZQ_OK;
  if (!A || !B || !C) return ZQ_ERR_ARG;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  Tc32Args g{};
  g.cplx = cplx ? 1 : 0;
  g.m = m; g.n = n; g.nseg = 1;
  Tc32Seg& s = g.seg[0];
  s.k = k;
  // A (m x k): N and R are row-contiguous, T and C are K-contiguous
  s.a.p = A; s.a.ld = lda; s.a.kfast = (opa == OP_T || opa == OP_C) ? 1 : 0; s.a.conj = (opa == OP_C || opa == OP_R);
  s.a.sign = 1.f;
  // B (k x n) addressed by output column: N and R are K-contiguous
  s.b.p = B; s.b.ld = ldb; s.b.kfast = (opb == OP_N || opb == OP_R) ? 1 : 0; s.b.conj = (opb == OP_C || opb == OP_R);
  s.b.sign = 1.f;
  g.alpha = make_float2(1.f, 0.f); g.beta = make_float2(0.f, 0.f);
  g.C = C; g.ldc = ldc;
  g.splits = splits;
  void* mem = nullptr;
  const size_t pbytes = splits > 1 ? (size_t)splits * m * n * (cplx ? 8 : 4) : 0;
  ZQ_CUDA(cudaMallocAsync(&mem, pbytes + 256, st));
  g.err = reinterpret_cast<int*>(mem);
  g.P = splits > 1 ? reinterpret_cast<float*>(reinterpret_cast<char*>(mem) + 256) : nullptr;
  int rc = ZQ_OK;
  if (cudaMemsetAsync(g.err, 0, sizeof(int), st) != cudaSuccess) rc = ZQ_ERR_CUDA;
  if (rc == ZQ_OK) rc = tc32_gemm(g, st);
  int herr = 0;
  cudaMemcpyAsync(&herr, g.err, sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaFreeAsync(mem, st);
  const cudaError_t e = cudaStreamSynchronize(st);
  if (rc == ZQ_OK && e != cudaSuccess) { set_last_error(e, "cudaStreamSynchronize", __FILE__, __LINE__); rc = ZQ_ERR_CUDA; }
  if (rc == ZQ_OK && herr) { set_error_message("k_tc32: a pipeline wait ran out of time (kernel stopped)"); rc = ZQ_ERR_TIMEOUT; }
  return rc;
}
