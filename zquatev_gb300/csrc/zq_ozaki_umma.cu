// Ozaki slice products on the 5th-generation tensor cores (tcgen05 + TMEM + TMA).
//
// Same arithmetic as k_oz_gemm (zq_ozaki.cu): for every level l (slice pairs
// (t, u) with t + u = l) the exact integer sum over the concatenated K terms
// of A_t . B_u is formed and C += sigma_i tau_j 2^(-BETA (l + 2)) I_l. Here a
// CTA owns a 128 x 128 output tile and computes its real and imaginary parts
// with one 128 x 256 x 16 bf16 MMA per K step (B operand = [Bre tile; Bim
// tile]); the FP32 accumulators live in tensor memory.
//
// Roles (320 threads, one CTA per SM by its shared memory):
//   warp 0      TMA producer: A, Bre, Bim boxes (64 K x 128 rows, 128-byte
//               swizzle) into a 4-stage ring (48 KB per stage);
//   warp 1      allocates 512 TMEM columns (two 256-column accumulators); one
//               elected thread issues tcgen05.mma and the commits;
//   warps 2..9  drain an accumulator every 512 K terms (tcgen05.ld; the FP32
//               sums of at most 512 products of 7-bit digits are exact
//               integers below 2^24), add them into int32 registers, and at
//               the end of each (level, super-chunk) add the scaled result
//               into the FP64 output. Warp w reads TMEM lanes 32 (w % 4)..;
//               two warps share a lane quarter and split the columns.
// The accumulators are double buffered, so draining one overlaps the MMAs
// into the other.
//
// Every wait on an mbarrier is bounded (default about 2 s of SM clock; the
// limit is a kernel argument, set by zq_set_pipeline_wait). On a timeout the
// kernel raises the error flag the host reads after the launch, stops issuing
// work, waits (bounded, always at the default limit) for its own copies and
// MMAs in flight, frees its TMEM and returns.
#include "zq_common.cuh"
#include "zq_kernels.h"

#include <atomic>
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <mutex>

namespace zq {
namespace {

constexpr int UM_BM = 128;           // output rows per CTA (TMEM lanes)
constexpr int UM_BN = 128;           // output columns per CTA (Re and Im: 256 accumulator columns)
constexpr int UM_BK = 64;            // K per stage: one 128-byte swizzle row of bf16
constexpr int UM_CH = 512;           // K terms per exact FP32 accumulation (512 * 127^2 < 2^24)
constexpr int UM_SUPER = 64 * 1024;  // K terms per int32 partial (65536 * 127^2 < 2^31)
constexpr int UM_BETA = 7;
constexpr int UM_THREADS = 320;
constexpr int UM_GROUP = 16;          // row tiles per group of the full-tile launch order
constexpr int UM_EPI = 4;             // C columns whose previous values the epilogue loads together
constexpr uint32_t UM_A_BYTES = UM_BM * UM_BK * 2;       // 16 KB
constexpr uint32_t UM_BH_BYTES = UM_BN * UM_BK * 2;      // 16 KB (Bre or Bim half)
constexpr uint32_t UM_RING_BYTES = 4 * (UM_A_BYTES + 2 * UM_BH_BYTES);  // 192 KB of stages
constexpr uint32_t UM_TMEM_COLS = 512;
// 1 KB alignment slack, the ring, the barriers, and 16 KB of slack after them
// so that every operand window an MMA descriptor of the last stage can span
// (up to one B half past the stage in the 2-SM form) lies inside the allocation
constexpr int UM_SMEM = 1024 + UM_RING_BYTES + 256 + 16384;
constexpr long long UM_WAIT_CYCLES = 4000000000LL;  // default wait limit: about 2 s of SM clock
// kind::f16 instruction descriptor: D f32, A and B bf16, both K-major, N = 256, M = 128
constexpr uint32_t UM_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((256u >> 3) << 17) | ((128u >> 4) << 24);
// the same for the 2-SM MMA: M = 256 (128 rows in each CTA of the pair)
constexpr uint32_t UM_IDESC_PAIR = (1u << 4) | (1u << 7) | (1u << 10) | ((256u >> 3) << 17) | ((256u >> 4) << 24);

struct UmArgs {
  int mp, np, Kp, m, n, nsl, lower;
  const int* ea;
  const int* eb;
  double2* C;
  int64_t ldc;
  int* err;
  long long wait;  // limit of every pipeline wait, SM clock cycles
};

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
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
// Bounded wait for the phase with the given parity. False when `limit` cycles
// pass (the abort flag is raised) or when another role has aborted.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* abort, long long limit) {
  const long long t0 = clock64();
  while (!mbar_try(bar, parity)) {
    if (*abort) return false;
    if (clock64() - t0 > limit) { *abort = 1; return false; }
  }
  return true;
}
// Bounded wait that ignores the abort flag (clean-up of work in flight): always
// the default limit, as copies and MMAs already issued finish in microseconds.
__device__ __forceinline__ void mbar_drain(uint32_t bar, uint32_t parity, long long limit = UM_WAIT_CYCLES) {
  const long long t0 = clock64();
  while (!mbar_try(bar, parity) && clock64() - t0 <= limit) {
  }
}

// the same box written to this CTA and its cluster peer (same shared offsets);
// complete_tx is signalled on the mbarrier at `bar` in each destination
__device__ __forceinline__ void tma_2d_mc(uint32_t dst, const CUtensorMap* tm, int x, int y, uint32_t bar, uint16_t mask) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes.multicast::cluster [%0], [%1, {%2, %3}], "
      "[%4], %5;" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(bar), "h"(mask)
      : "memory");
}
__device__ __forceinline__ void umma_commit_mc(uint32_t bar, uint16_t mask) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::"r"(
                   bar),
               "h"(mask)
               : "memory");
}
// address of the same shared variable in CTA `rank` of the cluster
__device__ __forceinline__ uint32_t mapa_shared(uint32_t addr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
  return r;
}
__device__ __forceinline__ void mbar_arrive_remote(uint32_t cluster_addr) {
  asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(cluster_addr) : "memory");
}
// TMA load into this CTA's shared memory whose completion is signalled on an
// mbarrier of either CTA of the pair
__device__ __forceinline__ void tma_2d_pair(uint32_t dst, const CUtensorMap* tm, int x, int y, uint32_t bar_cluster) {
  asm volatile(
      "cp.async.bulk.tensor.2d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(bar_cluster)
      : "memory");
}
__device__ __forceinline__ void umma_bf16_pair(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(UM_IDESC_PAIR), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void umma_commit_pair_mc(uint32_t bar, uint16_t mask) {
  asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::"r"(
                   bar),
               "h"(mask)
               : "memory");
}
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

__device__ __forceinline__ void tma_2d(uint32_t dst, const CUtensorMap* tm, int x, int y, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

// shared-memory matrix descriptor: K-major operand, 128-byte swizzle, 8-row
// groups 1024 bytes apart (the layout TMA writes for a 128-byte-wide box)
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) | ((uint64_t)1 << 46) |
         ((uint64_t)2 << 61);
}
__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(UM_IDESC), "r"(accumulate)
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

__device__ __forceinline__ double um_pow2i(int E) {
  if (E < -1022) return 0.0;
  return __longlong_as_double((long long)(1023 + E) << 52);
}

// Variants (template V):
//   0  one CTA per 128 x 128 tile: A box + Bre box + Bim box per stage (48 KB),
//      4 stages.
//   1  clusters of two CTAs on vertically adjacent tiles of the same column
//      tile, which share B: each CTA loads its own A box and one half of B
//      (rank 0 Bre, rank 1 Bim) multicast to both, so a CTA reads 32 KB per
//      stage from L2 instead of 48 KB; still 48 KB of shared memory per stage.
//      A stage is refilled once both CTAs' MMAs have released it.
//   2  the same pairs computed by 2-SM MMAs (tcgen05.mma.cta_group::2, M =
//      256): each CTA stages only its own A box and one half of B (rank 0
//      Bre, rank 1 Bim), 32 KB per stage, 6 stages; rank 0 issues the MMAs for
//      both SMs, each SM's tensor core reads its own A rows and both halves of
//      B, and each CTA's TMEM holds its 128 rows. Per MMA an SM writes and
//      reads 8 KB of shared memory instead of 12 KB, the rate that limits the
//      one-CTA form. Both CTAs' TMA loads complete on rank 0's full barrier;
//      the MMA commits arrive on both CTAs' empty and accumulator barriers;
//      rank 1's drain warps release an accumulator on rank 0's barrier.
// In variants 1 and 2 a cluster's second tile past the last row tile is
// computed but not written.
template <int V>
struct UmShape {
  static constexpr uint32_t stage_bytes = V == 2 ? UM_A_BYTES + UM_BH_BYTES : UM_A_BYTES + 2 * UM_BH_BYTES;
  static constexpr int stages = V == 2 ? 6 : 4;
};
static_assert(UmShape<0>::stages * UmShape<0>::stage_bytes <= UM_RING_BYTES, "ring");
static_assert(UmShape<2>::stages * UmShape<2>::stage_bytes <= UM_RING_BYTES, "ring");

template <int V>
__global__ void __launch_bounds__(UM_THREADS, 1)
    k_oz_umma(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmBr,
              const __grid_constant__ CUtensorMap tmBi, UmArgs g) {
  constexpr bool PAIR = V != 0;
  constexpr int STAGES = UmShape<V>::stages;
  constexpr uint32_t STAGE_BYTES = UmShape<V>::stage_bytes;
  extern __shared__ __align__(1024) unsigned char um_smem_raw[];
  // 1024-byte aligned stage ring (128-byte swizzle atoms), barriers after it
  const uint32_t raw = su32(um_smem_raw);
  const uint32_t ring = (raw + 1023u) & ~1023u;
  unsigned char* bar_area = um_smem_raw + (ring - raw) + UM_RING_BYTES;
  uint64_t* bars = reinterpret_cast<uint64_t*>(bar_area);  // full[S], empty[S], accf[2], acce[2], done
  const uint32_t full0 = su32(bars), empty0 = full0 + 8 * STAGES, accf0 = empty0 + 8 * STAGES,
                 acce0 = accf0 + 16, done_bar = acce0 + 16;
  __shared__ uint32_t s_tmem;
  __shared__ int s_abort;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t rank = PAIR ? cluster_rank() : 0u;
  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, V == 1 ? 2 : 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(accf0 + 8 * b, 1);
      mbar_init(acce0 + 8 * b, V == 2 ? 16 : 8);
    }
    mbar_init(done_bar, 1);
    s_abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 1) {
    if (V == 2) {
      // one warp of each CTA of the pair allocates collectively: the same
      // columns in both SMs' tensor memory
      asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&s_tmem)),
                   "r"(UM_TMEM_COLS)
                   : "memory");
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
    } else {
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&s_tmem)),
                   "r"(UM_TMEM_COLS)
                   : "memory");
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (PAIR) cluster_sync();  // the peer's barriers are initialised before any multicast or remote arrival
  const uint32_t tmem = s_tmem;
  volatile int* abort = &s_abort;

  int bi, bj;
  if (PAIR) {
    const int tm = g.mp / UM_BM, tn = g.np / UM_BN;
    const int p = (int)(blockIdx.x >> 1);
    if (g.lower) {
      // pairs (bj + 2q, bj + 2q + 1) down column bj, columns in order
      int col = 0, first = 0;
      while (col + 1 < tm && p >= first + (tm - col + 1) / 2) { first += (tm - col + 1) / 2; ++col; }
      bj = col;
      bi = col + 2 * (p - first) + (int)rank;
    } else {
      // groups of UM_GROUP / 2 row-tile pairs sweep the column tiles together
      const int P = (tm + 1) / 2, G2 = UM_GROUP / 2;
      const int per = G2 * tn, grp = p / per, firstp = grp * G2;
      const int gm = (P - firstp) < G2 ? (P - firstp) : G2;
      bi = 2 * (firstp + (p % per) % gm) + (int)rank;
      bj = (p % per) / gm;
    }
  } else if (g.lower) {
    tri_tile((int)blockIdx.x, bi, bj);
  } else {
    // grouped order: runs of UM_GROUP row tiles sweep the column tiles
    // together, so the CTAs resident at one time share their A and B slices
    // in L2 (a wave covers ~16 x 10 tiles instead of all row tiles x 2)
    const int tm = g.mp / UM_BM, tn = g.np / UM_BN;  // the host's grid is tm * tn
    const int t = (int)blockIdx.x, per = UM_GROUP * tn, grp = t / per, first = grp * UM_GROUP;
    const int gm = (tm - first) < UM_GROUP ? (tm - first) : UM_GROUP;
    bi = first + (t % per) % gm;
    bj = (t % per) / gm;
  }
  const int i0 = bi * UM_BM, j0 = bj * UM_BN;
  const int Kp = g.Kp;

  if (warp == 0) {
    // ------------------------------------------------------------ producer
    int issued = 0;
    if (lane == 0) {
      int ks = 0;
      bool ok = true;
      // variant 2: both CTAs' copies complete on rank 0's full barrier
      const uint32_t full_lead = V == 2 ? mapa_shared(full0, 0) : full0;
      for (int lev = 0; lev < g.nsl && ok; ++lev) {
        const int64_t total = (int64_t)(lev + 1) * Kp;
        for (int64_t kg = 0; kg < total && ok; kg += UM_BK) {
          const int stage = ks % STAGES, round = ks / STAGES;
          if (!mbar_wait(empty0 + 8 * stage, (round & 1) ^ 1, abort, g.wait)) { ok = false; break; }
          const uint32_t sA = ring + stage * STAGE_BYTES;
          const int t = (int)(kg / Kp), kk = (int)(kg % Kp), u = lev - t;
          if (V == 2) {
            if (rank == 0) mbar_expect_tx(full0 + 8 * stage, 2 * STAGE_BYTES);
            tma_2d_pair(sA, &tmA, kk, t * g.mp + i0, full_lead + 8 * stage);
            if (rank == 0) tma_2d_pair(sA + UM_A_BYTES, &tmBr, kk, u * g.np + j0, full_lead + 8 * stage);
            else tma_2d_pair(sA + UM_A_BYTES, &tmBi, kk, u * g.np + j0, full_lead + 8 * stage);
          } else {
            mbar_expect_tx(full0 + 8 * stage, STAGE_BYTES);
            tma_2d(sA, &tmA, kk, t * g.mp + i0, full0 + 8 * stage);
            if (V == 1) {
              if (rank == 0) tma_2d_mc(sA + UM_A_BYTES, &tmBr, kk, u * g.np + j0, full0 + 8 * stage, (uint16_t)3);
              else tma_2d_mc(sA + UM_A_BYTES + UM_BH_BYTES, &tmBi, kk, u * g.np + j0, full0 + 8 * stage, (uint16_t)3);
            } else {
              tma_2d(sA + UM_A_BYTES, &tmBr, kk, u * g.np + j0, full0 + 8 * stage);
              tma_2d(sA + UM_A_BYTES + UM_BH_BYTES, &tmBi, kk, u * g.np + j0, full0 + 8 * stage);
            }
          }
          ++ks;
        }
      }
      issued = ks;
      // copies in flight finish before the CTA may exit (after an abort in a
      // cluster a stage may lack the peer's part and never complete: its own
      // copies land within microseconds, so wait about a millisecond there).
      // In variant 2 only rank 0 holds the full barriers; rank 1 is held at
      // the final cluster barrier until rank 0 has drained them.
      if (V != 2 || rank == 0)
        for (int q = (issued > STAGES ? issued - STAGES : 0); q < issued; ++q)
          mbar_drain(full0 + 8 * (q % STAGES), (q / STAGES) & 1, PAIR ? 2000000LL : UM_WAIT_CYCLES);
    }
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer
    if (lane == 0 && (V != 2 || rank == 0)) {
      int ks = 0, ci = 0;
      bool ok = true;
      for (int lev = 0; lev < g.nsl && ok; ++lev) {
        const int64_t total = (int64_t)(lev + 1) * Kp;
        for (int64_t kbeg = 0; kbeg < total && ok; kbeg += UM_SUPER) {
          const int64_t kend = kbeg + UM_SUPER < total ? kbeg + UM_SUPER : total;
          for (int64_t cb = kbeg; cb < kend && ok; cb += UM_CH) {
            const int64_t ce = cb + UM_CH < kend ? cb + UM_CH : kend;
            const int buf = ci & 1;
            if (!mbar_wait(acce0 + 8 * buf, ((ci >> 1) & 1) ^ 1, abort, g.wait)) { ok = false; break; }
            tc_fence_after();
            const uint32_t d = tmem + (uint32_t)(buf * 256);
            for (int64_t kg = cb; kg < ce; kg += UM_BK) {
              const int stage = ks % STAGES, round = ks / STAGES;
              if (!mbar_wait(full0 + 8 * stage, round & 1, abort, g.wait)) { ok = false; break; }
              tc_fence_after();
              const uint32_t sA = ring + stage * STAGE_BYTES;
              const uint64_t ad = sw128_desc(sA), bd = sw128_desc(sA + UM_A_BYTES);
#pragma unroll
              for (int k = 0; k < UM_BK / 16; ++k) {  // 16 bf16 = 32 bytes along the swizzled row
                if (V == 2) umma_bf16_pair(d, ad + 2 * k, bd + 2 * k, (kg != cb || k > 0) ? 1u : 0u);
                else umma_bf16(d, ad + 2 * k, bd + 2 * k, (kg != cb || k > 0) ? 1u : 0u);
              }
              if (V == 2) umma_commit_pair_mc(empty0 + 8 * stage, (uint16_t)3);
              else if (V == 1) umma_commit_mc(empty0 + 8 * stage, (uint16_t)3);
              else umma_commit(empty0 + 8 * stage);
              ++ks;
            }
            if (!ok) break;
            if (V == 2) umma_commit_pair_mc(accf0 + 8 * buf, (uint16_t)3);
            else umma_commit(accf0 + 8 * buf);
            ++ci;
          }
        }
      }
      // every MMA issued has completed before TMEM is released
      if (V == 2) umma_commit_pair_mc(done_bar, (uint16_t)1);
      else umma_commit(done_bar);
      mbar_drain(done_bar, 0);
    }
  } else {
    // ------------------------------------------------------------ drain / epilogue
    const int q = warp & 3;             // TMEM lane quarter this warp may access
    const int h = (warp - 2) >> 2;      // column half (0: j0..j0+63, 1: j0+64..j0+127)
    const int row = i0 + 32 * q + lane;
    const uint32_t lane_base = tmem + ((uint32_t)(32 * q) << 16);
    // variant 2: an accumulator is free once both CTAs' drain warps released it
    const uint32_t acce_lead = V == 2 ? mapa_shared(acce0, 0) : acce0;
    int ir[64], ii[64];
#pragma unroll
    for (int c = 0; c < 64; ++c) { ir[c] = 0; ii[c] = 0; }
    int ci = 0, sc = 0;
    bool ok = true;
    const int e_row = row < g.m ? g.ea[row] : -1100;
    for (int lev = 0; lev < g.nsl && ok; ++lev) {
      const int64_t total = (int64_t)(lev + 1) * Kp;
      for (int64_t kbeg = 0; kbeg < total && ok; kbeg += UM_SUPER) {
        const int64_t kend = kbeg + UM_SUPER < total ? kbeg + UM_SUPER : total;
        for (int64_t cb = kbeg; cb < kend; cb += UM_CH) {
          const int buf = ci & 1;
          // warp-uniform outcome: the TMEM loads below are .sync.aligned
          const bool got = mbar_wait(accf0 + 8 * buf, (ci >> 1) & 1, abort, g.wait);
          if (!__all_sync(0xffffffffu, got)) { ok = false; break; }
          tc_fence_after();
          const uint32_t base = lane_base + (uint32_t)(buf * 256 + 64 * h);
#pragma unroll
          for (int gq = 0; gq < 4; ++gq) {
            uint32_t re[16], im[16];
            tmem_ld16(base + 16 * gq, re);
            tmem_ld16(base + 128 + 16 * gq, im);
            tmem_wait_ld();
#pragma unroll
            for (int c = 0; c < 16; ++c) {
              ir[16 * gq + c] += __float2int_rz(__uint_as_float(re[c]));
              ii[16 * gq + c] += __float2int_rz(__uint_as_float(im[c]));
            }
          }
          tc_fence_before();
          __syncwarp();
          if (lane == 0) {
            if (V == 2 && rank != 0) mbar_arrive_remote(acce_lead + 8 * buf);
            else mbar_arrive(acce0 + 8 * buf);
          }
          ++ci;
        }
        if (!ok) break;
        // C += 2^(ea_i + eb_j - BETA (lev + 2)) (ir + i ii) for this (level, super-chunk)
        // The previous values of UM_EPI columns are loaded together before any
        // of them is stored: in one load-add-store loop every load waits for
        // the store before it (they may alias), which left the MMAs without a
        // free accumulator for the length of 64 round trips (measured at
        // n2 = 8192: 4 columns at a time take the second refinement step from
        // 122 to 116 ms with 2-SM MMAs, from 130 to 124 ms with one CTA).
        if (row < g.m) {
#pragma unroll
          for (int c0 = 0; c0 < 64; c0 += UM_EPI) {
            double2 cur[UM_EPI];  // addresses clamped into the matrix: no branch around the loads
#pragma unroll
            for (int c = 0; c < UM_EPI; ++c) {
              const int col = j0 + 64 * h + c0 + c;
              cur[c] = sc ? __ldcg(g.C + row + (int64_t)(col < g.n ? col : g.n - 1) * g.ldc) : make_double2(0.0, 0.0);
            }
#pragma unroll
            for (int c = 0; c < UM_EPI; ++c) {
              const int col = j0 + 64 * h + c0 + c;
              if (col < g.n) {
                const int e_col = g.eb[col];
                const double s = (e_row > -1000 && e_col > -1000) ? um_pow2i(e_row + e_col - UM_BETA * (lev + 2)) : 0.0;
                g.C[row + (int64_t)col * g.ldc] =
                    make_double2(cur[c].x + s * (double)ir[c0 + c], cur[c].y + s * (double)ii[c0 + c]);
              }
              ir[c0 + c] = 0;
              ii[c0 + c] = 0;
            }
          }
        } else {
#pragma unroll
          for (int c = 0; c < 64; ++c) { ir[c] = 0; ii[c] = 0; }
        }
        ++sc;
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  // variant 2: both CTAs' MMAs and drains are finished before the collective release
  if (V == 2) cluster_sync();
  if (warp == 1) {
    if (V == 2)
      asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(UM_TMEM_COLS) : "memory");
    else
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(UM_TMEM_COLS) : "memory");
  }
  if (threadIdx.x == 0 && s_abort) atomicExch(g.err, 1);
  // neither CTA leaves while its peer may still copy into it or arrive on its barriers
  if (PAIR) cluster_sync();
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(tensor_map_encode_fn());
}

// rows x Kp bf16, row-major (Kp contiguous); boxes of 64 K x 128 rows, 128-byte swizzle
int make_map(CUtensorMap* tm, const __nv_bfloat16* base, int64_t Kp, int64_t rows) {
  auto enc = encode_fn();
  if (!enc) { set_error_message("cuTensorMapEncodeTiled unavailable"); return ZQ_ERR_CUDA; }
  cuuint64_t dims[2] = {(cuuint64_t)Kp, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)Kp * 2};
  cuuint32_t box[2] = {(cuuint32_t)UM_BK, 128u};
  cuuint32_t es[2] = {1u, 1u};
  const CUresult r = enc(tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<__nv_bfloat16*>(base), dims, strides, box, es,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) { set_error_message("cuTensorMapEncodeTiled failed"); return ZQ_ERR_CUDA; }
  return ZQ_OK;
}

std::atomic<long long> g_wait_cycles{UM_WAIT_CYCLES};

}  // namespace

void* tensor_map_encode_fn() {
  static std::once_flag once;
  static void* fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = p;
  });
  return fn;
}

int oz_umma_smem_bytes() { return UM_SMEM; }

void set_pipeline_wait_cycles(long long cycles) { g_wait_cycles.store(cycles > 0 ? cycles : UM_WAIT_CYCLES); }
long long pipeline_wait_cycles() { return g_wait_cycles.load(); }

// C (m x n, FP64 complex) from the slices (layout [S][rows padded to 128][Kp]);
// err: device int, zeroed here, raised by the kernel on a wait timeout.
int oz_umma_gemm(const __nv_bfloat16* As, const __nv_bfloat16* Brs, const __nv_bfloat16* Bis, int mp, int np, int Kp,
                 int m, int n, int nsl, int lower, const int* ea, const int* eb, double2* C, int64_t ldc, int* err,
                 cudaStream_t st, int variant) {
  if (variant < 0 || variant > 2) { set_error_message("oz_umma_gemm: variant 0..2"); return ZQ_ERR_ARG; }
  if (mp % UM_BM || np % UM_BN || Kp % UM_BK || nsl < 1) { set_error_message("oz_umma_gemm: bad padding"); return ZQ_ERR_ARG; }
  CUtensorMap ta, tbr, tbi;
  if (int rc = make_map(&ta, As, Kp, (int64_t)nsl * mp)) return rc;
  if (int rc = make_map(&tbr, Brs, Kp, (int64_t)nsl * np)) return rc;
  if (int rc = make_map(&tbi, Bis, Kp, (int64_t)nsl * np)) return rc;
  {
    static std::atomic<unsigned long long> attr_set{0};
    int dev = 0;
    ZQ_CUDA(cudaGetDevice(&dev));
    const unsigned long long bit = 1ull << (dev & 63);
    if (!(attr_set.load() & bit)) {
      ZQ_CUDA(cudaFuncSetAttribute(k_oz_umma<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, UM_SMEM));
      ZQ_CUDA(cudaFuncSetAttribute(k_oz_umma<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, UM_SMEM));
      ZQ_CUDA(cudaFuncSetAttribute(k_oz_umma<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, UM_SMEM));
      attr_set.fetch_or(bit);
    }
  }
  UmArgs a{};
  a.mp = mp; a.np = np; a.Kp = Kp; a.m = m; a.n = n; a.nsl = nsl; a.lower = lower;
  a.ea = ea; a.eb = eb; a.C = C; a.ldc = ldc; a.err = err;
  a.wait = g_wait_cycles.load();
  const int tm = mp / UM_BM, tn = np / UM_BN;
  ZQ_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
  if (variant != 0) {
    // clusters of two row-adjacent tiles (the last pair of a column may hold a tile past the matrix)
    int pairs = 0;
    if (lower) for (int col = 0; col < tm; ++col) pairs += (tm - col + 1) / 2;
    else pairs = ((tm + 1) / 2) * tn;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)(2 * pairs), 1, 1);
    cfg.blockDim = dim3(UM_THREADS, 1, 1);
    cfg.dynamicSmemBytes = UM_SMEM;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 2;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (variant == 1) ZQ_CUDA(cudaLaunchKernelEx(&cfg, k_oz_umma<1>, ta, tbr, tbi, a));
    else ZQ_CUDA(cudaLaunchKernelEx(&cfg, k_oz_umma<2>, ta, tbr, tbi, a));
  } else {
    const dim3 grid = lower ? dim3((unsigned)(tm * (tm + 1) / 2), 1) : dim3((unsigned)(tm * tn), 1);
    k_oz_umma<0><<<grid, UM_THREADS, UM_SMEM, st>>>(ta, tbr, tbi, a);
  }
  ZQ_LAUNCH_CHECK();
  return ZQ_OK;
}

}  // namespace zq
