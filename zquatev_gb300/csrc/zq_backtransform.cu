// Back-transformation and output assembly.
//
// Reference: zquatev.cc:74-98 -- band extraction + zhbev, U = Q0 Z and
// V = Q1 Z by zgemm3m (zquatev.cc:86-90), the explicit Q0/Q1 accumulated
// during the panels (blocked.cc:477-544), and the symmetry fill of the right
// half (zquatev.cc:92-98).
//
// Here Q is never accumulated during the reduction. After the tridiagonal is
// known:
//   1. phase_reduce: the quaternion subdiagonal e_k is made real by unit
//      quaternions phi with phi_{k+1} = e_k phi_k / |e_k|, so that
//      phi_{k+1}^H e_k phi_k = |e_k| (exact similarity, FP64);
//   2. form_q: X = Q * [diag(alpha); diag(beta)] (the left half of Q Phi) by
//      applying the stored reflectors backwards in compact-WY blocks,
//      Q_blk = I - V T V^H, with the structured 2x2-block T built from the
//      Gram matrix of the block's reflectors. Only the trailing (L x L)
//      sub-blocks that can be non-zero are touched (zungtr-style);
//   3. apply_z: (U; V) = X Z with the REAL eigenvector matrix Z of the
//      real tridiagonal; complex X is read as a real array with twice the
//      rows, so this is one real DGEMM;
//   4. symmetry_fill: D[:, n:] = (-conj(V); conj(U)).
#include "zq_common.cuh"
#include "zq_kernels.h"
#include "zq_tc32.h"

#include <atomic>
#include <cstdlib>
#include <type_traits>

namespace zq {

// Quaternion phases: phi_0 = 1, phi_{k+1} = u_k phi_k with u_k = e_k / |e_k|
// (phi reset to 1 where e_k = 0), i.e. a segmented prefix product of unit
// quaternions. One CTA: each thread takes a contiguous chunk, a Hillis-Steele
// scan over the 1024 chunk products combines them (quaternion products are
// associative), then every thread rewrites its chunk; each phi is normalised
// when written.
struct Quat { double a0, a1, b0, b1; int reset; };
// q(a1, b1) q(a2, b2) = q(a1 a2 - conj(b1) b2, b1 a2 + conj(a1) b2)
__device__ __forceinline__ Quat qmul(const Quat& x, const Quat& y) {
  Quat r;
  r.a0 = (x.a0 * y.a0 - x.a1 * y.a1) - (x.b0 * y.b0 + x.b1 * y.b1);
  r.a1 = (x.a0 * y.a1 + x.a1 * y.a0) - (x.b0 * y.b1 - x.b1 * y.b0);
  r.b0 = (x.b0 * y.a0 - x.b1 * y.a1) + (x.a0 * y.b0 + x.a1 * y.b1);
  r.b1 = (x.b0 * y.a1 + x.b1 * y.a0) + (x.a0 * y.b1 - x.a1 * y.b0);
  r.reset = 0;
  return r;
}
// later o earlier (segmented: a reset in `later` drops `earlier`)
__device__ __forceinline__ Quat qcombine(const Quat& later, const Quat& earlier) {
  if (later.reset) return later;
  Quat r = qmul(later, earlier);
  r.reset = earlier.reset;
  return r;
}
__device__ __forceinline__ Quat qunit_of(const double* e, int k, double& nrm) {
  const double ea0 = e[4 * k], ea1 = e[4 * k + 1], eb0 = e[4 * k + 2], eb1 = e[4 * k + 3];
  nrm = sqrt(ea0 * ea0 + ea1 * ea1 + eb0 * eb0 + eb1 * eb1);
  Quat u;
  if (nrm > 0.0) { const double s = 1.0 / nrm; u.a0 = ea0 * s; u.a1 = ea1 * s; u.b0 = eb0 * s; u.b1 = eb1 * s; u.reset = 0; }
  else { u.a0 = 1.0; u.a1 = 0.0; u.b0 = 0.0; u.b1 = 0.0; u.reset = 1; }
  return u;
}
constexpr int PH_T = 1024;
__global__ void __launch_bounds__(PH_T) k_phase(const double* e, int n, double* offd, double* phi) {
  __shared__ Quat s_q[PH_T];
  const int t = threadIdx.x;
  const int m = n - 1;                      // number of u_k
  const int per = (m + PH_T - 1) / PH_T;
  const int k0 = t * per, k1 = (k0 + per < m) ? k0 + per : m;
  Quat acc{1.0, 0.0, 0.0, 0.0, 0};
  for (int k = k0; k < k1; ++k) {
    double nrm;
    const Quat u = qunit_of(e, k, nrm);
    acc = qcombine(u, acc);
  }
  s_q[t] = acc;
  __syncthreads();
  for (int off = 1; off < PH_T; off <<= 1) {
    Quat v = s_q[t];
    if (t >= off) v = qcombine(v, s_q[t - off]);
    __syncthreads();
    s_q[t] = v;
    __syncthreads();
  }
  // exclusive prefix of this chunk = inclusive prefix of the previous one
  Quat run = (t > 0) ? s_q[t - 1] : Quat{1.0, 0.0, 0.0, 0.0, 0};
  if (t == 0) { phi[0] = 1.0; phi[1] = 0.0; phi[2] = 0.0; phi[3] = 0.0; }
  for (int k = k0; k < k1; ++k) {
    double nrm;
    const Quat u = qunit_of(e, k, nrm);
    offd[k] = nrm;
    run = qcombine(u, run);
    const double s = 1.0 / sqrt(run.a0 * run.a0 + run.a1 * run.a1 + run.b0 * run.b0 + run.b1 * run.b1);
    phi[4 * (k + 1) + 0] = run.a0 * s; phi[4 * (k + 1) + 1] = run.a1 * s;
    phi[4 * (k + 1) + 2] = run.b0 * s; phi[4 * (k + 1) + 3] = run.b1 * s;
  }
}

int phase_reduce(const double* e, int n, double* offd, double* phi, cudaStream_t st) {
  if (n <= 0) return ZQ_OK;
  k_phase<<<1, PH_T, 0, st>>>(e, n, offd, phi);
  ZQ_LAUNCH_CHECK();
  return ZQ_OK;
}

// X = [diag(alpha); diag(beta)]
template <typename Z>
__global__ void k_init_x(Z* X, int64_t ldx, int n, const double* phi) {
  const int64_t total = (int64_t)2 * n * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(t % (2 * n));
    const int c = (int)(t / (2 * n));
    Z v = czero<Z>();
    if (r == c) { v.x = phi[4 * c]; v.y = phi[4 * c + 1]; }
    else if (r == n + c) { v.x = phi[4 * c + 2]; v.y = phi[4 * c + 3]; }
    X[r + (int64_t)c * ldx] = v;
  }
}

// pack the block's reflectors: Wa[r, i] = A(p+1+r, p+i) for r >= i, else 0 (same for B)
template <typename Z>
__global__ void k_pack_w(const Z* M, int64_t ldm, int n, int p, int kb, int L, Z* Wa, Z* Wb) {
  const int64_t total = (int64_t)L * kb;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(t % L), i = (int)(t / L);
    Z va = czero<Z>(), vb = va;
    if (r >= i) {
      const int64_t o = (p + 1 + r) + (int64_t)(p + i) * ldm;
      va = M[o];
      vb = M[n + o];
    }
    Wa[r + (int64_t)i * L] = va;
    Wb[r + (int64_t)i * L] = vb;
  }
}

// T (kb x kb quaternion, upper triangular) from G1 = <w_i, w_l>, G2 = [w_i, w_l]:
//   T[k][k] = 1,  T[i][k] = - sum_{i<=l<k} T[i][l] q(G1[l][k], G2[l][k])
// One CTA of 1024 threads: thread (i, g) sums the l = i+g, i+g+16, ... terms of
// column k; the 16 partials of each row are reduced in shared memory.
constexpr int BT_G = 16;
template <typename Z>
__global__ void __launch_bounds__(1024) k_build_t(const Z* G1, const Z* G2, int kb, Z* Ta, Z* Tb) {
  const int tid = threadIdx.x;
  const int i = tid & 63, g = tid >> 6;
  __shared__ Z red[BT_G][64][2];
  for (int t = tid; t < kb * kb; t += blockDim.x) { Ta[t] = czero<Z>(); Tb[t] = czero<Z>(); }
  __syncthreads();
  for (int k = 0; k < kb; ++k) {
    Z sa = czero<Z>(), sb = sa;
    if (i < k) {
      for (int l = i + g; l < k; l += BT_G) {
        const Z ta = Ta[i + l * kb], tb = Tb[i + l * kb];
        const Z g1 = G1[l + k * kb], g2 = G2[l + k * kb];
        // q(ta, tb) q(g1, g2) = q(ta g1 - conj(tb) g2, tb g1 + conj(ta) g2)
        cfma(sa, ta, g1); cfmac(sa, cneg(tb), g2);
        cfma(sb, tb, g1); cfmac(sb, ta, g2);
      }
    }
    red[g][i][0] = sa;
    red[g][i][1] = sb;
    __syncthreads();
    if (g == 0) {
      if (i < k) {
        Z ta = czero<Z>(), tb = ta;
        for (int q = 0; q < BT_G; ++q) { ta = cadd(ta, red[q][i][0]); tb = cadd(tb, red[q][i][1]); }
        Ta[i + k * kb] = cneg(ta);
        Tb[i + k * kb] = cneg(tb);
      } else if (i == k) {
        Z one = czero<Z>();
        one.x = 1;
        Ta[k + k * kb] = one;
        Tb[k + k * kb] = czero<Z>();
      }
    }
    __syncthreads();
  }
}

// The same recurrence for FP32 with G1, G2, Ta, Tb in shared memory (4 kb^2
// complex64, 128 KB at kb = 64): each step reads what the previous one wrote
// a shared-memory load away instead of an L2 round trip.
__global__ void __launch_bounds__(1024) k_build_t_sm(const float2* G1, const float2* G2, int kb, float2* Ta,
                                                     float2* Tb) {
  extern __shared__ float2 bt_sm[];
  float2* g1 = bt_sm;
  float2* g2 = g1 + kb * kb;
  float2* ta_s = g2 + kb * kb;
  float2* tb_s = ta_s + kb * kb;
  const int tid = threadIdx.x;
  const int i = tid & 63, g = tid >> 6;
  __shared__ float2 red[BT_G][64][2];
  for (int t = tid; t < kb * kb; t += blockDim.x) {
    g1[t] = G1[t]; g2[t] = G2[t];
    ta_s[t] = czero<float2>(); tb_s[t] = czero<float2>();
  }
  __syncthreads();
  for (int k = 0; k < kb; ++k) {
    float2 sa = czero<float2>(), sb = sa;
    if (i < k) {
      for (int l = i + g; l < k; l += BT_G) {
        const float2 ta = ta_s[i + l * kb], tb = tb_s[i + l * kb];
        const float2 a1 = g1[l + k * kb], a2 = g2[l + k * kb];
        cfma(sa, ta, a1); cfmac(sa, cneg(tb), a2);
        cfma(sb, tb, a1); cfmac(sb, ta, a2);
      }
    }
    red[g][i][0] = sa;
    red[g][i][1] = sb;
    __syncthreads();
    if (g == 0) {
      if (i < k) {
        float2 ta = czero<float2>(), tb = ta;
        for (int q = 0; q < BT_G; ++q) { ta = cadd(ta, red[q][i][0]); tb = cadd(tb, red[q][i][1]); }
        ta_s[i + k * kb] = cneg(ta);
        tb_s[i + k * kb] = cneg(tb);
      } else if (i == k) {
        ta_s[k + k * kb] = make_float2(1.f, 0.f);
        tb_s[k + k * kb] = czero<float2>();
      }
    }
    __syncthreads();
  }
  for (int t = tid; t < kb * kb; t += blockDim.x) { Ta[t] = ta_s[t]; Tb[t] = tb_s[t]; }
}

// split-K partial buffer of the Q formation (complex elements)
static int64_t fq_pcap(int n, int nbq) { return (int64_t)64 * nbq * (n > 64 ? n : 64); }

// Most K blocks (16 complex terms each) per split of the tensor-core W^H X
// product (env ZQ_FORMQ_KSPLIT; 0: only as many splits as fill the GPU). Each
// split accumulates in tensor memory, whose FP32 sums truncate; the splits are
// added in FP32 by the reduce. 8 blocks keep the refinement's second-step
// correction at 6.2e-8 at n2 = 8192 (one accumulation per output: 2.6e-7).
static int formq_kblocks_per_split() {
  static const int v = [] {
    const char* s = getenv("ZQ_FORMQ_KSPLIT");
    return s ? atoi(s) : 8;
  }();
  return v;
}

// split-K partials of the look-ahead stream's Gram products (complex elements)
static int64_t fq_hcap(int nbq) { return (int64_t)64 * nbq * nbq; }

size_t form_q_workspace_bytes(int n, int nbq) {
  // Wa, Wb (n x nbq), G1, G2, Ta, Tb (nbq^2), C1e, C1o, C2e, C2o (nbq x n), split-K partials;
  // then the look-ahead slot: Wa, Wb, G1, G2, Ta, Tb and its Gram products' partials
  return sizeof(double2) * ((size_t)2 * n * nbq + 4 * (size_t)nbq * nbq + 4 * (size_t)nbq * n + (size_t)fq_pcap(n, nbq) +
                            (size_t)2 * n * nbq + 4 * (size_t)nbq * nbq + (size_t)fq_hcap(nbq)) +
         256;
}

// Operand source of the tensor-core product (zq_tc32.cu) over a complex64 array.
static Tc32Src tsrc(const float2* p, int64_t ld, int kfast, int conj = 0, float sign = 1.f) {
  Tc32Src s{};
  s.p = reinterpret_cast<const float*>(p); s.ld = ld; s.kfast = kfast; s.conj = conj; s.sign = sign;
  return s;
}

template <typename R>
int form_q(const cplx<R>* M, int64_t ldm, int n, const double* phi, cplx<R>* X, int64_t ldx, int nbq, void* ws,
           cudaStream_t st, int* tc_err) {
  using Z = cplx<R>;
  using Args = ZgemmArgsT<R>;
  if (n <= 0) return ZQ_OK;
  // FP32 path: the two large products per block on the tensor cores
  const bool fp32 = std::is_same<R, float>::value && tc_err != nullptr;
  const bool use_tc = fp32 && fp32_products_on_tensor_cores(TC_USE_FORMQ);     // C1 = W^H X (inner L)
  const bool use_tc_x = fp32 && fp32_products_on_tensor_cores(TC_USE_FORMQ_X); // X -= W C2 (inner nbq)
  k_init_x<Z><<<ceil_div(2 * n * n, 256) > 4096 ? 4096 : ceil_div(2 * n * n, 256), 256, 0, st>>>(X, ldx, n, phi);
  ZQ_LAUNCH_CHECK();
  const int nref = n - 2;  // reflectors exist for columns 0..n-3
  if (nref <= 0) return ZQ_OK;
  // Per block: W (the block's reflectors, packed), its Gram matrices G1, G2
  // and T depend only on the reflectors, not on X; they form a slot. In the
  // FP32 path the next block's slot is prepared on a look-ahead stream while
  // this block's products with X run (two slots, events in both directions).
  struct Slot { Z *Wa, *Wb, *G1, *G2, *Ta, *Tb; };
  Z* p = reinterpret_cast<Z*>(ws);
  Slot slot[2];
  slot[0].Wa = p; p += (size_t)n * nbq;
  slot[0].Wb = p; p += (size_t)n * nbq;
  slot[0].G1 = p; p += (size_t)nbq * nbq;
  slot[0].G2 = p; p += (size_t)nbq * nbq;
  slot[0].Ta = p; p += (size_t)nbq * nbq;
  slot[0].Tb = p; p += (size_t)nbq * nbq;
  Z* C1e = p; p += (size_t)nbq * n;
  Z* C1o = p; p += (size_t)nbq * n;
  Z* C2e = p; p += (size_t)nbq * n;
  Z* C2o = p; p += (size_t)nbq * n;
  Z* Pk = p;
  const int64_t pcap = fq_pcap(n, nbq);
  p += pcap;
  slot[1].Wa = p; p += (size_t)n * nbq;
  slot[1].Wb = p; p += (size_t)n * nbq;
  slot[1].G1 = p; p += (size_t)nbq * nbq;
  slot[1].G2 = p; p += (size_t)nbq * nbq;
  slot[1].Ta = p; p += (size_t)nbq * nbq;
  slot[1].Tb = p; p += (size_t)nbq * nbq;
  Z* Ph = p;
  const int64_t hcap = fq_hcap(nbq);
  Z* Xa = X;
  Z* Xb = X + n;
  Z one = czero<Z>(), zero = czero<Z>(), mone = czero<Z>();
  one.x = 1; mone.x = -1;
  const int nblocks = ceil_div(nref, nbq);
  // pack W of block bi, its Gram matrices and T into s, on stream sp
  auto prep = [&](int bi, const Slot& s, cudaStream_t sp, Z* P, int64_t pc) -> int {
    const int pb = bi * nbq;
    const int kb = (nbq < nref - pb) ? nbq : (nref - pb);
    const int L = n - 1 - pb;
    k_pack_w<Z><<<ceil_div(L * kb, 256) > 2048 ? 2048 : ceil_div(L * kb, 256), 256, 0, sp>>>(M, ldm, n, pb, kb, L, s.Wa,
                                                                                           s.Wb);
    ZQ_LAUNCH_CHECK();
    // G1 = Wa^H Wa + Wb^H Wb ; G2 = Wa^T Wb - Wb^T Wa   (kb x kb, inner L)
    Args g{};
    g.P = P; g.pcap = pc;
    g.m = kb; g.n = kb; g.k1 = L; g.k2 = L;
    g.A1 = s.Wa; g.lda1 = L; g.B1 = s.Wa; g.ldb1 = L;
    g.A2 = s.Wb; g.lda2 = L; g.B2 = s.Wb; g.ldb2 = L;
    g.s2 = (R)1; g.alpha = one; g.beta = zero;
    g.C = s.G1; g.ldc = kb;
    if (int rc = zgemm(OP_C, OP_N, OP_C, OP_N, g, 1, sp)) return rc;
    g.A1 = s.Wa; g.B1 = s.Wb; g.A2 = s.Wb; g.B2 = s.Wa; g.s2 = (R)-1; g.C = s.G2;
    if (int rc = zgemm(OP_T, OP_N, OP_T, OP_N, g, 1, sp)) return rc;
    if constexpr (std::is_same<R, float>::value) {
      const size_t sm = sizeof(float2) * 4 * (size_t)kb * kb;  // kb <= 64: <= 128 KB
      static std::atomic<unsigned long long> attr_set{0};  // per device
      int dev = 0;
      ZQ_CUDA(cudaGetDevice(&dev));
      const unsigned long long bit = 1ull << (dev & 63);
      if (!(attr_set.load() & bit)) {
        ZQ_CUDA(cudaFuncSetAttribute(k_build_t_sm, cudaFuncAttributeMaxDynamicSharedMemorySize, 4 * 64 * 64 * 8));
        attr_set.fetch_or(bit);
      }
      k_build_t_sm<<<1, 1024, sm, sp>>>(s.G1, s.G2, kb, s.Ta, s.Tb);
    } else {
      k_build_t<Z><<<1, 1024, 0, sp>>>(s.G1, s.G2, kb, s.Ta, s.Tb);
    }
    ZQ_LAUNCH_CHECK();
    return ZQ_OK;
  };
  // look-ahead stream and its events (FP32 path, more than one block)
  bool ahead = fp32 && nblocks > 1;
  cudaStream_t sh = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_ready[2] = {nullptr, nullptr}, ev_free[2] = {nullptr, nullptr};
  struct Release {
    cudaStream_t& sh; cudaEvent_t& f; cudaEvent_t* r; cudaEvent_t* w;
    ~Release() {
      // safe with work pending: resources are released once it completes
      for (int i = 0; i < 2; ++i) { if (r[i]) cudaEventDestroy(r[i]); if (w[i]) cudaEventDestroy(w[i]); }
      if (f) cudaEventDestroy(f);
      if (sh) cudaStreamDestroy(sh);
    }
  } release{sh, ev_fork, ev_ready, ev_free};
  if (ahead) {
    // without the stream or its events (resources exhausted) the blocks run
    // one after another on st, as in the FP64 path
    bool ok = cudaStreamCreateWithFlags(&sh, cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming) == cudaSuccess;
    for (int i = 0; i < 2 && ok; ++i)
      ok = cudaEventCreateWithFlags(&ev_ready[i], cudaEventDisableTiming) == cudaSuccess &&
           cudaEventCreateWithFlags(&ev_free[i], cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
      (void)cudaGetLastError();
      ahead = false;
    }
  }
  if (ahead) {
    // the look-ahead stream starts after everything already queued on st
    ZQ_CUDA(cudaEventRecord(ev_fork, st));
    ZQ_CUDA(cudaStreamWaitEvent(sh, ev_fork, 0));
    const int b0 = nblocks - 1;
    if (int rc = prep(b0, slot[b0 & 1], sh, Ph, hcap)) return rc;
    ZQ_CUDA(cudaEventRecord(ev_ready[b0 & 1], sh));
  }
  for (int bi = nblocks - 1; bi >= 0; --bi) {
    const int pb = bi * nbq;
    const int kb = (nbq < nref - pb) ? nbq : (nref - pb);
    const int L = n - 1 - pb;
    const int si = ahead ? (bi & 1) : 0;
    const Slot& cur = slot[si];
    if (ahead) {
      if (bi >= 1) {
        // next block into the other slot, once the block that used it last
        // (bi + 1) has finished its X update
        if (bi + 1 <= nblocks - 1) ZQ_CUDA(cudaStreamWaitEvent(sh, ev_free[si ^ 1], 0));
        if (int rc = prep(bi - 1, slot[si ^ 1], sh, Ph, hcap)) return rc;
        ZQ_CUDA(cudaEventRecord(ev_ready[si ^ 1], sh));
      }
      ZQ_CUDA(cudaStreamWaitEvent(st, ev_ready[si], 0));
    } else {
      if (int rc = prep(bi, cur, st, Pk, pcap)) return rc;
    }
    Z* const Wa = cur.Wa;
    Z* const Wb = cur.Wb;
    Z* const Ta = cur.Ta;
    Z* const Tb = cur.Tb;
    Args g{};
    // C1e = Wa^H Xa_sub + Wb^H Xb_sub ; C1o = Wa^T Xb_sub - Wb^T Xa_sub   (kb x L)
    Z* Xas = Xa + (pb + 1) + (int64_t)(pb + 1) * ldx;
    Z* Xbs = Xb + (pb + 1) + (int64_t)(pb + 1) * ldx;
    Z* C1eu = C1e;
    Z* C1ou = C1o;
    int64_t ldc1 = kb;
    if (use_tc) {
      if constexpr (std::is_same<R, float>::value) {
        // both halves in one tensor-core product, formed transposed so that the
        // long inner dimension L is contiguous in X and W:
        //   [C1e; C1o]^T (L x 2kb) = [Xa_sub^T | Xb_sub^T] [[conj(Wa), -Wb]; [conj(Wb), Wa]]
        // stored as C1 = [C1e; C1o] (2kb x L, ld 2kb) in the C1e/C1o area
        ldc1 = 2 * kb;
        C1eu = C1e;
        C1ou = C1e + kb;
        Tc32Args t{};
        t.cplx = 1; t.m = L; t.n = 2 * kb; t.nseg = 2;
        t.seg[0].a = tsrc(Xas, ldx, 1);
        t.seg[0].b = tsrc(Wa, L, 1, 1);
        t.seg[0].b2 = tsrc(Wb, L, 1, 0, -1.f);
        t.seg[0].nsplit = kb; t.seg[0].k = L;
        t.seg[1].a = tsrc(Xbs, ldx, 1);
        t.seg[1].b = tsrc(Wb, L, 1, 1);
        t.seg[1].b2 = tsrc(Wa, L, 1);
        t.seg[1].nsplit = kb; t.seg[1].k = L;
        t.alpha = make_float2(1.f, 0.f); t.beta = make_float2(0.f, 0.f);
        t.C = reinterpret_cast<float*>(C1e); t.ldc = ldc1; t.ctrans = 1;
        // split K over enough CTAs to fill the GPU (partials in the split-K buffer)
        const int tiles = ceil_div(L, 128), kblk = 2 * ceil_div(L, 16);
        int splits = 1;
        while (tiles * splits < 2 * 152 && kblk / (2 * splits) >= 4 && (int64_t)(2 * splits) * L * 2 * kb <= pcap) splits *= 2;
        // shorter accumulations in tensor memory, summed in FP32 by the reduce
        if (const int per = formq_kblocks_per_split())
          while (kblk / splits > per && (int64_t)(2 * splits) * L * 2 * kb <= pcap) splits *= 2;
        t.splits = splits;
        t.P = reinterpret_cast<float*>(Pk);
        t.err = tc_err;
        prof_begin(PC_FORMQ_GEMM, st);
        const int rc = tc32_gemm(t, st);
        prof_end(PC_FORMQ_GEMM, st);
        if (rc) return rc;
      }
    } else {
      g = Args{};
      g.P = Pk; g.pcap = pcap;
      g.m = kb; g.n = L; g.k1 = L; g.k2 = L;
      g.A1 = Wa; g.lda1 = L; g.B1 = Xas; g.ldb1 = ldx;
      g.A2 = Wb; g.lda2 = L; g.B2 = Xbs; g.ldb2 = ldx;
      g.s2 = (R)1; g.alpha = one; g.beta = zero;
      g.C = C1e; g.ldc = kb;
      if (int rc = zgemm(OP_C, OP_N, OP_C, OP_N, g, 1, st)) return rc;
      g.A1 = Wa; g.B1 = Xbs; g.A2 = Wb; g.B2 = Xas; g.s2 = (R)-1; g.C = C1o;
      if (int rc = zgemm(OP_T, OP_N, OP_T, OP_N, g, 1, st)) return rc;
    }
    // C2e = Ta C1e - conj(Tb) C1o ; C2o = Tb C1e + conj(Ta) C1o   (kb x L)
    g = Args{};
    g.P = Pk; g.pcap = pcap;
    g.m = kb; g.n = L; g.k1 = kb; g.k2 = kb;
    g.A1 = Ta; g.lda1 = kb; g.B1 = C1eu; g.ldb1 = ldc1;
    g.A2 = Tb; g.lda2 = kb; g.B2 = C1ou; g.ldb2 = ldc1;
    g.s2 = (R)-1; g.alpha = one; g.beta = zero;
    g.C = C2e; g.ldc = kb;
    if (int rc = zgemm(OP_N, OP_N, OP_R, OP_N, g, 1, st)) return rc;
    g.A1 = Tb; g.A2 = Ta; g.s2 = (R)1; g.C = C2o;
    if (int rc = zgemm(OP_N, OP_N, OP_R, OP_N, g, 1, st)) return rc;
    // Xa_sub -= Wa C2e - conj(Wb) C2o ; Xb_sub -= Wb C2e + conj(Wa) C2o   (L x L)
    if (use_tc_x) {
      if constexpr (std::is_same<R, float>::value) {
        for (int half = 0; half < 2; ++half) {
          Tc32Args t{};
          t.cplx = 1; t.m = L; t.n = L; t.nseg = 2;
          t.seg[0].a = tsrc(half ? Wb : Wa, L, 0);
          t.seg[0].b = tsrc(C2e, kb, 1);
          t.seg[0].k = kb;
          t.seg[1].a = tsrc(half ? Wa : Wb, L, 0, 1, half ? 1.f : -1.f);
          t.seg[1].b = tsrc(C2o, kb, 1);
          t.seg[1].k = kb;
          t.alpha = make_float2(-1.f, 0.f); t.beta = make_float2(1.f, 0.f);
          t.C = reinterpret_cast<float*>(half ? Xbs : Xas); t.ldc = ldx;
          t.splits = 1;
          t.err = tc_err;
          prof_begin(PC_FORMQ_GEMM, st);
          const int rc = tc32_gemm(t, st);
          prof_end(PC_FORMQ_GEMM, st);
          if (rc) return rc;
        }
      }
      if (ahead) ZQ_CUDA(cudaEventRecord(ev_free[si], st));  // this slot may be refilled
      continue;
    }
    g = Args{};
    g.P = Pk; g.pcap = pcap;
    g.m = L; g.n = L; g.k1 = kb; g.k2 = kb;
    g.A1 = Wa; g.lda1 = L; g.B1 = C2e; g.ldb1 = kb;
    g.A2 = Wb; g.lda2 = L; g.B2 = C2o; g.ldb2 = kb;
    g.s2 = (R)-1; g.alpha = mone; g.beta = one;
    g.C = Xas; g.ldc = ldx;
    if (int rc = zgemm(OP_N, OP_N, OP_R, OP_N, g, 1, st)) return rc;
    g.A1 = Wb; g.A2 = Wa; g.s2 = (R)1; g.C = Xbs;
    if (int rc = zgemm(OP_N, OP_N, OP_R, OP_N, g, 1, st)) return rc;
    if (ahead) ZQ_CUDA(cudaEventRecord(ev_free[si], st));  // this slot may be refilled
  }
  return ZQ_OK;
}

template <typename R>
int apply_z(const cplx<R>* X, int64_t ldx, const R* Z, int64_t ldz, int n, cplx<R>* out, int64_t ldo,
            DgemmDescT<R>* dev_desc, cudaStream_t st, int* tc_err) {
  if (n <= 0) return ZQ_OK;
  if constexpr (std::is_same<R, float>::value) {
    if (tc_err && fp32_products_on_tensor_cores(TC_USE_APPLYZ)) {
      // one real product on the tensor cores: (4n x n) real view of X times Z
      Tc32Args t{};
      t.cplx = 0; t.m = 4 * n; t.n = n; t.nseg = 1;
      t.seg[0].a.p = reinterpret_cast<const float*>(X); t.seg[0].a.ld = 2 * ldx; t.seg[0].a.kfast = 0;
      t.seg[0].a.sign = 1.f;
      t.seg[0].b.p = Z; t.seg[0].b.ld = ldz; t.seg[0].b.kfast = 1; t.seg[0].b.sign = 1.f;
      t.seg[0].k = n;
      t.alpha = make_float2(1.f, 0.f); t.beta = make_float2(0.f, 0.f);
      t.C = reinterpret_cast<float*>(out); t.ldc = 2 * ldo;
      t.splits = 1;
      t.err = tc_err;
      prof_begin(PC_APPLYZ, st);
      const int rc = tc32_gemm(t, st);
      prof_end(PC_APPLYZ, st);
      return rc;
    }
  }
  DgemmDescT<R> d{};
  d.A = reinterpret_cast<const R*>(X); d.lda = 2 * ldx;
  d.B = Z; d.ldb = ldz;
  d.C = reinterpret_cast<R*>(out); d.ldc = 2 * ldo;
  d.m = 4 * n; d.n = n; d.k = n;
  d.alpha = 1; d.beta = 0;
  prof_begin(PC_APPLYZ, st);
  const int rc = dgemm_grouped<R>(&d, 1, dev_desc, st);
  prof_end(PC_APPLYZ, st);
  return rc;
}

template int form_q<double>(const cplx<double>*, int64_t, int, const double*, cplx<double>*, int64_t, int, void*, cudaStream_t, int*);
template int form_q<float>(const cplx<float>*, int64_t, int, const double*, cplx<float>*, int64_t, int, void*, cudaStream_t, int*);
template int apply_z<double>(const cplx<double>*, int64_t, const double*, int64_t, int, cplx<double>*, int64_t, DgemmDescT<double>*, cudaStream_t, int*);
template int apply_z<float>(const cplx<float>*, int64_t, const float*, int64_t, int, cplx<float>*, int64_t, DgemmDescT<float>*, cudaStream_t, int*);

__global__ void k_symfill(double2* D, int64_t ld, int n) {
  const int64_t total = (int64_t)n * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(t % n), i = (int)(t / n);
    const double2 u = D[j + (int64_t)i * ld];
    const double2 v = D[n + j + (int64_t)i * ld];
    D[j + (int64_t)(n + i) * ld] = make_double2(-v.x, v.y);      // -conj(V)
    D[n + j + (int64_t)(n + i) * ld] = make_double2(u.x, -u.y);  // conj(U)
  }
}

int symmetry_fill(double2* D, int64_t ld, int n, cudaStream_t st) {
  if (n <= 0) return ZQ_OK;
  const int64_t total = (int64_t)n * n;
  const int blocks = (int)((total + 255) / 256 > 8192 ? 8192 : (total + 255) / 256);
  k_symfill<<<blocks, 256, 0, st>>>(D, ld, n);
  ZQ_LAUNCH_CHECK();
  return ZQ_OK;
}

}  // namespace zq
