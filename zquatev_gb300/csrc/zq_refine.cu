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
__global__ void k_d_to_f(const double* __restrict__ src, float* __restrict__ dst, int64_t n) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    dst[t] = (float)src[t];
}
// x += (double) y   (2D, complex)
__global__ void k_add_c64_to_c128(const float2* __restrict__ y, int64_t ldy, double2* __restrict__ x, int64_t ldx,
                                  int rows, int cols) {
  const int64_t total = (int64_t)rows * cols;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(t % rows), c = (int)(t / rows);
    const float2 v = y[r + (int64_t)c * ldy];
    double2 w = x[r + (int64_t)c * ldx];
    w.x += (double)v.x; w.y += (double)v.y;
    x[r + (int64_t)c * ldx] = w;
  }
}

// H X from P1 = [A;B] U and P2 = [A;B] conj(V) (both 2n x n, ld):
//   (HX)_top = P1_top - conj(P2_bot),  (HX)_bot = P1_bot + conj(P2_top)
__global__ void k_hx_combine(const double2* __restrict__ P1, const double2* __restrict__ P2, int64_t ldp, int n,
                             double2* __restrict__ HX, int64_t ldh) {
  const int64_t total = (int64_t)n * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(t % n), c = (int)(t / n);
    const double2 p1t = P1[r + (int64_t)c * ldp], p1b = P1[n + r + (int64_t)c * ldp];
    const double2 p2t = P2[r + (int64_t)c * ldp], p2b = P2[n + r + (int64_t)c * ldp];
    HX[r + (int64_t)c * ldh] = make_double2(p1t.x - p2b.x, p1t.y + p2b.y);
    HX[n + r + (int64_t)c * ldh] = make_double2(p1b.x + p2t.x, p1b.y - p2t.y);
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
  double ss = 0.0, rr = 0.0, lm = 0.0;
  const int64_t total = (int64_t)n * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % n), j = (int)(t / n);
    const int64_t o = i + (int64_t)j * ld;
    double2 s1 = S1[o], g1 = G1[o];
    if (i == j) { s1.x -= lam[j]; g1.x -= 1.0; }
    const double2 s2 = S2[o], g2 = G2[o];
    ss = fmax(ss, fmax(fmax(fabs(s1.x), fabs(s1.y)), fmax(fabs(s2.x), fabs(s2.y))));
    rr = fmax(rr, fmax(fmax(fabs(g1.x), fabs(g1.y)), fmax(fabs(g2.x), fabs(g2.y))));
    if (i == 0) lm = fmax(lm, fabs(lam[j]));
  }
  ss = block_max(ss, sh);
  rr = block_max(rr, sh);
  lm = block_max(lm, sh);
  if (threadIdx.x == 0) {
    part[3 * blockIdx.x + 0] = ss;
    part[3 * blockIdx.x + 1] = rr;
    part[3 * blockIdx.x + 2] = lm;
  }
}

// E_top (n x n) and E_bot (n x n), written as complex64 for the FP32 update,
// plus per-block max |E| off the Kramers pairs (convergence measure).
__global__ void k_oa_build_e(const double2* __restrict__ S1, const double2* __restrict__ S2,
                             const double2* __restrict__ G1, const double2* __restrict__ G2, int64_t ld, int n,
                             const double* __restrict__ lam, const double* __restrict__ part, int nparts,
                             float2* __restrict__ Et, float2* __restrict__ Eb, int64_t lde, double* __restrict__ emax) {
  __shared__ double sh[32];
  __shared__ double s_delta;
  if (threadIdx.x == 0) {
    double ss = 0.0, rr = 0.0, lm = 0.0;
    for (int q = 0; q < nparts; ++q) { ss = fmax(ss, part[3 * q]); rr = fmax(rr, part[3 * q + 1]); lm = fmax(lm, part[3 * q + 2]); }
    // 2-norm estimates of the 2n x 2n perturbations from their largest entries
    s_delta = 2.0 * sqrt(2.0 * n) * (ss + lm * rr);
  }
  __syncthreads();
  const double delta = s_delta;
  double em = 0.0;
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
    double2 e1, e2;
    if (i != j && fabs(gap) > delta) {
      const double2 s1 = S1[o];
      e1 = make_double2((s1.x + lj * r1.x) / gap, (s1.y + lj * r1.y) / gap);
    } else {
      e1 = make_double2(0.5 * r1.x, 0.5 * r1.y);
    }
    if (fabs(gap) > delta) {
      const double2 s2 = S2[o];
      e2 = make_double2((s2.x + lj * r2.x) / gap, (s2.y + lj * r2.y) / gap);
    } else {
      e2 = make_double2(0.5 * r2.x, 0.5 * r2.y);
    }
    Et[i + (int64_t)j * lde] = make_float2((float)e1.x, (float)e1.y);
    Eb[i + (int64_t)j * lde] = make_float2((float)e2.x, (float)e2.y);
    em = fmax(em, fmax(fabs(e1.x), fabs(e1.y)));
    em = fmax(em, fmax(fabs(e2.x), fabs(e2.y)));
  }
  em = block_max(em, sh);
  if (threadIdx.x == 0) emax[blockIdx.x] = em;
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
  b += sizeof(float2) * 2 * nn;         // Et, Eb
  b += sizeof(float2) * 2 * nn * 2;     // Xf, XEf (2n x n each)
  b += sizeof(float) * nn;              // Zf
  b += tridiag_workspace_bytes<float>(n, 64);
  b += form_q_workspace_bytes(n, nbq);  // sized for double2, enough for float2
  b += sizeof(double) * (16 * (size_t)n + 3 * 8192 + 8192 + 64);
  b += sizeof(int) * (size_t)n;
  b += 64 * 256;
  return b;
}

// accurate complex product: native FP64 (mode 0) or Ozaki-sliced tensor-core products (mode 1).
// Structured outputs (G1, S1 Hermitian; G2, S2 antisymmetric) are made exactly
// structured from their lower triangles, so that the symmetric part of E is R
// exactly and the orthogonality of the update does not depend on eigenvalue gaps.
static int zgemm_acc(int mode, int opa1, int opb1, int opa2, int opb2, const ZgemmArgs& g, void* ows, size_t ows_bytes,
                     cudaStream_t st, int slices, int structured, int reuse_a) {
  if (mode == 1) {
    OzOpts o{};
    o.slices = slices; o.structured = structured; o.reuse_a = reuse_a;
    return zgemm_ozaki(opa1, opb1, opa2, opb2, g, ows, ows_bytes, st, o);
  }
  if (int rc = zgemm<double>(opa1, opb1, opa2, opb2, g, 1, st)) return rc;
  if (structured != 0) return structured_fill(g.C, g.ldc, g.m, structured, st);
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
  float2* Et = reinterpret_cast<float2*>(take(sizeof(float2) * nn));
  float2* Eb = reinterpret_cast<float2*>(take(sizeof(float2) * nn));
  float2* Xf = reinterpret_cast<float2*>(take(sizeof(float2) * 2 * nn));
  float2* XEf = reinterpret_cast<float2*>(take(sizeof(float2) * 2 * nn));
  float* Zf = reinterpret_cast<float*>(take(sizeof(float) * nn));
  void* tri_ws = take(tridiag_workspace_bytes<float>(n, 64));
  void* fq_ws = take(form_q_workspace_bytes(n, ra.nbq));
  double* sm = reinterpret_cast<double*>(take(sizeof(double) * (16 * (size_t)n + 3 * 8192 + 8192 + 64)));
  int* rank = reinterpret_cast<int*>(take(sizeof(int) * (size_t)n));
  double* d = sm; sm += n;
  double* e = sm; sm += 4 * (size_t)n;
  double* tau = sm; sm += n;
  double* offd = sm; sm += n;
  double* phi = sm; sm += 4 * (size_t)n;
  double* lam = sm; sm += n;
  double* lam2 = sm; sm += n;
  double* part = sm; sm += 3 * 8192;
  double* emax = sm;
  const int64_t ldd = ra.ldd;
  double2* X = ra.dD;  // (U; V) lives in the output's left half

  // A. FP32 eigendecomposition
  ZQ_CUDA(cudaMemcpy2DAsync(H0, sizeof(double2) * n2, ra.dD, sizeof(double2) * ldd, sizeof(double2) * n2, n,
                            cudaMemcpyDeviceToDevice, st));
  k_c128_to_c64<<<grid_for((int64_t)n2 * n), 256, 0, st>>>(H0, n2, Mf, n2, n2, n);
  ZQ_LAUNCH_CHECK();
  TridiagView<float> vf = tridiag_bind<float>(tri_ws, Mf, n, n2, 64, d, e, tau);
  if (int rc = tridiagonalize<float>(vf, ra.nb, st)) return rc;
  if (int rc = phase_reduce(e, n, offd, phi, st)) return rc;
  double* Zd = nullptr;
  if (int rc = ra.dc->run(d, offd, lam, Zd, st)) return rc;
  float2* XfQ = Mf + (int64_t)n * n2;  // right half of Mf
  if (int rc = form_q<float>(Mf, n2, n, phi, XfQ, n2, ra.nbq, fq_ws, st)) return rc;
  k_d_to_f<<<grid_for((int64_t)nn), 256, 0, st>>>(Zd, Zf, (int64_t)nn);
  ZQ_LAUNCH_CHECK();
  if (int rc = apply_z<float>(XfQ, n2, Zf, n, n, Mf, n2, ra.fdesc, st)) return rc;
  k_c64_to_c128<<<grid_for((int64_t)n2 * n), 256, 0, st>>>(Mf, n2, X, ldd, n2, n);
  ZQ_LAUNCH_CHECK();

  // B. refinement
  prof_begin(PC_REFINE, st);
  const double2 one = make_double2(1.0, 0.0), zero = make_double2(0.0, 0.0);
  const int nparts = 1024;
  ra.iters = 0;
  ra.last_emax = 1.0;
  const int ne = 1024;
  std::vector<double> hemax(ne);
  for (int it = 0; it < ra.max_iter; ++it) {
    // the first correction only has to reach ~1e-8 (the next step squares the
    // error): 5 slices (35 bits); later steps use 8 (56 bits)
    const int sl = (it == 0) ? 5 : 8;
    double2* U = X;
    double2* V = X + n;
    ZgemmArgs g{};
    // G1 = X^H X
    g = ZgemmArgs{};
    g.m = n; g.n = n; g.k1 = n2; g.A1 = X; g.lda1 = ldd; g.B1 = X; g.ldb1 = ldd;
    g.alpha = one; g.beta = zero; g.C = G1; g.ldc = n;
    if (int rc = zgemm_acc(ra.mode, OP_C, OP_N, OP_N, OP_N, g, ra.ows, ra.ows_bytes, st, sl, 1, 0)) return rc;
    // G2 = U^T V - V^T U
    g = ZgemmArgs{};
    g.m = n; g.n = n; g.k1 = n; g.k2 = n;
    g.A1 = U; g.lda1 = ldd; g.B1 = V; g.ldb1 = ldd; g.A2 = V; g.lda2 = ldd; g.B2 = U; g.ldb2 = ldd; g.s2 = -1.0;
    g.alpha = one; g.beta = zero; g.C = G2; g.ldc = n;
    if (int rc = zgemm_acc(ra.mode, OP_T, OP_N, OP_T, OP_N, g, ra.ows, ra.ows_bytes, st, sl, -1, 0)) return rc;
    // P1 = [A;B] U, P2 = [A;B] conj(V)
    g = ZgemmArgs{};
    g.m = n2; g.n = n; g.k1 = n; g.A1 = H0; g.lda1 = n2; g.B1 = U; g.ldb1 = ldd;
    g.alpha = one; g.beta = zero; g.C = P1; g.ldc = n2;
    if (int rc = zgemm_acc(ra.mode, OP_N, OP_N, OP_N, OP_N, g, ra.ows, ra.ows_bytes, st, sl, 0, 0)) return rc;
    g.B1 = V; g.C = P2;
    if (int rc = zgemm_acc(ra.mode, OP_N, OP_R, OP_N, OP_N, g, ra.ows, ra.ows_bytes, st, sl, 0, 1)) return rc;
    k_hx_combine<<<grid_for((int64_t)nn), 256, 0, st>>>(P1, P2, n2, n, HX, n2);
    ZQ_LAUNCH_CHECK();
    // S1 = X^H HX ; S2 = U^T HX_bot - V^T HX_top
    g = ZgemmArgs{};
    g.m = n; g.n = n; g.k1 = n2; g.A1 = X; g.lda1 = ldd; g.B1 = HX; g.ldb1 = n2;
    g.alpha = one; g.beta = zero; g.C = S1; g.ldc = n;
    if (int rc = zgemm_acc(ra.mode, OP_C, OP_N, OP_N, OP_N, g, ra.ows, ra.ows_bytes, st, sl, 1, 0)) return rc;
    g = ZgemmArgs{};
    g.m = n; g.n = n; g.k1 = n; g.k2 = n;
    g.A1 = U; g.lda1 = ldd; g.B1 = HX + n; g.ldb1 = n2; g.A2 = V; g.lda2 = ldd; g.B2 = HX; g.ldb2 = n2; g.s2 = -1.0;
    g.alpha = one; g.beta = zero; g.C = S2; g.ldc = n;
    if (int rc = zgemm_acc(ra.mode, OP_T, OP_N, OP_T, OP_N, g, ra.ows, ra.ows_bytes, st, sl, -1, 0)) return rc;
    // lambda, delta, E
    k_oa_lambda<<<ceil_div(n, 256), 256, 0, st>>>(S1, G1, n, n, lam);
    ZQ_LAUNCH_CHECK();
    k_oa_norms<<<nparts, 256, 0, st>>>(S1, S2, G1, G2, n, n, lam, part);
    ZQ_LAUNCH_CHECK();
    k_oa_build_e<<<ne, 256, 0, st>>>(S1, S2, G1, G2, n, n, lam, part, nparts, Et, Eb, n, emax);
    ZQ_LAUNCH_CHECK();
    ZQ_CUDA(cudaMemcpyAsync(hemax.data(), emax, sizeof(double) * ne, cudaMemcpyDeviceToHost, st));
    ZQ_CUDA(cudaStreamSynchronize(st));
    double em = 0.0;
    for (double v : hemax) em = v > em ? v : em;
    ra.last_emax = em;
    // X += X E_top + J conj(X) E_bot  (FP32 product, FP64 accumulation)
    k_c128_to_c64<<<grid_for((int64_t)n2 * n), 256, 0, st>>>(X, ldd, Xf, n2, n2, n);
    ZQ_LAUNCH_CHECK();
    ZgemmArgsT<float> f{};
    const float2 fone = make_float2(1.f, 0.f), fzero = make_float2(0.f, 0.f);
    f.m = n; f.n = n; f.k1 = n; f.k2 = n;
    f.A1 = Xf; f.lda1 = n2; f.B1 = Et; f.ldb1 = n; f.A2 = Xf + n; f.lda2 = n2; f.B2 = Eb; f.ldb2 = n; f.s2 = -1.f;
    f.alpha = fone; f.beta = fzero; f.C = XEf; f.ldc = n2;
    if (int rc = zgemm<float>(OP_N, OP_N, OP_R, OP_N, f, 1, st)) return rc;
    f.A1 = Xf + n; f.A2 = Xf; f.s2 = 1.f; f.C = XEf + n;
    if (int rc = zgemm<float>(OP_N, OP_N, OP_R, OP_N, f, 1, st)) return rc;
    k_add_c64_to_c128<<<grid_for((int64_t)n2 * n), 256, 0, st>>>(XEf, n2, X, ldd, n2, n);
    ZQ_LAUNCH_CHECK();
    ra.iters = it + 1;
    if (em <= ra.tol && (ra.mode == 0 || sl == 8)) break;
  }
  prof_end(PC_REFINE, st);
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
