// Stage (c): GPU divide-and-conquer eigensolver for a real symmetric
// tridiagonal matrix (all FP64).
//
// Replaces LAPACK zhbev("V","L",n,kd=1) at zquatev.cc:74-84. The reference's
// tridiagonal is complex Hermitian; the quaternion reduction here produces a
// quaternion tridiagonal whose off-diagonal phases are removed exactly by a
// diagonal quaternion similarity (zq_backtransform.cu), leaving this real
// symmetric problem T = Z diag(lambda) Z^T.
//
// Method (Cuppen's divide and conquer with Gu-Eisenstat eigenvectors, written
// from the published algorithm):
//   * scale T to max |entry| = 1;
//   * tear every off-diagonal e_i: T = blockdiag(T1, T2) + e_i u u^T, so the
//     recursion bottoms out at 1x1 leaves (d_i - e_{i-1} - e_i);
//   * merge bottom-up, one batched launch sequence per tree depth:
//       prepare  - z from the children's eigenvectors, merge-sort the poles,
//                  deflate small z and close poles (Givens), sort the deflated;
//       secular  - one thread per root of 1 + rho sum z_k^2/(d_k - x), solved in
//                  coordinates shifted to the nearer pole with a safeguarded
//                  two-pole rational model (bisection fallback);
//       zhat     - recompute z from the roots (Gu-Eisenstat) for orthogonality;
//       vectors  - eigenvectors of the rank-one problem, scattered into the
//                  merge matrix M in final (ascending) order;
//       rotate   - fold the deflation rotations into M's rows;
//       gemm     - Z_node = blockdiag(Z1, Z2) * M  (grouped DGEMM).
#include "zq_common.cuh"
#include "zq_kernels.h"
#include "zq_tc32.h"

#include <algorithm>
#include <atomic>
#include <type_traits>
#include <vector>

namespace zq {

constexpr double DEPS = 1.1102230246251565e-16;  // 2^-53

__device__ __forceinline__ int dc_find_node(const DcNode* nodes, int cnt, int pos) {
  // nodes sorted by a; returns index of node with a <= pos < b, or -1
  int lo = 0, hi = cnt - 1, r = -1;
  while (lo <= hi) {
    const int mid = (lo + hi) >> 1;
    if (nodes[mid].a <= pos) { r = mid; lo = mid + 1; } else hi = mid - 1;
  }
  if (r >= 0 && pos < nodes[r].b) return r;
  return -1;
}

template <typename ZT>
__global__ void k_dc_leaf(const DcNode* nodes, int cnt, const double* dmod, ZT* Zout, double* lamout, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cnt) return;
  const int a = nodes[i].a;
  Zout[a + (int64_t)a * n] = (ZT)1;
  lamout[a] = dmod[a];
}

// one CTA per internal node. The merged poles (value, z, source column) are
// staged in shared memory when the node fits (m <= scap). Deflation runs in
// parallel unless two kept poles are close enough to need a rotation (see the
// fast path); then the sequential scan runs (each rotation changes the next
// comparison) in one thread, with its operands a shared-memory load away, and
// the deflated list is ranked from shared memory.
constexpr int DC_SCAP = 8192;  // largest node staged in shared memory (20 bytes per pole)
template <typename ZT>
__global__ void __launch_bounds__(256) k_dc_prepare(DcNode* nodes, DcWork w, const ZT* Zin, const double* lamin, int n,
                                                    int scap) {
  extern __shared__ double dc_sm[];
  DcNode& nd = nodes[blockIdx.x];
  const int a = nd.a, c = nd.c, b = nd.b;
  const int m = b - a, n1 = c - a, n2 = b - c;
  const int tid = threadIdx.x;
  const double rho2 = 2.0 * nd.rho;
  const double rs2 = 0.70710678118654752440;
  const bool staged = m <= scap;
  double* D = staged ? dc_sm : w.sd + a;
  double* Zs = staged ? dc_sm + scap : w.sz + a;
  int* P = staged ? reinterpret_cast<int*>(dc_sm + 2 * scap) : w.perm + a;
  __shared__ double s_red[8];
  __shared__ int s_cnt[3];
  // merge the two sorted eigenvalue lists; z in sorted order
  double dm = 0.0, zm = 0.0;
  for (int i = tid; i < m; i += blockDim.x) {
    double val, z;
    int pos;
    if (i < n1) {
      val = lamin[a + i];
      z = (double)Zin[(c - 1) + (int64_t)(a + i) * n] * rs2;
      // count of right values strictly less than val
      int lo = 0, hi = n2;
      while (lo < hi) { const int mid = (lo + hi) >> 1; if (lamin[c + mid] < val) lo = mid + 1; else hi = mid; }
      pos = i + lo;
    } else {
      const int i2 = i - n1;
      val = lamin[c + i2];
      z = (double)Zin[c + (int64_t)(a + i) * n] * rs2;
      int lo = 0, hi = n1;
      while (lo < hi) { const int mid = (lo + hi) >> 1; if (lamin[a + mid] <= val) lo = mid + 1; else hi = mid; }
      pos = i2 + lo;
    }
    D[pos] = val;
    Zs[pos] = z;
    P[pos] = i;
    dm = fmax(dm, fabs(val));
    zm = fmax(zm, fabs(z));
  }
  const double dmax = block_max(dm, s_red);  // (its barriers also publish D, Zs, P)
  const double zmax = block_max(zm, s_red);
  const double tol = 8.0 * DEPS * fmax(dmax, zmax);
  // Fast path (all threads): z-deflation flags, compaction by a block scan,
  // then the close-pole test on every consecutive pair of the kept poles with
  // their original values. The sequential scan below changes a pole only
  // after a test passes, and every test before the first pass sees original
  // values: so if no pair passes here, the scan would rotate nothing and its
  // lists are exactly these (the deflated ones already in ascending order).
  // Any passing pair sends the node to the sequential scan.
  {
    const int per = (m + (int)blockDim.x - 1) / (int)blockDim.x;  // contiguous entries per thread
    const int i0 = tid * per, i1 = (i0 + per < m) ? i0 + per : m;
    int keep = 0;
    for (int i = i0; i < i1; ++i) keep += !(rho2 * fabs(Zs[i]) <= tol);
    // exclusive scan of the per-thread counts (warp shuffles, then the warps)
    const int lane = tid & 31, wid = tid >> 5;
    int incl = keep;
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    __shared__ int s_wsum[8], s_flag;
    if (lane == 31) s_wsum[wid] = incl;
    if (tid == 0) s_flag = 0;
    __syncthreads();
    int wbase = 0;
    for (int q = 0; q < wid; ++q) wbase += s_wsum[q];
    int Ktot = 0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) Ktot += s_wsum[q];
    int kpos = wbase + incl - keep;   // kept poles before this thread's chunk
    int dpos = i0 - kpos;             // deflated ones before it
    for (int i = i0; i < i1; ++i) {
      if (!(rho2 * fabs(Zs[i]) <= tol)) {
        w.nd_val[a + kpos] = D[i]; w.nd_z[a + kpos] = Zs[i]; w.nd_col[a + kpos] = P[i]; ++kpos;
      } else {
        w.df_val[a + dpos] = D[i]; w.df_col[a + dpos] = P[i];
        w.df_sval[a + dpos] = D[i]; w.df_scol[a + dpos] = P[i]; ++dpos;
      }
    }
    __syncthreads();
    // pair test on the kept poles (k - 1, k), as the sequential scan forms it
    for (int q = tid + 1; q < Ktot; q += blockDim.x) {
      double sv = w.nd_z[a + q - 1], cc = w.nd_z[a + q];
      const double tau = hypot(cc, sv);
      cc /= tau; sv = -sv / tau;
      const double t = w.nd_val[a + q] - w.nd_val[a + q - 1];
      if (fabs(t * cc * sv) <= tol) s_flag = 1;
    }
    __syncthreads();
    if (!s_flag) {
      if (tid == 0) { nd.K = Ktot; nd.ndefl = m - Ktot; nd.nrot = 0; nd.rho2 = rho2; }
      return;
    }
  }
  if (tid == 0) {
    int K = 0, nd_ = 0, nr = 0;
    int pj = -1;
    for (int j = 0; j < m; ++j) {
      if (rho2 * fabs(Zs[j]) <= tol) {
        w.df_val[a + nd_] = D[j]; w.df_col[a + nd_] = P[j]; ++nd_;
        continue;
      }
      if (pj < 0) { pj = j; continue; }
      double s = Zs[pj], cc = Zs[j];
      const double tau = hypot(cc, s);
      cc /= tau; s = -s / tau;
      const double t = D[j] - D[pj];
      if (fabs(t * cc * s) <= tol) {
        Zs[j] = tau; Zs[pj] = 0.0;
        w.rot_p[a + nr] = P[pj]; w.rot_j[a + nr] = P[j];
        w.rot_c[a + nr] = cc; w.rot_s[a + nr] = s; ++nr;
        const double tt = D[pj] * cc * cc + D[j] * s * s;
        D[j] = D[pj] * s * s + D[j] * cc * cc;
        D[pj] = tt;
        w.df_val[a + nd_] = D[pj]; w.df_col[a + nd_] = P[pj]; ++nd_;
        pj = j;
      } else {
        w.nd_val[a + K] = D[pj]; w.nd_z[a + K] = Zs[pj]; w.nd_col[a + K] = P[pj]; ++K;
        pj = j;
      }
    }
    if (pj >= 0) { w.nd_val[a + K] = D[pj]; w.nd_z[a + K] = Zs[pj]; w.nd_col[a + K] = P[pj]; ++K; }
    nd.K = K; nd.ndefl = nd_; nd.nrot = nr; nd.rho2 = rho2;
    s_cnt[0] = nd_;
  }
  __syncthreads();
  // sort the deflated list (values, columns) by rank; ties by index
  const int nd_ = s_cnt[0];
  const double* fv = w.df_val + a;
  if (staged) {  // the staged poles are dead now: their space holds the deflated values
    for (int i = tid; i < nd_; i += blockDim.x) dc_sm[i] = w.df_val[a + i];
    __syncthreads();
    fv = dc_sm;
  }
  for (int i = tid; i < nd_; i += blockDim.x) {
    const double v = fv[i];
    int rank = 0;
    for (int l = 0; l < nd_; ++l) {
      const double u = fv[l];
      rank += (u < v) || (u == v && l < i);
    }
    w.df_sval[a + rank] = v;
    w.df_scol[a + rank] = w.df_col[a + i];
  }
}

// secular equation: one warp per root; the lanes split the sums over the
// poles (butterfly reductions leave identical totals on every lane, so the
// iteration's control flow stays warp-uniform)
__global__ void __launch_bounds__(128) k_dc_secular(const DcNode* nodes, int cnt, DcWork w) {
  const int pos = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  const int ni = dc_find_node(nodes, cnt, pos);
  if (ni < 0) return;
  const DcNode nd = nodes[ni];
  const int a = nd.a, K = nd.K;
  const int i = pos - a;
  if (i >= K) return;
  const double* D = w.nd_val + a;
  const double* z = w.nd_z + a;
  const double rho = nd.rho2;
  int o;
  double lo, hi;
  if (i < K - 1) {
    const double gap = D[i + 1] - D[i];
    const double mid = 0.5 * gap;
    double fs = 0.0;
    for (int k = lane; k < K; k += 32) fs += rho * z[k] * z[k] / ((D[k] - D[i]) - mid);
    const double f = 1.0 + warp_sum(fs);
    if (f >= 0.0) { o = i; lo = 0.0; hi = mid; }
    else { o = i + 1; lo = -mid; hi = 0.0; }
  } else {
    o = K - 1; lo = 0.0; hi = rho;
  }
  const double Do = D[o];
  double tau = 0.5 * (lo + hi);
  for (int it = 0; it < 200; ++it) {
    double psi = 0.0, phi = 0.0, dpsi = 0.0, dphi = 0.0;
    for (int k = lane; k < K; k += 32) {
      const double del = (D[k] - Do) - tau;
      const double inv = 1.0 / del;
      const double t = rho * z[k] * z[k] * inv;
      if (k <= i) { psi += t; dpsi += t * inv; } else { phi += t; dphi += t * inv; }
    }
    psi = warp_sum(psi); phi = warp_sum(phi); dpsi = warp_sum(dpsi); dphi = warp_sum(dphi);
    const double f = 1.0 + psi + phi;
    if (f == 0.0) break;
    if (f < 0.0) lo = tau; else hi = tau;
    const double errb = 8.0 * DEPS * (1.0 + fabs(psi) + fabs(phi)) + DEPS * fabs(tau) * (dpsi + dphi);
    if (fabs(f) <= errb) break;
    if (hi - lo <= 2.0 * DEPS * fmax(fabs(lo), fabs(hi))) break;
    // two-pole rational model around the current point
    const double di = (D[i] - Do) - tau;
    double eta;
    bool ok = false;
    if (i < K - 1) {
      const double dj = (D[i + 1] - Do) - tau;
      const double B1 = di * di * dpsi, B2 = dj * dj * dphi;
      const double cc0 = f - B1 / di - B2 / dj;
      const double qa = cc0;
      const double qb = cc0 * (di + dj) + B1 + B2;
      const double qc = cc0 * di * dj + B1 * dj + B2 * di;
      // roots of qa x^2 - qb x + qc = 0
      if (qa == 0.0) {
        if (qb != 0.0) { eta = qc / qb; ok = true; }
      } else {
        const double disc = qb * qb - 4.0 * qa * qc;
        if (disc >= 0.0) {
          const double sq = sqrt(disc);
          const double den = (qb >= 0.0) ? (qb + sq) : (qb - sq);
          const double r1 = den / (2.0 * qa);
          const double r2 = (den != 0.0) ? 2.0 * qc / den : r1;
          const bool in1 = (r1 > di && r1 < dj), in2 = (r2 > di && r2 < dj);
          if (in2) { eta = r2; ok = true; } else if (in1) { eta = r1; ok = true; }
        }
      }
    } else {
      const double B1 = di * di * dpsi;
      const double cc0 = f - B1 / di;
      if (cc0 > 0.0) { eta = di + B1 / cc0; ok = true; }
    }
    double tn = ok ? tau + eta : 0.5 * (lo + hi);
    if (!(tn > lo && tn < hi)) tn = 0.5 * (lo + hi);
    if (tn == tau) break;
    tau = tn;
  }
  if (lane == 0) {
    w.r_orig[a + i] = o;
    w.r_tau[a + i] = tau;
    w.r_lam[a + i] = Do + tau;
  }
}

// Gu-Eisenstat: zhat_k from the computed roots; one warp per k, the product
// over the roots split over the lanes
__global__ void __launch_bounds__(128) k_dc_zhat(const DcNode* nodes, int cnt, DcWork w) {
  const int pos = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  const int ni = dc_find_node(nodes, cnt, pos);
  if (ni < 0) return;
  const DcNode nd = nodes[ni];
  const int a = nd.a, K = nd.K;
  const int k = pos - a;
  if (k >= K) return;
  const double* D = w.nd_val + a;
  const double Dk = D[k];
  const int* O = w.r_orig + a;
  const double* T = w.r_tau + a;
  // (lambda_{K-1} - D_k) / rho
  double prod = (lane == 0) ? ((D[O[K - 1]] - Dk) + T[K - 1]) / nd.rho2 : 1.0;
  for (int j = lane; j < K - 1; j += 32) {
    const double num = (D[O[j]] - Dk) + T[j];  // lambda_j - D_k
    const double den = (j < k) ? (D[j] - Dk) : (D[j + 1] - Dk);
    prod *= num / den;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) prod *= __shfl_xor_sync(0xffffffffu, prod, off);
  if (lane == 0) {
    const double zk = w.nd_z[a + k];
    const double zh = sqrt(fmax(prod, 0.0));
    w.zhat[a + k] = (zk >= 0.0) ? zh : -zh;
  }
}

// one CTA per column slot of every internal node: writes a full column of M
template <typename ZT>
__global__ void __launch_bounds__(128) k_dc_vectors(const DcNode* nodes, int cnt, DcWork w, ZT* Mb, double* lamout, int n) {
  const int pos = blockIdx.x;
  const int ni = dc_find_node(nodes, cnt, pos);
  if (ni < 0) return;
  const DcNode nd = nodes[ni];
  const int a = nd.a, m = nd.b - nd.a, K = nd.K, ndf = nd.ndefl;
  const int s = pos - a;
  const int tid = threadIdx.x;
  __shared__ double s_red[4];
  int outpos;
  double val;
  if (s < K) {
    val = w.r_lam[a + s];
    int lo = 0, hi = ndf;  // deflated values strictly below
    while (lo < hi) { const int mid = (lo + hi) >> 1; if (w.df_sval[a + mid] < val) lo = mid + 1; else hi = mid; }
    outpos = s + lo;
  } else {
    const int i = s - K;
    val = w.df_sval[a + i];
    int lo = 0, hi = K;  // roots <= val
    while (lo < hi) { const int mid = (lo + hi) >> 1; if (w.r_lam[a + mid] <= val) lo = mid + 1; else hi = mid; }
    outpos = i + lo;
  }
  ZT* col = Mb + a + (int64_t)(a + outpos) * n;
  for (int r = tid; r < m; r += blockDim.x) col[r] = (ZT)0;
  __syncthreads();
  if (s < K) {
    const double* D = w.nd_val + a;
    const int o = w.r_orig[a + s];
    const double t = w.r_tau[a + s];
    const double Do = D[o];
    double ss = 0.0;
    for (int k = tid; k < K; k += blockDim.x) {
      const double del = (D[k] - Do) - t;
      const double vk = w.zhat[a + k] / del;
      ss += vk * vk;
    }
    ss = warp_sum(ss);
    if ((tid & 31) == 0) s_red[tid >> 5] = ss;
    __syncthreads();
    const double nrm = sqrt(s_red[0] + s_red[1] + s_red[2] + s_red[3]);
    const double inv = 1.0 / nrm;
    for (int k = tid; k < K; k += blockDim.x) {
      const double del = (D[k] - Do) - t;
      col[w.nd_col[a + k]] = (ZT)(w.zhat[a + k] / del * inv);
    }
  } else {
    if (tid == 0) col[w.df_scol[a + (s - K)]] = (ZT)1;
  }
  if (tid == 0) lamout[a + outpos] = val;
}

// apply the deflation rotations (in reverse order) to every column of M
template <typename ZT>
__global__ void k_dc_rotate(const DcNode* nodes, int cnt, DcWork w, ZT* Mb, int n) {
  const int pos = blockIdx.x * blockDim.x + threadIdx.x;
  const int ni = dc_find_node(nodes, cnt, pos);
  if (ni < 0) return;
  const DcNode nd = nodes[ni];
  if (nd.nrot == 0) return;
  const int a = nd.a;
  ZT* col = Mb + a + (int64_t)pos * n;
  for (int r = nd.nrot - 1; r >= 0; --r) {
    const int P = w.rot_p[a + r], J = w.rot_j[a + r];
    const double c = w.rot_c[a + r], s = w.rot_s[a + r];
    const double vp = col[P], vj = col[J];
    col[P] = (ZT)(c * vp - s * vj);
    col[J] = (ZT)(s * vp + c * vj);
  }
}

__global__ void k_dc_scale_in(const double* d, const double* e, int n, double* dmod, double* es, const double* scal) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double inv = (scal[0] > 0.0) ? 1.0 / scal[0] : 1.0;
  const double el = (i > 0) ? e[i - 1] * inv : 0.0;
  const double er = (i < n - 1) ? e[i] * inv : 0.0;
  dmod[i] = d[i] * inv - el - er;
  if (i < n - 1) es[i] = er;
}

__global__ void k_dc_maxabs(const double* d, const double* e, int n, double* out) {
  __shared__ double sh[32];
  double m = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    m = fmax(m, fabs(d[i]));
    if (i < n - 1) m = fmax(m, fabs(e[i]));
  }
  m = block_max(m, sh);
  if (threadIdx.x == 0) out[0] = m;
}

__global__ void k_dc_unscale(double* lam, int n, const double* scal) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && scal[0] > 0.0) lam[i] *= scal[0];
}

__global__ void k_dc_setrho(DcNode* nodes, int cnt, const double* es) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < cnt && nodes[i].b - nodes[i].a > 1) nodes[i].rho = es[nodes[i].c - 1];
}

// ----------------------------------------------------------------------------
// host side: plan (tree, descriptors) and execution
// ----------------------------------------------------------------------------
size_t DcPlan::workspace_doubles(int n) {
  // Z x2, M, lam x2, dmod, es, scal + the per-position DcWork arrays
  const size_t nn = (size_t)n * n;
  return 3 * nn + 2 * (size_t)n + 2 * (size_t)n + 8 + 16 * (size_t)n;
}

int DcPlan::build(int n_) {
  n = n_;
  nodes_host.clear();
  depth_off.clear();
  depth_cnt.clear();
  leaf_off.clear();
  leaf_cnt.clear();
  if (n <= 0) return ZQ_OK;
  // recursive halving, breadth first
  struct Tmp { int a, b, depth; };
  std::vector<Tmp> all;
  std::vector<Tmp> cur = {{0, n, 0}};
  int depth = 0;
  while (!cur.empty()) {
    std::vector<Tmp> nxt;
    for (auto& t : cur) {
      all.push_back(t);
      if (t.b - t.a > 1) {
        const int c = t.a + (t.b - t.a) / 2;
        nxt.push_back({t.a, c, depth + 1});
        nxt.push_back({c, t.b, depth + 1});
      }
    }
    cur.swap(nxt);
    ++depth;
  }
  max_depth = depth - 1;
  // group by depth: internal nodes and leaves separately, each sorted by a
  depth_mmax.clear();
  for (int t = 0; t <= max_depth; ++t) {
    depth_off.push_back((int)nodes_host.size());
    int cnt = 0, mmax = 0;
    for (auto& x : all)
      if (x.depth == t && x.b - x.a > 1) {
        DcNode nd{};
        nd.a = x.a; nd.b = x.b; nd.c = x.a + (x.b - x.a) / 2;
        nodes_host.push_back(nd);
        ++cnt;
        mmax = std::max(mmax, x.b - x.a);
      }
    depth_cnt.push_back(cnt);
    depth_mmax.push_back(mmax);
  }
  for (int t = 0; t <= max_depth; ++t) {
    leaf_off.push_back((int)nodes_host.size());
    int cnt = 0;
    for (auto& x : all)
      if (x.depth == t && x.b - x.a == 1) {
        DcNode nd{};
        nd.a = x.a; nd.b = x.b; nd.c = x.a;
        nodes_host.push_back(nd);
        ++cnt;
      }
    leaf_cnt.push_back(cnt);
  }
  // GEMM descriptors per depth (pointers bound at execution time by offsets)
  gemm_host.clear();
  gemm_off.clear();
  gemm_tiles.clear();
  for (int t = 0; t <= max_depth; ++t) {
    gemm_off.push_back((int)gemm_host.size());
    int tiles = 0;
    for (int q = 0; q < depth_cnt[t]; ++q) {
      const DcNode& nd = nodes_host[depth_off[t] + q];
      const int m = nd.b - nd.a, n1 = nd.c - nd.a, n2 = nd.b - nd.c;
      DgemmDesc top{}, bot{};
      top.m = n1; top.n = m; top.k = n1; top.alpha = 1.0; top.beta = 0.0;
      // offsets stored as element indices; converted to pointers in run()
      top.off_a = nd.a + (int64_t)nd.a * n; top.off_b = nd.a + (int64_t)nd.a * n; top.off_c = nd.a + (int64_t)nd.a * n;
      bot.m = n2; bot.n = m; bot.k = n2; bot.alpha = 1.0; bot.beta = 0.0;
      bot.off_a = nd.c + (int64_t)nd.c * n; bot.off_b = nd.c + (int64_t)nd.a * n; bot.off_c = nd.c + (int64_t)nd.a * n;
      top.lda = top.ldb = top.ldc = n;
      bot.lda = bot.ldb = bot.ldc = n;
      top.tile0 = tiles; tiles += ceil_div(top.m, 64) * ceil_div(top.n, 64);
      bot.tile0 = tiles; tiles += ceil_div(bot.m, 64) * ceil_div(bot.n, 64);
      gemm_host.push_back(top);
      gemm_host.push_back(bot);
    }
    gemm_tiles.push_back(tiles);
  }
  return ZQ_OK;
}

// Binds device pointers into the descriptor copies and uploads everything.
int DcPlan::upload(double* ws, DcNode* dnodes, DgemmDesc* ddescs, cudaStream_t st) {
  base = ws;
  const size_t nn = (size_t)n * n;
  Z[0] = ws; Z[1] = ws + nn; Mb = ws + 2 * nn;
  double* p = ws + 3 * nn;
  lam[0] = p; p += n; lam[1] = p; p += n;
  dmod = p; p += n; es = p; p += n;
  scal = p; p += 8;
  w.sd = p; p += n; w.sz = p; p += n;
  w.nd_val = p; p += n; w.nd_z = p; p += n;
  w.df_val = p; p += n; w.df_sval = p; p += n;
  w.rot_c = p; p += n; w.rot_s = p; p += n;
  w.r_tau = p; p += n; w.r_lam = p; p += n; w.zhat = p; p += n;
  int* ip = reinterpret_cast<int*>(p);
  w.perm = ip; ip += n; w.nd_col = ip; ip += n; w.df_col = ip; ip += n; w.df_scol = ip; ip += n;
  w.rot_p = ip; ip += n; w.rot_j = ip; ip += n; w.r_orig = ip; ip += n;
  nodes_dev = dnodes;
  descs_dev = ddescs;
  // bind pointers: at depth t, A (children) lives in Z[(t+1)&1], output in Z[t&1]
  std::vector<DgemmDesc> bound = gemm_host;
  for (int t = 0; t <= max_depth; ++t) {
    for (int q = 0; q < 2 * depth_cnt[t]; ++q) {
      DgemmDesc& d = bound[gemm_off[t] + q];
      d.A = Z[(t + 1) & 1] + d.off_a;
      d.B = Mb + d.off_b;
      d.C = Z[t & 1] + d.off_c;
    }
  }
  // single-precision views of the same buffers (Z, M as float) for run_single
  Zf[0] = reinterpret_cast<float*>(Z[0]);
  Zf[1] = reinterpret_cast<float*>(Z[1]);
  Mbf = reinterpret_cast<float*>(Mb);
  fdescs_dev = reinterpret_cast<DgemmDescT<float>*>(ddescs + gemm_host.size() + 2);
  std::vector<DgemmDescT<float>> fbound(gemm_host.size());
  for (size_t i = 0; i < gemm_host.size(); ++i) {
    const DgemmDesc& h = gemm_host[i];
    DgemmDescT<float>& f = fbound[i];
    f.lda = h.lda; f.ldb = h.ldb; f.ldc = h.ldc;
    f.off_a = h.off_a; f.off_b = h.off_b; f.off_c = h.off_c;
    f.m = h.m; f.n = h.n; f.k = h.k; f.ta = h.ta; f.tb = h.tb; f.tile0 = h.tile0;
    f.alpha = 1.f; f.beta = 0.f;
  }
  for (int t = 0; t <= max_depth; ++t) {
    for (int q = 0; q < 2 * depth_cnt[t]; ++q) {
      DgemmDescT<float>& d = fbound[gemm_off[t] + q];
      d.A = Zf[(t + 1) & 1] + d.off_a;
      d.B = Mbf + d.off_b;
      d.C = Zf[t & 1] + d.off_c;
    }
  }
  if (!nodes_host.empty())
    ZQ_CUDA(cudaMemcpyAsync(dnodes, nodes_host.data(), sizeof(DcNode) * nodes_host.size(), cudaMemcpyHostToDevice, st));
  if (!bound.empty())
    ZQ_CUDA(cudaMemcpyAsync(ddescs, bound.data(), sizeof(DgemmDesc) * bound.size(), cudaMemcpyHostToDevice, st));
  if (!fbound.empty())
    ZQ_CUDA(cudaMemcpyAsync(fdescs_dev, fbound.data(), sizeof(DgemmDescT<float>) * fbound.size(), cudaMemcpyHostToDevice,
                            st));
  // the host copies must outlive the async copies: synchronise once at plan time
  ZQ_CUDA(cudaStreamSynchronize(st));
  return ZQ_OK;
}

template <typename ZT>
static int dc_run(DcPlan& P, const double* d, const double* e, double* lam_out, ZT* const Zb[2], ZT* Mb,
                  const DgemmDescT<ZT>* descs, cudaStream_t st) {
  const int n = P.n;
  // scale, tear
  k_dc_maxabs<<<1, 1024, 0, st>>>(d, e, n, P.scal);
  ZQ_LAUNCH_CHECK();
  k_dc_scale_in<<<ceil_div(n, 256), 256, 0, st>>>(d, e, n, P.dmod, P.es, P.scal);
  ZQ_LAUNCH_CHECK();
  if (!P.nodes_host.empty()) {
    k_dc_setrho<<<ceil_div((int)P.nodes_host.size(), 256), 256, 0, st>>>(P.nodes_dev, (int)P.nodes_host.size(), P.es);
    ZQ_LAUNCH_CHECK();
  }
  // Z buffers need zeros outside the diagonal blocks only where they are read:
  // every read is inside a node's block, which is fully written first.
  for (int t = P.max_depth; t >= 0; --t) {
    ZT* Zo = Zb[t & 1];
    ZT* Zi = Zb[(t + 1) & 1];
    double* lo = P.lam[t & 1];
    const double* li = P.lam[(t + 1) & 1];
    if (P.leaf_cnt[t] > 0) {
      k_dc_leaf<ZT><<<ceil_div(P.leaf_cnt[t], 128), 128, 0, st>>>(P.nodes_dev + P.leaf_off[t], P.leaf_cnt[t], P.dmod, Zo,
                                                                    lo, n);
      ZQ_LAUNCH_CHECK();
    }
    const int cnt = P.depth_cnt[t];
    if (cnt == 0) continue;
    DcNode* nd = P.nodes_dev + P.depth_off[t];
    {
      // shared-memory staging of the merged poles for the depth's largest node
      const int scap = P.depth_mmax[t] <= DC_SCAP ? P.depth_mmax[t] : 0;
      const size_t smem = (size_t)scap * 20;
      if (smem > 48 * 1024) {
        static std::atomic<unsigned long long> attr_set{0};
        int dev = 0;
        ZQ_CUDA(cudaGetDevice(&dev));
        const unsigned long long bit = 1ull << (dev & 63);
        if (!(attr_set.load() & bit)) {
          ZQ_CUDA(cudaFuncSetAttribute(k_dc_prepare<ZT>, cudaFuncAttributeMaxDynamicSharedMemorySize, DC_SCAP * 20));
          attr_set.fetch_or(bit);
        }
      }
      k_dc_prepare<ZT><<<cnt, 256, smem, st>>>(nd, P.w, Zi, li, n, scap);
      ZQ_LAUNCH_CHECK();
    }
    k_dc_secular<<<ceil_div(n, 4), 128, 0, st>>>(nd, cnt, P.w);
    ZQ_LAUNCH_CHECK();
    k_dc_zhat<<<ceil_div(n, 4), 128, 0, st>>>(nd, cnt, P.w);
    ZQ_LAUNCH_CHECK();
    k_dc_vectors<ZT><<<n, 128, 0, st>>>(nd, cnt, P.w, Mb, lo, n);
    ZQ_LAUNCH_CHECK();
    k_dc_rotate<ZT><<<ceil_div(n, 128), 128, 0, st>>>(nd, cnt, P.w, Mb, n);
    ZQ_LAUNCH_CHECK();
    if (P.gemm_tiles[t] > 0) {
      bool done = false;
      if constexpr (std::is_same<ZT, float>::value) {
        // FP32 merges of large nodes on the tensor cores (TF32 x3), one product per child
        if (P.tc_err && P.depth_mmax[t] >= 512 && fp32_products_on_tensor_cores(TC_USE_DC)) {
          for (int q = 0; q < 2 * cnt; ++q) {
            const DgemmDesc& h = P.gemm_host[P.gemm_off[t] + q];
            Tc32Args g{};
            g.cplx = 0; g.m = h.m; g.n = h.n; g.nseg = 1;
            g.seg[0].a.p = Zi + h.off_a; g.seg[0].a.ld = h.lda; g.seg[0].a.kfast = 0; g.seg[0].a.sign = 1.f;
            g.seg[0].b.p = Mb + h.off_b; g.seg[0].b.ld = h.ldb; g.seg[0].b.kfast = 1; g.seg[0].b.sign = 1.f;
            g.seg[0].k = h.k;
            g.alpha = make_float2(1.f, 0.f); g.beta = make_float2(0.f, 0.f);
            g.C = Zo + h.off_c; g.ldc = h.ldc;
            g.splits = 1;
            g.err = P.tc_err;
            if (int rc = tc32_gemm(g, st)) return rc;
          }
          done = true;
        }
      }
      if (!done) {
        grouped_launch<ZT>(descs + P.gemm_off[t], 2 * cnt, P.gemm_tiles[t], st);
        ZQ_LAUNCH_CHECK();
      }
    }
  }
  k_dc_unscale<<<ceil_div(n, 256), 256, 0, st>>>(P.lam[0], n, P.scal);
  ZQ_LAUNCH_CHECK();
  ZQ_CUDA(cudaMemcpyAsync(lam_out, P.lam[0], sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
  return ZQ_OK;
}

int DcPlan::run(const double* d, const double* e, double* lam_out, double*& z_out, cudaStream_t st) {
  if (n <= 0) return ZQ_OK;
  if (int rc = dc_run<double>(*this, d, e, lam_out, Z, Mb, descs_dev, st)) return rc;
  z_out = Z[0];
  return ZQ_OK;
}

int DcPlan::run_single(const double* d, const double* e, double* lam_out, float*& z_out, cudaStream_t st) {
  if (n <= 0) return ZQ_OK;
  if (int rc = dc_run<float>(*this, d, e, lam_out, Zf, Mbf, fdescs_dev, st)) return rc;
  z_out = Zf[0];
  return ZQ_OK;
}

}  // namespace zq
