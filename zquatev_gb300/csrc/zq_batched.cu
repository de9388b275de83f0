// Batched solve of many small quaternion-Hermitian matrices in ONE persistent
// kernel launch (one CTA per matrix, work handed out largest-first through a
// device counter).
//
// Reference: the same four steps as ts::zquatev (zquatev.cc:42-100) run once
// per matrix; the reference has no batched entry point, and below n = nb + 2
// it runs only its unblocked path (unblocked.cc:44-131), which is the regime
// of this kernel. Per matrix, inside one CTA (FP64 throughout):
//   1. unblocked quaternion tridiagonalisation of [A; B] in place: per column
//      one quaternion reflector (same construction as zq_tridiag.cu), the
//      quaternion Hermitian mat-vec g = H w on the trailing lower triangles
//      (thread per row), y = g - (w^H g / 2) w and the structured rank-2
//      update of the trailing lower triangles of A and B; w is kept in the
//      reduced column;
//   2. phase reduction of the quaternion subdiagonal (unit quaternions);
//   3. implicit QL with Wilkinson shifts on the real tridiagonal, rotations of
//      each sweep recorded by one thread and applied to the rows of Z by all
//      threads (classic tql2 scheme);
//   4. X = Phi Z (ascending eigenvalue order) in the right half of D, the
//      reflectors applied backwards (warp per column, coalesced over rows),
//      then the (U -V*; V U*) layout written out.
#include "zq_common.cuh"
#include "zq_kernels.h"

#include <atomic>
#include <cstdlib>
#include <mutex>

namespace zq {

constexpr int BT = 256;        // threads per CTA
constexpr int BNMAX = 256;     // largest quaternion order handled in one CTA

struct BatchTask {
  long long off;    // complex offset of D (from the launch's D) when Dp is null
  long long eoff;   // offset of eig (from the launch's eig) when Ep is null
  double2* Dp;      // or the matrix itself (requests in separate allocations)
  double* Ep;
  int n, ld;
  int out_slot;     // index into the info array
  int pad;
};

struct BatchArgs {
  const BatchTask* tasks;
  int count;
  int* counter;     // work counter (zeroed before the launch)
  double2* D;
  double* eig;
  double* ws;       // per-CTA workspace, slot stride ws_stride doubles
  long long ws_stride;
  int* info;        // per task: 0 ok, >0 QL non-convergence
};

// Shared memory of one solving group: a CTA (G = 256, n <= 256) or a warp
// (G = 32, n <= 32).
template <int NM>
struct GroupSmem {
  double2 swa[NM], swb[NM], sya[NM], syb[NM];
  double sc[NM], ss[NM];
  double sred[8];
  double sscal[8];
  int sflag[2];
  int s_m, s_cnt, s_done;
};
template <int G> __device__ __forceinline__ void gsync() {
  if (G == 32) __syncwarp(); else __syncthreads();
}
template <int G> __device__ __forceinline__ double gsum(double v, double* sh) {
  if (G == 32) return warp_sum(v);
  return block_sum(v, sh);
}
template <int G> __device__ __forceinline__ double gmax(double v, double* sh) {
  if (G == 32) return warp_max(v);
  return block_max(v, sh);
}

template <int G, int NM>
__device__ void batch_solve_group(const BatchTask& tk, const BatchArgs& a, double* ws, GroupSmem<NM>& sm, int tid) {
  const int n = tk.n;
  const int64_t ld = tk.ld;
  double2* A = tk.Dp ? tk.Dp : a.D + tk.off;
  double2* B = A + n;
  const int lane = tid & 31, warp = tid >> 5;
  double2* swa = sm.swa;
  double2* swb = sm.swb;
  double2* sya = sm.sya;
  double2* syb = sm.syb;
  double* sred = sm.sred;
  double* sscal = sm.sscal;
  double* sc_ = sm.sc;     // QL rotations of one sweep
  double* ss_ = sm.ss;
  int* sflag = sm.sflag;
  double* d = ws;                 // n
  double* e4 = d + NM;            // 4n quaternion subdiagonal
  double* offd = e4 + 4 * NM;     // n
  double* phi = offd + NM;        // 4n
  double* rank_d = phi + 4 * NM;  // n (eigenvalues, QL output)
  int* perm = reinterpret_cast<int*>(rank_d + NM);  // n
  double* Z = rank_d + 2 * NM;    // n x n, column-major, ld n

  // ---------------------------------------------------------------- step 1
  for (int j = 0; j < n; ++j) {
    const int L = n - 1 - j;
    if (tid == 0) d[j] = A[j + (int64_t)j * ld].x;
    if (L < 1) break;
    // norm of x = (A[j+1:, j], B[j+1:, j]) (max-scaled)
    double mx = 0.0;
    for (int i = tid; i < L; i += G) {
      const double2 xa = A[j + 1 + i + (int64_t)j * ld], xb = B[j + 1 + i + (int64_t)j * ld];
      mx = fmax(mx, fmax(fmax(fabs(xa.x), fabs(xa.y)), fmax(fabs(xb.x), fabs(xb.y))));
    }
    mx = gmax<G>(mx, sred);
    double ssq = 0.0;
    if (mx > 0.0) {
      const double inv = 1.0 / mx;
      for (int i = tid; i < L; i += G) {
        const double2 xa = A[j + 1 + i + (int64_t)j * ld], xb = B[j + 1 + i + (int64_t)j * ld];
        const double a0 = xa.x * inv, a1 = xa.y * inv, b0 = xb.x * inv, b1 = xb.y * inv;
        ssq += a0 * a0 + a1 * a1 + b0 * b0 + b1 * b1;
      }
    }
    ssq = gsum<G>(ssq, sred);
    if (tid == 0) {
      const double nu = mx * sqrt(ssq);
      const double2 qa = A[j + 1 + (int64_t)j * ld], qb = B[j + 1 + (int64_t)j * ld];
      const double q1 = sqrt(qa.x * qa.x + qa.y * qa.y + qb.x * qb.x + qb.y * qb.y);
      double f = 0.0, m0 = 0, m1 = 0, m2 = 0, m3 = 0;
      double ee0 = qa.x, ee1 = qa.y, ee2 = qb.x, ee3 = qb.y;
      if (L >= 2) {
        if (nu > 0.0) {
          if (q1 > 0.0) {
            const double s = nu / q1;
            f = 1.0 / (sqrt(nu) * sqrt(nu + q1));
            m0 = qa.x * (1 + s); m1 = qa.y * (1 + s); m2 = qb.x * (1 + s); m3 = qb.y * (1 + s);
            ee0 = -s * qa.x; ee1 = -s * qa.y; ee2 = -s * qb.x; ee3 = -s * qb.y;
          } else {
            f = 1.0 / nu; m0 = nu;
            ee0 = -nu; ee1 = 0; ee2 = 0; ee3 = 0;
          }
        } else {
          ee0 = ee1 = ee2 = ee3 = 0.0;
        }
      }
      e4[4 * j] = ee0; e4[4 * j + 1] = ee1; e4[4 * j + 2] = ee2; e4[4 * j + 3] = ee3;
      sscal[0] = f; sscal[1] = m0 * f; sscal[2] = m1 * f; sscal[3] = m2 * f; sscal[4] = m3 * f;
    }
    gsync<G>();
    const double f = sscal[0];
    // w in place of x (and in shared memory)
    for (int i = tid; i < L; i += G) {
      double2 wa = make_double2(0, 0), wb = wa;
      if (f > 0.0) {
        if (i == 0) { wa = make_double2(sscal[1], sscal[2]); wb = make_double2(sscal[3], sscal[4]); }
        else { wa = cscale(A[j + 1 + i + (int64_t)j * ld], f); wb = cscale(B[j + 1 + i + (int64_t)j * ld], f); }
      }
      A[j + 1 + i + (int64_t)j * ld] = wa;
      B[j + 1 + i + (int64_t)j * ld] = wb;
      swa[i] = wa; swb[i] = wb;
    }
    gsync<G>();
    if (f == 0.0) continue;
    // g = H_trail w  (rows j+1.., thread per row; lower triangles only)
    const int r0 = j + 1;
    double cp = 0.0;
    for (int i = tid; i < L; i += G) {
      double2 ax = make_double2(0, 0), az = ax, bx = ax, bz = ax;
      const int gi = r0 + i;
      // the three ranges of c (row i left of the diagonal, the diagonal, column
      // i below it) in separate loops so the loads pipeline
#pragma unroll 4
      for (int c = 0; c < i; ++c) {
        const double2 x = swa[c], z = cconj(swb[c]);
        const int64_t o = gi + (int64_t)(r0 + c) * ld;
        const double2 am = A[o], bm = B[o];
        cfma(ax, am, x); cfma(az, am, z); cfma(bx, bm, x); cfma(bz, bm, z);
      }
      {
        const double2 x = swa[i], z = cconj(swb[i]);
        const double am = A[gi + (int64_t)gi * ld].x;
        ax.x += am * x.x; ax.y += am * x.y; az.x += am * z.x; az.y += am * z.y;
      }
#pragma unroll 4
      for (int c = i + 1; c < L; ++c) {
        const double2 x = swa[c], z = cconj(swb[c]);
        const int64_t o = (r0 + c) + (int64_t)gi * ld;
        const double2 am = A[o], bm = B[o];
        cfmac(ax, am, x); cfmac(az, am, z);           // conj(A[c,i])
        cfma(bx, cneg(bm), x); cfma(bz, cneg(bm), z); // B[i,c] = -B[c,i]
      }
      // ga = A x - conj(B z), gb = B x + conj(A z)
      const double2 ga = csub(ax, cconj(bz)), gb = cadd(bx, cconj(az));
      sya[i] = ga; syb[i] = gb;
      cp += swa[i].x * ga.x + swa[i].y * ga.y + swb[i].x * gb.x + swb[i].y * gb.y;
    }
    const double c = gsum<G>(cp, sred);
    for (int i = tid; i < L; i += G) {
      sya[i] = csub(sya[i], cscale(swa[i], 0.5 * c));
      syb[i] = csub(syb[i], cscale(swb[i], 0.5 * c));
    }
    gsync<G>();
    // rank-2 structured update of the trailing lower triangles: each thread
    // walks its row's segment (independent elements, so the loads pipeline)
    for (int i = tid; i < L; i += G) {
      const double2 wai = swa[i], wbi = swb[i], yai = sya[i], ybi = syb[i];
      const int64_t orow = r0 + i;
#pragma unroll 4
      for (int cc = 0; cc < i; ++cc) {
        const double2 wac = swa[cc], wbc = swb[cc], yac = sya[cc], ybc = syb[cc];
        const int64_t o = orow + (int64_t)(r0 + cc) * ld;
        double2 ta = make_double2(0, 0), tb = ta;
        cfmacb(ta, wai, yac); cfmac(ta, wbi, ybc); cfmacb(ta, yai, wac); cfmac(ta, ybi, wbc);
        cfmacb(tb, wbi, yac); cfmac(tb, cneg(wai), ybc); cfmacb(tb, ybi, wac); cfmac(tb, cneg(yai), wbc);
        const double2 av = A[o], bv = B[o];
        A[o] = csub(av, ta);
        B[o] = csub(bv, tb);
      }
      {  // diagonal element: A only (B's diagonal is zero)
        const double2 wac = swa[i], wbc = swb[i], yac = sya[i], ybc = syb[i];
        const int64_t o = orow + (int64_t)(r0 + i) * ld;
        double2 ta = make_double2(0, 0);
        cfmacb(ta, wai, yac); cfmac(ta, wbi, ybc); cfmacb(ta, yai, wac); cfmac(ta, ybi, wbc);
        A[o] = csub(A[o], ta);
      }
    }
    gsync<G>();
  }
  gsync<G>();

  // ---------------------------------------------------------------- step 2
  if (tid == 0) {
    double a0 = 1.0, a1 = 0.0, b0 = 0.0, b1 = 0.0;
    phi[0] = a0; phi[1] = a1; phi[2] = b0; phi[3] = b1;
    for (int k = 0; k + 1 < n; ++k) {
      const double ea0 = e4[4 * k], ea1 = e4[4 * k + 1], eb0 = e4[4 * k + 2], eb1 = e4[4 * k + 3];
      const double nrm = sqrt(ea0 * ea0 + ea1 * ea1 + eb0 * eb0 + eb1 * eb1);
      offd[k] = nrm;
      if (nrm > 0.0) {
        const double na0 = (ea0 * a0 - ea1 * a1) - (eb0 * b0 + eb1 * b1);
        const double na1 = (ea0 * a1 + ea1 * a0) - (eb0 * b1 - eb1 * b0);
        const double nb0 = (eb0 * a0 - eb1 * a1) + (ea0 * b0 + ea1 * b1);
        const double nb1 = (eb0 * a1 + eb1 * a0) + (ea0 * b1 - ea1 * b0);
        const double s = 1.0 / sqrt(na0 * na0 + na1 * na1 + nb0 * nb0 + nb1 * nb1);
        a0 = na0 * s; a1 = na1 * s; b0 = nb0 * s; b1 = nb1 * s;
      } else {
        a0 = 1.0; a1 = 0.0; b0 = 0.0; b1 = 0.0;
      }
      phi[4 * (k + 1)] = a0; phi[4 * (k + 1) + 1] = a1; phi[4 * (k + 1) + 2] = b0; phi[4 * (k + 1) + 3] = b1;
    }
    offd[n - 1] = 0.0;
    sflag[0] = 0;
  }
  // Z = I
  for (int t = tid; t < n * n; t += G) Z[t] = ((t % n) == (t / n)) ? 1.0 : 0.0;
  gsync<G>();

  // ---------------------------------------------------------------- step 3
  // implicit QL with Wilkinson shift; d <- eigenvalues, Z <- eigenvectors
  const double eps = 1.1102230246251565e-16;
  for (int l = 0; l < n; ++l) {
    for (int iter = 0;; ++iter) {
      int& s_m = sm.s_m;
      int& s_cnt = sm.s_cnt;
      int& s_done = sm.s_done;
      if (tid == 0) {
        int m = l;
        for (; m < n - 1; ++m) {
          const double dd = fabs(d[m]) + fabs(d[m + 1]);
          if (fabs(offd[m]) <= eps * dd || fabs(offd[m]) < 1e-300) break;
        }
        s_done = (m == l) || (iter >= 60);
        if (iter >= 60 && m != l) sflag[0] += 1;
        s_cnt = 0;
        if (!s_done) {
          double g = (d[l + 1] - d[l]) / (2.0 * offd[l]);
          double r = hypot(g, 1.0);
          g = d[m] - d[l] + offd[l] / (g + copysign(r, g));
          double s = 1.0, c = 1.0, p = 0.0;
          int i = m - 1;
          bool early = false;
          for (; i >= l; --i) {
            const double ff = s * offd[i], bb = c * offd[i];
            r = hypot(ff, g);
            offd[i + 1] = r;
            if (r == 0.0) { d[i + 1] -= p; offd[m] = 0.0; early = true; break; }
            s = ff / r; c = g / r;
            g = d[i + 1] - p;
            r = (d[i] - g) * s + 2.0 * c * bb;
            p = s * r;
            d[i + 1] = g + p;
            g = c * r - bb;
            sc_[s_cnt] = c; ss_[s_cnt] = s; ++s_cnt;
          }
          if (!early) { d[l] -= p; offd[l] = g; offd[m] = 0.0; }
          s_m = m;
        }
      }
      gsync<G>();
      if (s_done) break;
      // apply the sweep's rotations (columns m-1 .. lo of Z) to every row
      const int m = s_m, cnt = s_cnt;
      // the updated column i of one rotation is column i + 1 of the next: carry
      // it in a register (no reload of a value just stored)
      for (int r = tid; r < n; r += G) {
        double* zr = Z + r;
        if (cnt == 0) continue;
        double carry = zr[(int64_t)m * n];
        for (int q = 0; q < cnt; ++q) {
          const int i = m - 1 - q;
          const double c = sc_[q], s = ss_[q];
          const double zi = zr[(int64_t)i * n];
          zr[(int64_t)(i + 1) * n] = s * zi + c * carry;
          carry = c * zi - s * carry;
        }
        zr[(int64_t)(m - cnt) * n] = carry;
      }
      gsync<G>();
    }
  }
  // ascending order: rank of each eigenvalue (ties by index)
  for (int k = tid; k < n; k += G) {
    const double v = d[k];
    int rnk = 0;
    for (int q = 0; q < n; ++q) rnk += (d[q] < v) || (d[q] == v && q < k);
    perm[rnk] = k;
  }
  gsync<G>();

  // ---------------------------------------------------------------- step 4
  // X = Phi Z (sorted columns) in the right half: X_a[r, col] = alpha_r z_r, X_b = beta_r z_r
  double2* XA = A + (int64_t)n * ld;
  double2* XB = XA + n;
  for (int t = tid; t < n * n; t += G) {
    const int r = t % n, col = t / n;
    const double z = Z[r + (int64_t)perm[col] * n];
    XA[r + (int64_t)col * ld] = make_double2(phi[4 * r] * z, phi[4 * r + 1] * z);
    XB[r + (int64_t)col * ld] = make_double2(phi[4 * r + 2] * z, phi[4 * r + 3] * z);
  }
  double* eig_out = tk.Ep ? tk.Ep : a.eig + tk.eoff;
  for (int k = tid; k < n; k += G) eig_out[k] = d[perm[k]];
  gsync<G>();
  // reflectors backwards: x <- x - w <w,x> - w' [w,x], w' = (-conj(wb), conj(wa))
  for (int j = n - 3; j >= 0; --j) {
    const int L = n - 1 - j;
    for (int i = tid; i < L; i += G) { swa[i] = A[j + 1 + i + (int64_t)j * ld]; swb[i] = B[j + 1 + i + (int64_t)j * ld]; }
    gsync<G>();
    for (int col = warp; col < n; col += G / 32) {
      double2* xa = XA + (j + 1) + (int64_t)col * ld;
      double2* xb = XB + (j + 1) + (int64_t)col * ld;
      double2 c1 = make_double2(0, 0), c2 = c1;
      for (int i = lane; i < L; i += 32) {
        const double2 wa = swa[i], wb = swb[i], va = xa[i], vb = xb[i];
        cfmac(c1, wa, va); cfmac(c1, wb, vb);
        cfma(c2, wa, vb); cfma(c2, cneg(wb), va);
      }
      c1.x = warp_sum(c1.x); c1.y = warp_sum(c1.y);
      c2.x = warp_sum(c2.x); c2.y = warp_sum(c2.y);
      for (int i = lane; i < L; i += 32) {
        const double2 wa = swa[i], wb = swb[i];
        double2 va = xa[i], vb = xb[i];
        // va -= wa c1 - conj(wb) c2 ; vb -= wb c1 + conj(wa) c2
        double2 ta = make_double2(0, 0), tb = ta;
        cfma(ta, wa, c1); cfmac(ta, cneg(wb), c2);
        cfma(tb, wb, c1); cfmac(tb, wa, c2);
        xa[i] = csub(va, ta);
        xb[i] = csub(vb, tb);
      }
    }
    gsync<G>();
  }
  // output: left half (U; V) = X, right half (-conj(V); conj(U))
  for (int t = tid; t < n * n; t += G) {
    const int r = t % n, col = t / n;
    const double2 u = XA[r + (int64_t)col * ld], vv = XB[r + (int64_t)col * ld];
    A[r + (int64_t)col * ld] = u;
    B[r + (int64_t)col * ld] = vv;
    XA[r + (int64_t)col * ld] = make_double2(-vv.x, vv.y);
    XB[r + (int64_t)col * ld] = make_double2(u.x, -u.y);
  }
  if (tid == 0) a.info[tk.out_slot] = sflag[0];
  gsync<G>();
}

// Per-size variants in one persistent launch. Tasks come largest first; a CTA
// takes one at a time and solves it with all 256 threads while n > wmax. The
// first task of at most wmax (the autotuned switch size, <= 32) turns the CTA
// into eight independent warps: each warp solves whole matrices (one lane per
// row, warp-synchronous steps) and takes further tasks from the same counter,
// all of which are small from then on.
constexpr int WNM = 32;  // largest order a warp solves
constexpr long long WARP_WS = 12LL * WNM + (long long)WNM * WNM + 64;  // per-warp workspace (doubles)
union BatchSmem {
  GroupSmem<BNMAX> cta;
  GroupSmem<WNM> warp[BT / 32];
};
__device__ __forceinline__ void batch_solve_one(const BatchTask& tk, const BatchArgs& a, double* ws) {
  __shared__ BatchSmem s_one;
  batch_solve_group<BT, BNMAX>(tk, a, ws, s_one.cta, threadIdx.x);
}

__global__ void __launch_bounds__(BT, 3) k_batched(BatchArgs a, int wmax) {
  __shared__ int s_task;
  __shared__ BatchSmem smem;
  double* ws = a.ws + (int64_t)blockIdx.x * a.ws_stride;
  int t;
  for (;;) {
    if (threadIdx.x == 0) s_task = atomicAdd(a.counter, 1);
    __syncthreads();
    t = s_task;
    __syncthreads();
    if (t >= a.count) return;
    if (a.tasks[t].n <= wmax) break;  // the rest of the queue is small: warp mode
    const BatchTask tk = a.tasks[t];
    if (tk.n > 0) batch_solve_group<BT, BNMAX>(tk, a, ws, smem.cta, threadIdx.x);
  }
  // warp mode: warp 0 starts with task t, the others take their own
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double* wws = ws + (int64_t)warp * WARP_WS;
  GroupSmem<WNM>& wsm = smem.warp[warp];
  if (warp != 0) {
    int nt = 0;
    if (lane == 0) nt = atomicAdd(a.counter, 1);
    t = __shfl_sync(0xffffffffu, nt, 0);
  }
  while (t < a.count) {
    const BatchTask tk = a.tasks[t];
    if (tk.n > WNM) {
      // a queue not sorted largest first: never solve above the warp's size
      if (lane == 0) a.info[tk.out_slot] = -1;
    } else if (tk.n > 0) {
      batch_solve_group<32, WNM>(tk, a, wws, wsm, lane);
    }
    int nt = 0;
    if (lane == 0) nt = atomicAdd(a.counter, 1);
    t = __shfl_sync(0xffffffffu, nt, 0);
  }
}

long long batched_ws_stride() {
  // d (1), e4 (4), offd (1), phi (4), eigenvalues (1), perm (1, ints) -- 12 n -- then Z (n x n)
  return 12LL * BNMAX + (long long)BNMAX * BNMAX + 64;
}
int batched_max_n() { return BNMAX; }

// switch size of the warp variant for launches that are not autotuned
// (environment ZQ_BATCH_WARP_MAX overrides; 0 disables the warp variant)
static std::atomic<int> g_warp_max{-1};
int batched_warp_max() {
  int v = g_warp_max.load();
  if (v < 0) {
    v = 24;
    if (const char* e = getenv("ZQ_BATCH_WARP_MAX")) v = atoi(e);
    v = v < 0 ? 0 : (v > WNM ? WNM : v);
    g_warp_max.store(v);
  }
  return v;
}
void batched_set_warp_max(int v) { g_warp_max.store(v < 0 ? -1 : (v > WNM ? WNM : v)); }

int batched_launch(const void* dev_tasks, int count, int* dev_counter, double2* D, double* eig, double* ws,
                   int ctas, int* dev_info, cudaStream_t st, int wmax) {
  if (count <= 0) return ZQ_OK;
  BatchArgs a{};
  a.tasks = reinterpret_cast<const BatchTask*>(dev_tasks);
  a.count = count;
  a.counter = dev_counter;
  a.D = D;
  a.eig = eig;
  a.ws = ws;
  a.ws_stride = batched_ws_stride();
  a.info = dev_info;
  ZQ_CUDA(cudaMemsetAsync(dev_counter, 0, sizeof(int), st));
  prof_begin(PC_BATCHED, st);
  if (wmax < 0) wmax = batched_warp_max();
  k_batched<<<ctas, BT, 0, st>>>(a, wmax > WNM ? WNM : wmax);
  prof_end(PC_BATCHED, st);
  ZQ_LAUNCH_CHECK();
  return ZQ_OK;
}

size_t batched_task_bytes() { return sizeof(BatchTask); }

void batched_fill_task(void* dst, long long off, long long eoff, int n, int ld, int slot) {
  BatchTask* t = reinterpret_cast<BatchTask*>(dst);
  t->off = off; t->eoff = eoff; t->Dp = nullptr; t->Ep = nullptr; t->n = n; t->ld = ld; t->out_slot = slot; t->pad = 0;
}

void batched_fill_task_ptr(void* dst, double2* D, double* eig, int n, int ld, int slot) {
  BatchTask* t = reinterpret_cast<BatchTask*>(dst);
  t->off = 0; t->eoff = 0; t->Dp = D; t->Ep = eig; t->n = n; t->ld = ld; t->out_slot = slot; t->pad = 0;
}

// ----------------------------------------------------------------------------
// Single small solve that allocates nothing.
//
// For callers that cannot call cudaMalloc: code that runs under an external
// allocator which owns the device memory budget (a framework's caching
// allocator, a pre-sized memory pool), or in a context where allocating
// device memory is not allowed. The solver's scratch (one per-CTA workspace of
// the batched kernel) lives in the file-scope device array below, of fixed
// size; the caller passes D and eig as for zquatev_device.
//
// Limits and behaviour:
//   * n2 <= 2 * BNMAX = 512 (quaternion order 256); larger sizes are rejected
//     with ZQ_ERR_LIMIT before anything is launched.
//   * The scratch is ~537 KiB (NOALLOC_SCRATCH_DOUBLES doubles) and is held by
//     every GPU that loads this library until the process exits.
//   * The first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (once per device, with that device current); make
//     that first call before any stream capture.
//   * Every call shares the one array, which keeps the previous call's
//     contents; the kernel writes every scratch word before it reads it, so
//     nothing has to be cleared. Calls whose work overlaps on the GPU (on
//     different streams, or from different host threads) race on the array.
//   * The call waits for its stream and returns info (0, or > 0 when the
//     tridiagonal QL did not converge).
// ----------------------------------------------------------------------------
constexpr long long NOALLOC_SCRATCH_DOUBLES = 12LL * BNMAX + (long long)BNMAX * BNMAX + 64 + 8;
static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_SCRATCH_DOUBLES];

__global__ void __launch_bounds__(BT) k_solve_small_noalloc(BatchTask tk, double2* D, double* eig, double* scratch,
                                                            int* info) {
  BatchArgs a{};
  a.D = D;
  a.eig = eig;
  a.ws = scratch;
  a.info = info;
  batch_solve_one(tk, a, scratch);
}

static std::mutex g_noalloc_mu;
static double* g_noalloc_dev[64];  // device address of g_noalloc_scratch, per device

}  // namespace zq

extern "C" int zquatev_device_noalloc(int n2, double* dD, int ld2, double* deig, void* stream) {
  using namespace zq;
  if (n2 < 0 || (n2 & 1)) return ZQ_ERR_N2;
  if (n2 == 0) return ZQ_OK;
  if (!dD) return ZQ_ERR_D;
  if (ld2 < n2) return ZQ_ERR_LD;
  if (!deig) return ZQ_ERR_EIG;
  if (n2 > 2 * BNMAX) {
    set_error_message("zquatev_device_noalloc: n2 above its fixed limit of 512");
    return ZQ_ERR_LIMIT;
  }
  int dev = 0;
  ZQ_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return ZQ_ERR_ARG;
  double* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_dev[dev]) {
      void* p = nullptr;
      ZQ_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
      g_noalloc_dev[dev] = reinterpret_cast<double*>(p);
    }
    scratch = g_noalloc_dev[dev];
  }
  const long long stride = 12LL * BNMAX + (long long)BNMAX * BNMAX + 64;
  int* info_dev = reinterpret_cast<int*>(scratch + stride);
  BatchTask tk{};
  tk.off = 0; tk.eoff = 0; tk.Dp = nullptr; tk.Ep = nullptr; tk.n = n2 / 2; tk.ld = ld2; tk.out_slot = 0;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  (void)cudaGetLastError();  // an earlier, unrelated launch error of the caller is not this call's
  k_solve_small_noalloc<<<1, BT, 0, st>>>(tk, reinterpret_cast<double2*>(dD), deig, scratch, info_dev);
  ZQ_CUDA(cudaGetLastError());  // the launch itself failed: nothing was enqueued
  count_launch();
  // From here the kernel is queued: whatever happens, wait for the stream
  // before returning, so that no error return leaves it writing D, eig or the
  // shared scratch behind the caller's back.
  int info = 0;
  const cudaError_t ce = cudaMemcpyAsync(&info, info_dev, sizeof(int), cudaMemcpyDeviceToHost, st);
  const cudaError_t se = cudaStreamSynchronize(st);
  if (ce != cudaSuccess) { set_last_error(ce, "cudaMemcpyAsync(info)", __FILE__, __LINE__); return ZQ_ERR_CUDA; }
  if (se != cudaSuccess) { set_last_error(se, "cudaStreamSynchronize", __FILE__, __LINE__); return ZQ_ERR_CUDA; }
  return info;
}
