// Internal interfaces between the solver's translation units.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <vector>

#include "zq_common.cuh"

namespace zq {

// ---------------------------------------------------------------- tridiagonal
// widest panel of the blocked reduction (reflectors kept per panel)
constexpr int NBMAX = 128;

template <typename R>
struct TridiagView {
  cplx<R>* M;      // [A; B], 2n x n, column-major
  int n;
  int64_t ld;
  cplx<R>* Ya;     // panel aux vectors, n x nbmax (global row index), ld = ldy
  cplx<R>* Yb;
  int64_t ldy;
  int nbmax;
  cplx<R>* ga;     // g of the current column (n)
  cplx<R>* gb;
  cplx<R>* hpart;  // hemv tile partials: hblk x hblk x 64 x 4
  int hblk;
  cplx<R>* dpart;  // panel dot partials, one set per 128 rows: hblk x nbmax x 4 (room for 4x that)
  cplx<R>* dots;   // the summed panel dot products: 4 * nbmax
  double* npart;   // norm partials: 2 * hblk
  double* cpart;   // c partials, one per hreduce CTA: ceil(n / 8) + 1
  double* scal;    // per-column scalars (16): [0..3] x_1 of the column, [4] f, [5..8] f m (reflector head)
  unsigned* counter;  // colupd CTAs finished for the current column (the last one forms the reflector)
  double* d;       // diagonal (n)
  double* e;       // quaternion subdiagonal (4 doubles each, n)
  double* tau;     // 1 if reflector j exists else 0 (n)
  int* tc_err;     // FP32: tensor-core products allowed (their timeout flag); null: CUDA cores only
  int coop;        // 1: the FP32 panels may run as one cooperative launch each (no other solve runs beside it)
};

template <typename R>
size_t tridiag_workspace_bytes(int n, int nbmax);
template <typename R>
TridiagView<R> tridiag_bind(void* ws, cplx<R>* M, int n, int64_t ld, int nbmax, double* d, double* e, double* tau);
template <typename R>
int tridiagonalize(TridiagView<R> v, int nb, cudaStream_t st);

// ---------------------------------------------------------------------- GEMM
enum { OP_N = 0, OP_T = 1, OP_C = 2, OP_R = 3 };

template <typename R>
struct ZgemmArgsT {
  int m, n, k1, k2;
  const cplx<R>* A1; int64_t lda1;
  const cplx<R>* B1; int64_t ldb1;
  const cplx<R>* A2; int64_t lda2;   // null: single segment
  const cplx<R>* B2; int64_t ldb2;
  R s2;
  cplx<R> alpha, beta;
  cplx<R>* C; int64_t ldc;
  cplx<R>* P; int64_t pcap;          // optional split-K partial buffer (complex elements)
};
using ZgemmArgs = ZgemmArgsT<double>;
template <typename R>
int zgemm(int opa1, int opb1, int opa2, int opb2, const ZgemmArgsT<R>& g, int batch, cudaStream_t st);

template <typename R>
struct DgemmDescT {
  const R* A; const R* B; R* C;
  int64_t lda, ldb, ldc;
  int64_t off_a, off_b, off_c;  // plan-time offsets (bound to pointers before upload)
  int m, n, k;
  int ta, tb;
  int tile0;
  R alpha, beta;
};
using DgemmDesc = DgemmDescT<double>;
template <typename R>
int dgemm_grouped(DgemmDescT<R>* host_descs, int count, DgemmDescT<R>* dev_descs, cudaStream_t st);
template <typename R>
void grouped_launch(const DgemmDescT<R>* dev_descs, int count, int tiles, cudaStream_t st);
int dgemm_tiles(int m, int n);

// ------------------------------------------------------------------ D&C (c)
struct DcNode {
  int a, c, b;
  int K, ndefl, nrot;
  double rho, rho2;
};
struct DcWork {
  double *sd, *sz, *nd_val, *nd_z, *df_val, *df_sval, *rot_c, *rot_s, *r_tau, *r_lam, *zhat;
  int *perm, *nd_col, *df_col, *df_scol, *rot_p, *rot_j, *r_orig;
};
struct DcPlan {
  int n = 0;
  int max_depth = 0;
  std::vector<DcNode> nodes_host;
  std::vector<int> depth_off, depth_cnt, leaf_off, leaf_cnt;
  std::vector<int> depth_mmax;  // largest node (b - a) per depth
  std::vector<DgemmDesc> gemm_host;
  std::vector<int> gemm_off, gemm_tiles;
  // device
  double* base = nullptr;
  double* Z[2] = {nullptr, nullptr};
  double* Mb = nullptr;
  double* lam[2] = {nullptr, nullptr};
  double *dmod = nullptr, *es = nullptr, *scal = nullptr;
  DcWork w{};
  DcNode* nodes_dev = nullptr;
  DgemmDesc* descs_dev = nullptr;
  // single-precision views of Z and M, and their descriptors (after the double
  // ones and two spare slots in the descriptor area)
  float* Zf[2] = {nullptr, nullptr};
  float* Mbf = nullptr;
  DgemmDescT<float>* fdescs_dev = nullptr;
  int* tc_err = nullptr;  // run_single: merges of large nodes on the tensor cores (timeout flag) when set

  static size_t workspace_doubles(int n);
  int build(int n);
  size_t num_nodes() const { return nodes_host.size(); }
  size_t num_descs() const { return gemm_host.size(); }
  int upload(double* ws, DcNode* dnodes, DgemmDesc* ddescs, cudaStream_t st);
  // d (n), e (n-1) on device; lam_out (n) on device; z_out points into the workspace
  int run(const double* d, const double* e, double* lam_out, double*& z_out, cudaStream_t st);
  // same tree with Z and the merge products in FP32 (eigenvalues and the
  // secular equation stay FP64): the refined path's decomposition
  int run_single(const double* d, const double* e, double* lam_out, float*& z_out, cudaStream_t st);
  // descriptor area bytes for upload(): double descriptors + 2 spare + float descriptors
  static size_t desc_bytes(size_t ndescs) {
    return sizeof(DgemmDescT<double>) * (ndescs + 2) + sizeof(DgemmDescT<float>) * ndescs;
  }
};

// ------------------------------------------------------------ back-transform
// phase reduction of the quaternion tridiagonal: e (4 doubles per entry) ->
// real off-diagonal |e_k| and unit quaternions phi_k = (alpha_k, beta_k)
int phase_reduce(const double* e, int n, double* offd, double* phi, cudaStream_t st);
// X = [diag(alpha); diag(beta)] (2n x n complex, ld), then Q X by blocked reflectors
// tc_err (FP32 only, may be null): with it, the large products run on the
// tensor cores (zq_tc32.cu) and a pipeline-wait timeout raises *tc_err
template <typename R>
int form_q(const cplx<R>* M, int64_t ldm, int n, const double* phi, cplx<R>* X, int64_t ldx,
           int nbq, void* ws, cudaStream_t st, int* tc_err = nullptr);
size_t form_q_workspace_bytes(int n, int nbq);
// out (2n x n complex, ldo) = X (2n x n complex, ldx) * Z (n x n real, ldz)
template <typename R>
int apply_z(const cplx<R>* X, int64_t ldx, const R* Z, int64_t ldz, int n, cplx<R>* out, int64_t ldo,
            DgemmDescT<R>* dev_desc, cudaStream_t st, int* tc_err = nullptr);
// FP32 products of the refined decomposition that may run on the TF32x3
// tensor-core kernel: trailing update, Q formation (the W^H X products with
// inner dimension L, and the X updates with inner dimension nbq), back-transform,
// divide-and-conquer merges
enum { TC_USE_TRAIL = 0, TC_USE_FORMQ = 1, TC_USE_APPLYZ = 2, TC_USE_DC = 3, TC_USE_FORMQ_X = 4 };
bool fp32_products_on_tensor_cores(int use);
// right half of the n2 x n2 output from the left half (U; V)
int symmetry_fill(double2* D, int64_t ld, int n, cudaStream_t st);

// ------------------------------------------------------ refined (mixed) path
struct RefineArgs {
  double2* dD; int64_t ldd; int n; double* deig;
  void* ws;                    // refine_workspace_bytes(n, nbq)
  void* ows; size_t ows_bytes; // accurate-product workspace (mode 1)
  DcPlan* dc;                  // uploaded plan for n
  DgemmDescT<float>* fdesc;    // one device descriptor slot
  int nb, nbq, mode, max_iter;
  double tol;
  double cluster_tol;          // accepted in-cluster coupling (relative to max |lambda|)
  double pair_eps;             // first-order formula only where |coupling| <= pair_eps |gap| (first step)
  double pair_eps_late;        // the same bound in the later steps
  int slices0;                 // Ozaki slices of the first step's products
  int slices_res;              // Ozaki slices of the products with the residual R = HX - X Lambda
  int coop;                    // the FP32 reduction may use cooperative panel launches
  cudaStream_t st;
  cudaStream_t st2;            // second stream: Q formation overlaps the tridiagonal solve
  cudaEvent_t ev_fork, ev_join;
  int iters; double last_emax;  // outputs
  double last_cluster;         // in-cluster coupling of the last step (before rotation)
  int clusters;                // clusters resolved (-1: one too large)
  int cluster_max;             // largest cluster rotated
};
size_t refine_workspace_bytes(int n, int nbq);
int refined_solve(RefineArgs& ra);

// Ozaki-sliced FP64-accurate complex product (zq_ozaki.cu)
struct OzOpts {
  int slices;      // bf16 slices per operand (7 bits each), 2..8
  int structured;  // 0 general; +1 Hermitian / -1 antisymmetric square output (lower tiles computed)
  int reuse_a;     // 1: the A operand is the same as in the previous call (slices kept)
  int nofill;      // structured: leave the upper triangle to the caller (who fills it with structured_fill)
};
int zgemm_ozaki(int opa1, int opb1, int opa2, int opb2, const ZgemmArgs& g, void* ws, size_t ws_bytes, cudaStream_t st,
                const OzOpts& opt);
size_t ozaki_workspace_bytes(int n);
// limit of every mbarrier wait in the tensor-core pipelines, SM clock cycles
// (<= 0: the default, about 2 s); a test hook for the timeout path
void set_pipeline_wait_cycles(long long cycles);
long long pipeline_wait_cycles();
// the driver's cuTensorMapEncodeTiled (null when unavailable)
void* tensor_map_encode_fn();
// upper triangle of a square structured matrix from its lower triangle (sym +1 Hermitian, -1 antisymmetric)
int structured_fill(double2* C, int64_t ldc, int n, int sym, cudaStream_t st);

}  // namespace zq
