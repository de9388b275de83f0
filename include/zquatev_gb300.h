/*
 * C ABI of the GB300 quaternion eigensolver (libzquatev_gb300.so).
 *
 * A quaternion-Hermitian matrix H = (A -B*; B A*) of order n2 = 2n (A Hermitian,
 * B complex antisymmetric) is passed as a column-major n2 x ld2 array of
 * complex doubles (interleaved re, im). Only its left half [A; B] is read. On
 * return the array holds all n2 eigenvectors in the (U -V*; V U*) layout and
 * eig[0..n-1] the ascending eigenvalues (each is doubly degenerate; columns i
 * and i+n belong to eig[i]); eig[n..] is not touched.
 *
 * Return codes: 0 success; -1 bad n2 (odd or negative); -2 null D; -3 ld2 < n2;
 * -4 null eig; -5 other bad argument; -100 CUDA failure; -101 out of device
 * memory; -103 size above the fixed limit of the called entry point; -104 a
 * device-side pipeline wait ran out of time (the kernel stopped and said so).
 * zq_last_error() describes the last failure on the calling thread.
 */
#ifndef ZQUATEV_GB300_H
#define ZQUATEV_GB300_H

#ifdef __cplusplus
#include <complex>
extern "C" {
#endif

/* Replaces ts::zquatev(n2, D, ld2, eig) (reference zquatev.h:54,
 * zquatev.cc:42-100) for FFI callers: same arguments with D as interleaved
 * doubles in HOST memory. Unlike the reference, ld2 > n2 is handled (V is
 * stored at rows n..2n-1; reference quirk at zquatev.cc:84-90). */
int zquatev_c(int n2, double* D, int ld2, double* eig);

/* Eigenvalues only (jobz = 'N'): the reference always computes vectors
 * (zquatev.cc:84, blocked.cc:477-544); this skips Q formation and the
 * back-transform. D (host) is used as scratch; eig[0..n-1] receives the values. */
int zquatev_values(int n2, double* D, int ld2, double* eig);

/* Device-pointer variant of ts::zquatev (zquatev.h:54): dD is an n2 x ld2
 * complex array in DEVICE memory, deig >= n doubles in device memory. The work
 * is ordered after `stream` (a cudaStream_t, 0 = legacy default stream) and the
 * call returns without synchronising. */
int zquatev_device(int n2, double* dD, int ld2, double* deig, void* stream);

/* Device-pointer eigenvalues-only variant. */
int zquatev_values_device(int n2, double* dD, int ld2, double* deig, void* stream);

/* Real symmetric tridiagonal eigensolver (the stage that replaces zhbev at
 * zquatev.cc:74-84): d (n), e (n-1, the off-diagonal), lam (n, ascending) and
 * Z (n x ldz, column-major eigenvectors) all in device memory. */
int zq_stedc_device(int n, const double* d, const double* e, double* lam, double* Z, int ldz, void* stream);

/* Batched solve of `count` independent matrices held in device memory:
 * matrix b has order n2s[b] (even), starts at dD + 2*offs[b] doubles
 * (complex offset offs[b]) with leading dimension ld2s[b], and eigenvalues at
 * deig + eoffs[b]. All arrays n2s/ld2s/offs/eoffs are HOST arrays. Matrices
 * with n2 <= 512 run in one persistent kernel launch (one CTA per matrix,
 * largest first); larger ones through the per-matrix path. Ordered after
 * `stream`; returns after the batch has finished, with the largest per-matrix
 * info (0 = all converged). The reference solves one matrix per call; this has
 * no counterpart there. */
int zquatev_batched_device(int count, const int* n2s, const int* ld2s, const long long* offs,
                           const long long* eoffs, double* dD, double* deig, void* stream);

/* Mixed-precision solve with iterative refinement, same arguments and output
 * as zquatev_device (device memory, ordered after `stream`, synchronises once
 * per refinement step to read the correction size). An FP32 decomposition is
 * refined to FP64 accuracy by Ogita-Aishima iterations on the quaternion form;
 * mode 0 computes the refinement products in native FP64, mode 1 with
 * Ozaki-sliced bf16 tensor-core products accumulated exactly. The reference
 * has only the FP64 path (zquatev.cc:42-100). */
int zquatev_refined_device(int n2, double* dD, int ld2, double* deig, void* stream, int mode);
/* Iterations, final max |E| and whether the plain FP64 path had to be used
 * (refinement not converged, e.g. tightly clustered eigenvalues) for the last
 * refined solve on this device. */
int zq_refine_stats(int* iters, double* last_correction, int* fell_back);

/* Explicit paths of the host drop-in: plain FP64, or refined (with the FP64
 * fallback). zquatev_c / ts::zquatev / zquatev_device follow the path policy
 * set by zq_set_path: 0 FP64, 1 refined, 2 auto (default: refined for
 * n2 >= 96, FP64 below); environment ZQ_PATH=fp64|refined|auto overrides. */
int zquatev_fp64_c(int n2, double* D, int ld2, double* eig);
int zquatev_refined_c(int n2, double* D, int ld2, double* eig);
int zquatev_fp64_device(int n2, double* dD, int ld2, double* deig, void* stream);
int zq_set_path(int path);

/* FP64-accurate complex product C = op(A) op(B) (m x n, inner k; op 0 = N,
 * 1 = T, 2 = conjugate transpose, 3 = conjugate) on the bf16 tensor cores with
 * Ozaki slicing and exact accumulation (the engine of the refinement). All
 * pointers are device memory (interleaved complex, column-major); allocates
 * its scratch with cudaMallocAsync on `stream`. No reference counterpart. */
int zq_zgemm_accurate(int opa, int opb, int m, int n, int k, const double* A, int lda, const double* B, int ldb,
                      double* C, int ldc, void* stream);

/* Single solve of a small matrix (n2 <= 512) in device memory that allocates
 * nothing: for callers that cannot call cudaMalloc (code running under an
 * external allocator that owns the device memory, or where allocating device
 * memory is not allowed). Its scratch is a fixed ~537 KiB array in the
 * library's device memory, held by every GPU that loads the library until
 * exit. Larger n2 return -103 (ZQ_ERR_LIMIT). The first call on a device looks
 * up the array's address (make it before any stream capture). All calls share
 * the array: calls that overlap on the GPU race. Waits for `stream` and
 * returns info. No counterpart in the reference. */
int zquatev_device_noalloc(int n2, double* dD, int ld2, double* deig, void* stream);

/* Panel width of the blocked tridiagonalisation (the reference hard-codes
 * nb = 20 at zquatev.cc:64). Valid range 1..128; default 16 (the autotuned
 * table, zq_autotune_nb, overrides it per size bucket). */
int zq_set_block_size(int nb);
int zq_get_block_size(void);

/* Tensor-core kernel of the Ozaki products in the refined path and
 * zq_zgemm_accurate: 0 = mma.sync (bf16 m16n8k16, 64 x 64 tiles), 1 = tcgen05
 * (TMEM accumulators, TMA-fed 128 x 256 MMAs, one CTA per tile), 2 = tcgen05 in
 * clusters of two CTAs that share the B operand by TMA multicast, 3 = 2-SM
 * tcgen05 MMAs (cta_group::2, 256 x 256 per CTA pair; the default). Same
 * arithmetic and results. */
int zq_set_ozaki_kernel(int which);
int zq_get_ozaki_kernel(void);

/* Limit, in SM clock cycles, of every wait of the tensor-core pipelines
 * (mbarrier waits between the copy, MMA and drain roles); cycles <= 0 restores
 * the default (about 2 s). When a wait runs out, the kernel stops issuing
 * work, waits for what it already issued, frees its tensor memory and
 * returns, and the call returns -104. A test hook for that path: no
 * counterpart in the reference, which has no device code. */
int zq_set_pipeline_wait(long long cycles);

/* FP32-accurate product on the tcgen05 tensor cores (TF32, three passes:
 * hi*hi + hi*lo + lo*hi, FP32 accumulation in tensor memory), the kernel of
 * the refined path's Q formation, back-transform and large divide-and-conquer
 * merges (the reference forms those products with zgemm3m: blocked.cc:477-544,
 * zquatev.cc:86-90). C = op(A) op(B), column-major, complex64 (cplx = 1; op 0
 * N, 1 T, 2 conjugate transpose, 3 conjugate) or float32 (cplx = 0; op 0 N,
 * 1 T); splits > 1 divides K over that many CTAs per tile. Device pointers;
 * waits for `stream`. */
int zq_gemm_tf32x3(int cplx, int opa, int opb, int m, int n, int k, const float* A, int lda, const float* B,
                   int ldb, float* C, int ldc, int splits, void* stream);

/* Panel-width autotuner: times the quaternion tridiagonalisation of a seeded
 * random matrix of order n2 for nb in {16, 32, 64, 128} and stores the fastest
 * for n2's size bucket (powers of two of n) and precision (0: FP64 path, 1:
 * FP32 decomposition of the refined path); later solves of that bucket use it.
 * best_nb receives the choice, ms (4 doubles, may be NULL) the timings. The
 * reference hard-codes nb = 20 (zquatev.cc:64). zq_set_block_size clears the
 * table. */
int zq_autotune_nb(int n2, int precision, int* best_nb, double* ms);
/* Tuned width for n2's bucket (0 = not tuned), and setting it directly (e.g.
 * from a saved table; 0 clears). */
int zq_tuned_nb(int n2, int precision);
int zq_set_tuned_nb(int n2, int precision, int nb);

/* Batch plan: one layout of small matrices (every n2 <= 512; arguments as
 * zquatev_batched_device) solved repeatedly. Tasks are ordered largest first
 * and uploaded once. ctas_per_sm 1..4 fixes the persistent kernel's launch
 * shape; 0 lets the first run choose it by timing each candidate on the
 * caller's batch (the input is restored between candidates). The launch is
 * captured in a CUDA graph; each run replays it on `stream` without
 * synchronising (recaptured when dD or deig change). zq_batch_plan_info waits
 * for `stream` and returns the largest per-matrix info. No counterpart in the
 * reference. */
typedef struct zq_batch_plan zq_batch_plan;
zq_batch_plan* zq_batch_plan_create(int count, const int* n2s, const int* ld2s, const long long* offs,
                                    const long long* eoffs, int ctas_per_sm);
int zq_batch_plan_run(zq_batch_plan* p, double* dD, double* deig, void* stream);
int zq_batch_plan_info(zq_batch_plan* p, void* stream);
/* Chosen CTAs per SM, CTAs of the captured launch, and the tuning times (4 doubles, ms; 0 = not tried). */
int zq_batch_plan_shape(zq_batch_plan* p, int* ctas_per_sm, int* ctas, double* tune_ms);
/* The per-size kernel variant the plan's autotuner chose: matrices of order
 * n <= *warp_max_n are solved one per warp (eight per CTA), larger ones one per
 * CTA, in the same persistent launch. ms (4 doubles, may be NULL): the tuning
 * times for the switch sizes 0 (CTA variant only), 16, 24 and 32. No
 * counterpart in the reference (one matrix per call). */
int zq_batch_plan_variant(zq_batch_plan* p, int* warp_max_n, double* ms);
/* Switch size of the warp variant for batched launches that are not planned
 * (zquatev_batched_device, the request server): 0..32, or -1 for the default
 * (24; environment ZQ_BATCH_WARP_MAX). */
int zq_set_batch_warp_max(int n);
int zq_batch_plan_destroy(zq_batch_plan* p);

/* Kernel-class timing with CUDA events on the launching streams (for the
 * benchmark's roofline figures; off by default, adds two event records per
 * bracketed launch). Classes: 0 quaternion hemv, 1 trailing update, 2 panel
 * column kernels, 3 Q-formation GEMMs, 4 back-transform GEMM, 5 tridiagonal
 * eigensolver, 6 whole tridiagonalisation, 7 whole Q formation, 8 batched
 * kernel, 9 Ozaki tensor-core product, 10 whole refinement. No reference
 * counterpart. */
int zq_profile_enable(int mask);
int zq_profile_read(int cls, double* total_ms, long long* launches);
int zq_profile_reset(void);
/* Executed arithmetic counted for a class (currently the Ozaki tensor-core product, class 9). */
int zq_profile_flops(int cls, double* flops);

/* Kernels this library has launched since it was loaded (all devices, all
 * entry points; every launch is counted on the host right after it is made). */
long long zq_launch_count(void);

/* Frees the cached device workspace of the current device, and the device copy
 * of D that the host-memory entry points keep between calls (n2^2 complex). */
int zq_release_workspace(void);

/* ---------------------------------------------------------------- serving
 * A request server on the current device: ts::zquatev calls (zquatev.h:54) on
 * host arrays, submitted from any thread and solved as they arrive.
 * A request's footprint is its device matrix (n2 x n2 complex) plus
 * eigenvalues plus the workspace of its solve; requests are admitted in
 * arrival order while the admitted footprints fit hbm_budget_bytes (<= 0:
 * 80% of the free device memory at creation). An admitted request's matrix is
 * copied to the device at once and stays there until its result is copied
 * back into D and eig. Requests with n2 <= batch_max_n2 (at most 512) are
 * solved together in launches of the persistent batched kernel (every one that
 * is ready when a batch slot frees up, at most max_batch); larger ones run on
 * `lanes` concurrent lanes through the drop-in's default path (refined above
 * n2 = 512, FP64 below; FP64 fallback). D and eig must stay valid until zq_server_wait returns for the
 * request. No counterpart in the reference. */
typedef struct zq_server zq_server;
typedef struct zq_server_stats {
  long long submitted, completed;
  long long batches, batched_solves;      /* batched-kernel launches and the requests they solved */
  long long lane_solves, refined_solves, fp64_solves, fallbacks;
  long long queued;                       /* waiting for admission */
  long long in_flight;                    /* admitted, not finished */
  int lanes;
  double budget_bytes;
  double reserved_bytes;                  /* admitted footprints now */
  double peak_reserved_bytes;
  double mean_reserved_bytes;             /* time average from the first submission */
  double device_used_bytes;               /* device memory in use (all users) at the call */
} zq_server_stats;

/* Device bytes one solve of size n2 holds: its n2 x n2 matrix, eigenvalues
 * and workspace. path: 0 FP64, 1 refined (FP64 fallback included), 2 batched
 * kernel (n2 <= 512), -1 the one the server would pick. The server's
 * admission charges this figure. Negative on bad arguments. */
long long zq_solve_footprint(int n2, int path);

/* NULL on failure (zq_last_error). */
zq_server* zq_server_create(long long hbm_budget_bytes, int lanes, int max_batch, int batch_max_n2);
/* Request id (>= 0), or a negative code: argument errors as zquatev_c, -103 if
 * the footprint can never fit the budget. */
long long zq_server_submit(zq_server* s, int n2, double* D, int ld2, double* eig);
/* 1 finished, 0 not yet, -5 unknown id. */
int zq_server_test(zq_server* s, long long id);
/* Blocks until the request finished and returns its info. times_ms (4
 * doubles, may be NULL): submission, admission, start and end of the solve,
 * in ms since the server was created. path (may be NULL): 0 FP64, 1 refined,
 * 2 batched kernel, 3 refined with FP64 fallback. The id is released. */
int zq_server_wait(zq_server* s, long long id, double* times_ms, int* path);
int zq_server_stats_read(zq_server* s, zq_server_stats* out);
/* Waits for every submitted request, then stops the workers and frees the server. */
int zq_server_destroy(zq_server* s);

const char* zq_last_error(void);
int zq_version(void);

#ifdef __cplusplus
} /* extern "C" */

/* The reference's own C++ entry point, exported with the same mangled name
 * (_ZN2ts7zquatevEiPSt7complexIdEiPd), so programs linked against the
 * reference link against this library unchanged (zquatev.h:54). */
namespace ts {
int zquatev(const int n2, std::complex<double>* const D, const int ld2, double* const eig);
}
#endif

#endif /* ZQUATEV_GB300_H */
