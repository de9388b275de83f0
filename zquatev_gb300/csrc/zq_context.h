// Solver context: the streams, events and device workspace one solve at a
// time runs with. The drop-in entry points share one context per device; the
// request server (zq_serve.cu) owns one per lane and binds each request's
// workspace to it from the stream-ordered pool.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <mutex>
#include <vector>

#include "zq_kernels.h"

namespace zq {

struct RefineBuffers {
  void* dev = nullptr;
  size_t bytes = 0;
  bool external = false;  // bound by the caller: never freed or grown here
  int last_iters = 0;
  double last_emax = 0.0;
  int last_fallback = 0;
};

struct BatchBuffers {
  void* dev = nullptr;
  size_t bytes = 0;
  std::vector<char> host_tasks;
};

struct Context {
  int device = -1;
  cudaStream_t st = nullptr, st2 = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  void* ws = nullptr;
  size_t ws_bytes = 0;
  bool ws_external = false;  // bound by the caller: never freed or grown here
  int dc_n = -1;
  DcPlan dc;
  RefineBuffers rb;
  BatchBuffers bb;
  // solves of this context may use cooperative launches (off for the
  // server's lanes, whose solves run beside each other)
  bool coop = true;
  // device copy of D for the host-memory entry points, kept between calls
  // (a 1 GB cudaMallocAsync + cudaFreeAsync per n2 = 8192 call cost ~44 ms in
  // a process whose other allocations kept the pool from reusing the memory)
  void* hbuf = nullptr;
  size_t hbuf_bytes = 0;
  std::mutex mu;
};

// Streams and events of a new context on `device` (no workspace yet).
int context_create(int device, Context** out);
// Frees what the context owns (not bound workspace); synchronises its streams.
void context_destroy(Context* c);
// Device bytes one solve of quaternion size n needs: the FP64 path's workspace
// and, for refined = true, the refinement buffers on top (with the Ozaki
// product's slices).
void solve_workspace_bytes(int n, size_t* fp64_bytes, size_t* refine_bytes);
// Use caller-owned workspace for the next solves (nullptr/0 unbinds).
void context_bind(Context* c, void* ws, size_t ws_bytes, void* rws, size_t rws_bytes);

int ensure_ws(Context* c, size_t bytes);
int ensure_plan(Context* c, int n);
int solve_device(Context* c, double2* dD, int64_t ldd, int n, double* deig, bool vectors, cudaStream_t st);
int refined_device(Context* c, double2* dD, int64_t ldd, int n, double* deig, cudaStream_t st, int mode);
// drop-in policy: 0 FP64 path, 1 refined path for quaternion size n
int path_for(int n);
// tuned panel widths (prec 0: FP64 path, 1: FP32 decomposition), 0 = not tuned
void nb_table_set(int prec, int n, int nb);
int nb_table_get(int prec, int n);

// batched kernel (zq_batched.cu)
long long batched_ws_stride();
int batched_max_n();
// wmax: largest order solved by the warp variant (tasks sorted largest first;
// -1: the current default, 0: CTA variant only)
int batched_launch(const void* dev_tasks, int count, int* dev_counter, double2* D, double* eig, double* ws,
                   int ctas, int* dev_info, cudaStream_t st, int wmax = -1);
int batched_warp_max();
void batched_set_warp_max(int v);
size_t batched_task_bytes();
void batched_fill_task(void* dst, long long off, long long eoff, int n, int ld, int slot);
// task addressing its matrix and eigenvalues by pointer (D, eig of the launch unused for it)
void batched_fill_task_ptr(void* dst, double2* D, double* eig, int n, int ld, int slot);

}  // namespace zq
