// Host orchestration and the C ABI of the GB300 quaternion eigensolver.
//
// Drop-in for ts::zquatev (zquatev.h:54, zquatev.cc:42-100): same symbol, same
// arguments, same output layout. Per call:
//   H1  copy the left half [A; B] of D to the device           (zquatev.cc:47-54)
//   H4-H13 blocked quaternion tridiagonalisation (zq_tridiag.cu)  (zquatev.cc:68-72)
//   H14 phase reduction + D&C tridiagonal eigensolver (zq_stedc.cu) (zquatev.cc:74-84)
//   H12/H15 Q Phi formed from the stored reflectors, concurrently with the D&C
//       on a second stream, then (U; V) = (Q Phi) Z    (zquatev.cc:86-90)
//   H16 symmetry fill of the right half on the device    (zquatev.cc:92-98)
//   copy all of D and eig[0..n-1] back.
// H2/H3 (Q init, workspace) become device buffers owned by a per-device
// context; H17 (SuperMatrix, transpose helpers) has no counterpart.
//
// Differences from the reference, all deliberate:
//   * ld2 > n2 works (V is written at rows n..2n-1; the reference writes it at
//     row ld2/2 and reads the input at row n, zquatev.cc:52-53 vs :84,:90);
//   * argument errors return negative codes instead of asserting (zquatev.cc:43);
//   * eig[n..] is left untouched, as in the reference.
#include "zq_common.cuh"
#include "zq_kernels.h"
#include "zq_context.h"
#include "../../include/zquatev_gb300.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

namespace zq {

static thread_local std::string g_last_error;

static std::atomic<long long> g_launches{0};
void count_launch(int k) { g_launches.fetch_add(k, std::memory_order_relaxed); }

void set_last_error(cudaError_t e, const char* what, const char* file, int line) {
  char buf[512];
  snprintf(buf, sizeof(buf), "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
  g_last_error = buf;
}
const char* last_error_message() { return g_last_error.c_str(); }
static void set_msg(const char* m) { g_last_error = m; }
void set_error_message(const char* msg) { g_last_error = msg; }

// ----------------------------------------------------------------------------
// per-kernel-class event timing
// ----------------------------------------------------------------------------
struct Prof {
  std::mutex mu;
  int mask = 0;
  struct Pair { cudaEvent_t a, b; int cls; };
  std::vector<Pair> pairs;
  std::vector<cudaEvent_t> pool;
  int open_idx[PC_COUNT];
  double total_ms[PC_COUNT];
  long long launches[PC_COUNT];
  Prof() { for (int i = 0; i < PC_COUNT; ++i) { open_idx[i] = -1; total_ms[i] = 0; launches[i] = 0; } }
  cudaEvent_t get() {
    if (!pool.empty()) { cudaEvent_t e = pool.back(); pool.pop_back(); return e; }
    cudaEvent_t e; cudaEventCreate(&e); return e;
  }
  void collect() {
    for (auto& p : pairs) {
      float ms = 0.f;
      if (cudaEventSynchronize(p.b) == cudaSuccess && cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
        total_ms[p.cls] += ms;
        launches[p.cls] += 1;
      }
      pool.push_back(p.a); pool.push_back(p.b);
    }
    pairs.clear();
  }
};
static Prof g_prof;

static double g_prof_flops[PC_COUNT];
void prof_add_flops(int cls, double flops) {
  if (!(g_prof.mask & (1 << cls))) return;
  std::lock_guard<std::mutex> lk(g_prof.mu);
  g_prof_flops[cls] += flops;
}

void prof_begin(int cls, cudaStream_t st) {
  if (!(g_prof.mask & (1 << cls))) return;
  std::lock_guard<std::mutex> lk(g_prof.mu);
  Prof::Pair p{g_prof.get(), nullptr, cls};
  cudaEventRecord(p.a, st);
  g_prof.open_idx[cls] = (int)g_prof.pairs.size();
  g_prof.pairs.push_back(p);
}
void prof_end(int cls, cudaStream_t st) {
  if (!(g_prof.mask & (1 << cls))) return;
  std::lock_guard<std::mutex> lk(g_prof.mu);
  const int i = g_prof.open_idx[cls];
  if (i < 0) return;
  g_prof.pairs[i].b = g_prof.get();
  cudaEventRecord(g_prof.pairs[i].b, st);
  g_prof.open_idx[cls] = -1;
  if (g_prof.pairs.size() > 16384) g_prof.collect();
}

static std::mutex g_ctx_mu;
static Context* g_ctx[64];
static int g_nb = 16;   // panel width (autotuned table may override per n; 16 was fastest
                        // for both precisions at n2 = 1024 ... 8192)
static int g_nbq = 64;  // Q-formation block

// Panel width per precision (0 FP64 path, 1 FP32 decomposition of the refined
// path) and size bucket floor(log2 n), filled by zq_autotune_nb; 0 = default.
static std::atomic<int> g_nb_table[2][32];
static int nb_bucket(int n) { int b = 0; while ((2 << b) <= n && b < 31) ++b; return b; }
void nb_table_set(int prec, int n, int nb) { g_nb_table[prec & 1][nb_bucket(n)].store(nb); }
int nb_table_get(int prec, int n) { return g_nb_table[prec & 1][nb_bucket(n)].load(); }

static int nb_for(int n, int prec = 0) {
  if (const char* s = getenv("ZQ_NB")) { const int v = atoi(s); if (v >= 1 && v <= NBMAX) return v; }
  if (const int t = nb_table_get(prec, n)) return t;
  return g_nb;
}

int context_create(int device, Context** out) {
  Context* c = new Context();
  c->device = device;
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->st2, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    set_last_error(e, "context streams/events", __FILE__, __LINE__);
    context_destroy(c);
    return ZQ_ERR_CUDA;
  }
  *out = c;
  return ZQ_OK;
}

void context_destroy(Context* c) {
  if (!c) return;
  if (c->st) cudaStreamSynchronize(c->st);
  if (c->st2) cudaStreamSynchronize(c->st2);
  if (c->ws && !c->ws_external) cudaFree(c->ws);
  if (c->rb.dev && !c->rb.external) cudaFree(c->rb.dev);
  if (c->bb.dev) cudaFree(c->bb.dev);
  if (c->hbuf) cudaFree(c->hbuf);
  if (c->ev_fork) cudaEventDestroy(c->ev_fork);
  if (c->ev_join) cudaEventDestroy(c->ev_join);
  if (c->st) cudaStreamDestroy(c->st);
  if (c->st2) cudaStreamDestroy(c->st2);
  delete c;
}

void context_bind(Context* c, void* ws, size_t ws_bytes, void* rws, size_t rws_bytes) {
  if (c->ws && !c->ws_external) cudaFree(c->ws);
  if (c->rb.dev && !c->rb.external) cudaFree(c->rb.dev);
  c->ws = ws; c->ws_bytes = ws ? ws_bytes : 0; c->ws_external = ws != nullptr;
  c->rb.dev = rws; c->rb.bytes = rws ? rws_bytes : 0; c->rb.external = rws != nullptr;
  c->dc_n = -1;  // the D&C plan lives in the workspace: upload again
}

static int get_context(Context** out) {
  int dev = 0;
  ZQ_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) { set_msg("device ordinal out of range"); return ZQ_ERR_ARG; }
  std::lock_guard<std::mutex> lk(g_ctx_mu);
  if (!g_ctx[dev]) {
    Context* c = nullptr;
    if (int rc = context_create(dev, &c)) return rc;
    g_ctx[dev] = c;
    // the host entry points allocate the device copy of D per call from the
    // stream-ordered pool: keep freed blocks mapped instead of returning them
    // to the driver at every synchronisation
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      uint64_t thr = ~0ull;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
  }
  *out = g_ctx[dev];
  return ZQ_OK;
}

static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// workspace layout for one solve of quaternion size n (excluding the output D)
struct Layout {
  size_t tri, small, dc, fq, nodes, descs, total;
};
static Layout layout_for(int n, int nbmax, int nbq, size_t nnodes, size_t ndescs) {
  Layout L{};
  L.tri = align256(tridiag_workspace_bytes<double>(n, nbmax));
  L.small = align256(sizeof(double) * (size_t)(n + 4 * (size_t)n + n + n + 4 * (size_t)n + n + 16));
  L.dc = align256(sizeof(double) * DcPlan::workspace_doubles(n));
  L.fq = align256(form_q_workspace_bytes(n, nbq));
  L.nodes = align256(sizeof(DcNode) * (nnodes + 1));
  L.descs = align256(DcPlan::desc_bytes(ndescs));
  L.total = L.tri + L.small + L.dc + L.fq + L.nodes + L.descs;
  return L;
}

void solve_workspace_bytes(int n, size_t* fp64_bytes, size_t* refine_bytes) {
  DcPlan probe;
  probe.build(n);
  const Layout L = layout_for(n, NBMAX, g_nbq, probe.num_nodes(), probe.num_descs());
  if (fp64_bytes) *fp64_bytes = L.total;
  if (refine_bytes) *refine_bytes = refine_workspace_bytes(n, g_nbq) + ozaki_workspace_bytes(n) + 4096 + 256;
}

int ensure_ws(Context* c, size_t bytes) {
  if (c->ws_bytes >= bytes) return ZQ_OK;
  if (c->ws_external) { set_msg("bound workspace too small"); return ZQ_ERR_ARG; }
  if (c->ws) { cudaStreamSynchronize(c->st); cudaStreamSynchronize(c->st2); cudaFree(c->ws); c->ws = nullptr; c->ws_bytes = 0; }
  ZQ_CUDA(cudaMalloc(&c->ws, bytes));
  c->ws_bytes = bytes;
  c->dc_n = -1;  // plan pointers refer to the old buffer
  return ZQ_OK;
}

// Solve on device data. dD: n2 x n2 complex (ld ldd) whose left half holds [A; B];
// on return dD holds the eigenvectors and deig[0..n-1] the eigenvalues.
struct StageTimer {
  bool on = false;
  cudaEvent_t ev[8];
  const char* names[8];
  int k = 0;
  explicit StageTimer(bool enable) : on(enable) {
    if (on) for (int i = 0; i < 8; ++i) cudaEventCreate(&ev[i]);
  }
  void mark(const char* name, cudaStream_t st) {
    if (!on || k >= 8) return;
    names[k] = name;
    cudaEventRecord(ev[k++], st);
  }
  ~StageTimer() {
    if (!on) return;
    cudaEventSynchronize(ev[k - 1]);
    for (int i = 1; i < k; ++i) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, ev[i - 1], ev[i]);
      fprintf(stderr, "[zq] %-12s %9.3f ms\n", names[i], ms);
    }
    for (int i = 0; i < 8; ++i) cudaEventDestroy(ev[i]);
  }
};

int solve_device(Context* c, double2* dD, int64_t ldd, int n, double* deig, bool vectors, cudaStream_t st) {
  const int nb = nb_for(n);
  const char* tenv = getenv("ZQ_TIMING");
  StageTimer tm(tenv && tenv[0] == '1');
  const int nbq = g_nbq;
  if (c->dc_n != n) {
    DcPlan probe;
    probe.build(n);
    Layout L = layout_for(n, NBMAX, nbq, probe.num_nodes(), probe.num_descs());
    if (int rc = ensure_ws(c, L.total)) return rc;
    c->dc = probe;
    char* base = reinterpret_cast<char*>(c->ws);
    char* p = base + L.tri + L.small;
    double* dcws = reinterpret_cast<double*>(p); p += L.dc + L.fq;
    DcNode* nodes = reinterpret_cast<DcNode*>(p); p += L.nodes;
    DgemmDesc* descs = reinterpret_cast<DgemmDesc*>(p);
    if (int rc = c->dc.upload(dcws, nodes, descs, c->st)) return rc;
    c->dc_n = n;
  }
  Layout L = layout_for(n, NBMAX, nbq, c->dc.num_nodes(), c->dc.num_descs());
  char* base = reinterpret_cast<char*>(c->ws);
  void* tri_ws = base;
  double* sm = reinterpret_cast<double*>(base + L.tri);
  double* d = sm; sm += n;
  double* e = sm; sm += 4 * (size_t)n;
  double* tau = sm; sm += n;
  double* offd = sm; sm += n;
  double* phi = sm; sm += 4 * (size_t)n;
  double* lam = sm; sm += n;
  void* fq_ws = base + L.tri + L.small + L.dc;
  DgemmDesc* desc1 = reinterpret_cast<DgemmDesc*>(base + L.tri + L.small + L.dc + L.fq + L.nodes) + c->dc.num_descs();

  // the solve runs on the context's streams, ordered after the caller's stream
  ZQ_CUDA(cudaEventRecord(c->ev_fork, st));
  ZQ_CUDA(cudaStreamWaitEvent(c->st, c->ev_fork, 0));

  tm.mark("start", c->st);
  TridiagView<double> v = tridiag_bind<double>(tri_ws, dD, n, ldd, NBMAX, d, e, tau);
  prof_begin(PC_TRIDIAG, c->st);
  if (int rc = tridiagonalize<double>(v, nb, c->st)) return rc;
  prof_end(PC_TRIDIAG, c->st);
  if (int rc = phase_reduce(e, n, offd, phi, c->st)) return rc;
  tm.mark("tridiag", c->st);

  if (vectors) {
    // Q Phi on the second stream, overlapping the tridiagonal solve
    ZQ_CUDA(cudaEventRecord(c->ev_fork, c->st));
    ZQ_CUDA(cudaStreamWaitEvent(c->st2, c->ev_fork, 0));
    double2* X = dD + (int64_t)n * ldd;  // right half as workspace (as the reference does)
    prof_begin(PC_FORMQ, c->st2);
    if (int rc = form_q<double>(dD, ldd, n, phi, X, ldd, nbq, fq_ws, c->st2)) return rc;
    prof_end(PC_FORMQ, c->st2);
    ZQ_CUDA(cudaEventRecord(c->ev_join, c->st2));
    double* Z = nullptr;
    prof_begin(PC_STEDC, c->st);
    if (int rc = c->dc.run(d, offd, lam, Z, c->st)) return rc;
    prof_end(PC_STEDC, c->st);
    tm.mark("stedc", c->st);
    ZQ_CUDA(cudaStreamWaitEvent(c->st, c->ev_join, 0));
    tm.mark("formq-wait", c->st);
    if (int rc = apply_z<double>(X, ldd, Z, n, n, dD, ldd, desc1, c->st)) return rc;
    tm.mark("apply_z", c->st);
    if (int rc = symmetry_fill(dD, ldd, n, c->st)) return rc;
    tm.mark("symfill", c->st);
  } else {
    double* Z = nullptr;
    if (int rc = c->dc.run(d, offd, lam, Z, c->st)) return rc;
  }
  ZQ_CUDA(cudaMemcpyAsync(deig, lam, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->st));
  ZQ_CUDA(cudaEventRecord(c->ev_join, c->st));
  ZQ_CUDA(cudaStreamWaitEvent(st, c->ev_join, 0));
  return ZQ_OK;
}

static int check_args(int n2, const void* D, int ld2, const void* eig) {
  if (n2 < 0 || (n2 & 1)) { set_msg("n2 must be even and non-negative"); return ZQ_ERR_N2; }
  if (n2 == 0) return ZQ_OK;
  if (!D) { set_msg("D is null"); return ZQ_ERR_D; }
  if (ld2 < n2) { set_msg("ld2 < n2"); return ZQ_ERR_LD; }
  if (!eig) { set_msg("eig is null"); return ZQ_ERR_EIG; }
  return ZQ_OK;
}


// Page-locks a caller's pageable host range for the duration of one call, so
// that its copies run as direct DMA. A pageable copy of the same range was
// measured at 5.6 ms per GB D2H in a fresh process but 15-130 ms per GB once
// the process had churned large host allocations; registering 1 GB takes
// 2-5 ms. Memory that is already pinned, or that the driver refuses to
// register, is copied as it is.
struct HostPin {
  void* p = nullptr;
  HostPin(void* ptr, size_t bytes) {
    const char* env = getenv("ZQ_HOST_REGISTER");
    if ((env && env[0] == '0') || bytes < ((size_t)8 << 20)) return;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) { cudaGetLastError(); return; }
    if (a.type != cudaMemoryTypeUnregistered) return;
    if (cudaHostRegister(ptr, bytes, cudaHostRegisterDefault) == cudaSuccess) p = ptr;
    else cudaGetLastError();
  }
  ~HostPin() {
    if (p) cudaHostUnregister(p);
  }
};

// host-memory drop-in (path: -1 policy, 0 FP64, 1 refined)
static int zquatev_host(int n2, double2* D, int ld2, double* eig, bool vectors, int path = -1) {
  if (int rc = check_args(n2, D, ld2, eig)) return rc;
  if (n2 == 0) return ZQ_OK;
  const int n = n2 / 2;
  Context* c = nullptr;
  if (int rc = get_context(&c)) return rc;
  std::lock_guard<std::mutex> lk(c->mu);
  // device copy of D: n2 x n2 with ld = n2 (plus eigenvalues), in the
  // context's host-path buffer (grown on demand, kept between calls)
  const size_t dbytes = sizeof(double2) * (size_t)n2 * n2;
  const size_t need = dbytes + sizeof(double) * n + 256;
  if (c->hbuf_bytes < need) {
    if (c->hbuf) { cudaStreamSynchronize(c->st); cudaFree(c->hbuf); c->hbuf = nullptr; c->hbuf_bytes = 0; }
    ZQ_CUDA(cudaMalloc(&c->hbuf, need));
    c->hbuf_bytes = need;
  }
  double2* dD = reinterpret_cast<double2*>(c->hbuf);
  double* deig = reinterpret_cast<double*>(reinterpret_cast<char*>(dD) + dbytes);
  int rc = ZQ_OK;
  // ZQ_TIMING=1: host-clock time of each phase (the stream is synchronised after each)
  const char* tenv = getenv("ZQ_TIMING");
  const bool timing = tenv && tenv[0] == '1';
  auto t_last = std::chrono::steady_clock::now();
  auto phase = [&](const char* name) {
    if (!timing) return;
    cudaStreamSynchronize(c->st);
    const auto t = std::chrono::steady_clock::now();
    fprintf(stderr, "[zq] host %-8s %9.3f ms\n", name, std::chrono::duration<double, std::milli>(t - t_last).count());
    t_last = t;
  };
  // the span of D the call touches: the left half is read; with vectors all n2 columns are written
  const size_t span = sizeof(double2) * ((size_t)ld2 * ((vectors ? n2 : n) - 1) + n2);
  HostPin pin(D, span);
  phase("pin");
  do {
    // H1: only the left half is read
    if (cudaMemcpy2DAsync(dD, sizeof(double2) * n2, D, sizeof(double2) * (size_t)ld2, sizeof(double2) * n2, n,
                          cudaMemcpyHostToDevice, c->st) != cudaSuccess) { rc = ZQ_ERR_CUDA; set_msg("H2D copy failed"); break; }
    phase("h2d");
    const int p = (path >= 0) ? path : path_for(n);
    cudaEvent_t te[2];
    if (timing) { cudaEventCreate(&te[0]); cudaEventCreate(&te[1]); cudaEventRecord(te[0], c->st); }
    rc = (vectors && p == 1) ? refined_device(c, dD, n2, n, deig, c->st, 1) : solve_device(c, dD, n2, n, deig, vectors, c->st);
    if (timing) {
      float gms = 0.f;
      cudaEventRecord(te[1], c->st);
      cudaEventSynchronize(te[1]);
      cudaEventElapsedTime(&gms, te[0], te[1]);
      fprintf(stderr, "[zq] device solve %9.3f ms (events)\n", gms);
      cudaEventDestroy(te[0]); cudaEventDestroy(te[1]);
    }
    if (rc) break;
    phase("solve");
    if (vectors) {
      if (cudaMemcpy2DAsync(D, sizeof(double2) * (size_t)ld2, dD, sizeof(double2) * n2, sizeof(double2) * n2, n2,
                            cudaMemcpyDeviceToHost, c->st) != cudaSuccess) { rc = ZQ_ERR_CUDA; set_msg("D2H copy failed"); break; }
    }
    if (cudaMemcpyAsync(eig, deig, sizeof(double) * n, cudaMemcpyDeviceToHost, c->st) != cudaSuccess) {
      rc = ZQ_ERR_CUDA; set_msg("D2H eig copy failed"); break;
    }
    cudaError_t e = cudaStreamSynchronize(c->st);
    if (e != cudaSuccess) { set_last_error(e, "cudaStreamSynchronize", __FILE__, __LINE__); rc = ZQ_ERR_CUDA; break; }
    phase("d2h");
  } while (0);
  cudaStreamSynchronize(c->st);
  return rc;
}

// ----------------------------------------------------------------------------
// refined (mixed-precision) path
// ----------------------------------------------------------------------------

int ensure_plan(Context* c, int n) {
  if (c->dc_n == n) return ZQ_OK;
  DcPlan probe;
  probe.build(n);
  Layout L = layout_for(n, NBMAX, g_nbq, probe.num_nodes(), probe.num_descs());
  if (int rc = ensure_ws(c, L.total)) return rc;
  c->dc = probe;
  char* base = reinterpret_cast<char*>(c->ws);
  char* p = base + L.tri + L.small;
  double* dcws = reinterpret_cast<double*>(p); p += L.dc + L.fq;
  DcNode* nodes = reinterpret_cast<DcNode*>(p); p += L.nodes;
  if (int rc = c->dc.upload(dcws, nodes, reinterpret_cast<DgemmDesc*>(p), c->st)) return rc;
  c->dc_n = n;
  return ZQ_OK;
}

int refined_device(Context* c, double2* dD, int64_t ldd, int n, double* deig, cudaStream_t st, int mode) {
  if (int rc = ensure_plan(c, n)) return rc;
  RefineBuffers& rb = c->rb;
  const size_t need = refine_workspace_bytes(n, g_nbq) + (mode == 1 ? ozaki_workspace_bytes(n) : 0) + 4096;
  if (rb.bytes < need) {
    if (rb.external) { set_msg("bound refinement workspace too small"); return ZQ_ERR_ARG; }
    if (rb.dev) { cudaStreamSynchronize(c->st); cudaFree(rb.dev); rb.dev = nullptr; rb.bytes = 0; }
    ZQ_CUDA(cudaMalloc(&rb.dev, need));
    rb.bytes = need;
  }
  Layout L = layout_for(n, NBMAX, g_nbq, c->dc.num_nodes(), c->dc.num_descs());
  DgemmDesc* desc1 = reinterpret_cast<DgemmDesc*>(reinterpret_cast<char*>(c->ws) + L.tri + L.small + L.dc + L.fq + L.nodes) +
                     c->dc.num_descs();
  RefineArgs ra{};
  ra.dD = dD; ra.ldd = ldd; ra.n = n; ra.deig = deig;
  ra.ws = reinterpret_cast<char*>(rb.dev) + 4096;
  const size_t rws = refine_workspace_bytes(n, g_nbq);
  ra.ows = (mode == 1) ? reinterpret_cast<char*>(ra.ws) + ((rws + 255) & ~(size_t)255) : nullptr;
  ra.ows_bytes = (mode == 1) ? ozaki_workspace_bytes(n) : 0;
  ra.dc = &c->dc;
  ra.coop = c->coop ? 1 : 0;
  ra.fdesc = reinterpret_cast<DgemmDescT<float>*>(desc1);
  ra.nb = nb_for(n, 1); ra.nbq = g_nbq; ra.mode = mode;
  ra.max_iter = 6;
  ra.tol = 1e-7;   // the update squares the error: |E| <= 1e-7 leaves ~1e-14
  ra.cluster_tol = 1e-13;
  ra.pair_eps = 1e-4;  // |E| <= 1e-4 from the formula: two more steps reach 1e-7
  // After the first step a correction above 1e-6 means a pair whose gap is too
  // small for the first-order formula to converge quadratically (seen on a
  // random n2 = 8192 matrix: one pair's |E| stayed at 5e-5 for two steps); such
  // pairs are rotated like clusters instead.
  ra.pair_eps_late = 1e-6;
  if (const char* s = getenv("ZQ_REFINE_EPS_LATE")) { const double v = atof(s); if (v > 0.0 && v < 0.5) ra.pair_eps_late = v; }
  ra.slices0 = 5;
  if (const char* s = getenv("ZQ_REFINE_SLICES0")) { const int v = atoi(s); if (v >= 3 && v <= 8) ra.slices0 = v; }
  ra.slices_res = 4;
  if (const char* s = getenv("ZQ_REFINE_RSLICES")) { const int v = atoi(s); if (v >= 2 && v <= 8) ra.slices_res = v; }
  if (const char* s = getenv("ZQ_REFINE_MAXIT")) ra.max_iter = atoi(s);
  if (const char* s = getenv("ZQ_REFINE_EPS")) { const double v = atof(s); if (v > 0.0 && v < 0.5) ra.pair_eps = v; }
  ra.st = c->st;
  ra.st2 = c->st2;
  ra.ev_fork = c->ev_fork;
  ra.ev_join = c->ev_join;
  ZQ_CUDA(cudaEventRecord(c->ev_fork, st));
  ZQ_CUDA(cudaStreamWaitEvent(c->st, c->ev_fork, 0));
  if (int rc = refined_solve(ra)) return rc;
  rb.last_iters = ra.iters;
  rb.last_emax = ra.last_emax;
  rb.last_fallback = 0;
  if (!(ra.last_emax <= ra.tol) || ra.clusters < 0) {
    // not converged (e.g. clustered eigenvalues): restore the input saved at
    // the start of the refined solve and run the plain FP64 path
    const double2* H0 = reinterpret_cast<const double2*>(ra.ws);
    ZQ_CUDA(cudaMemcpy2DAsync(dD, sizeof(double2) * ldd, H0, sizeof(double2) * 2 * n, sizeof(double2) * 2 * n, n,
                              cudaMemcpyDeviceToDevice, c->st));
    rb.last_fallback = 1;
    if (int rc = solve_device(c, dD, ldd, n, deig, true, c->st)) return rc;
  }
  ZQ_CUDA(cudaEventRecord(c->ev_join, c->st));
  ZQ_CUDA(cudaStreamWaitEvent(st, c->ev_join, 0));
  return ZQ_OK;
}

// path policy of the drop-in entry points: 0 FP64, 1 refined, 2 auto
static int g_path = 2;
int path_for(int n) {
  int p = g_path;
  if (const char* s = getenv("ZQ_PATH")) {
    if (!strcmp(s, "fp64")) p = 0; else if (!strcmp(s, "refined")) p = 1; else if (!strcmp(s, "auto")) p = 2;
  }
  if (p == 2) p = (n >= 48) ? 1 : 0;  // refined measured faster from n = 48 up (2-4x)
  return p;
}

// ----------------------------------------------------------------------------
// batched: small matrices (n <= batched_max_n()) in one persistent kernel,
// larger ones through the per-matrix path on the same stream
// ----------------------------------------------------------------------------

static int g_batch_ctas_per_sm = 2;

static int batched_solve(int count, const int* n2s, const int* ld2s, const long long* offs, const long long* eoffs,
                         double2* dD, double* deig, cudaStream_t st) {
  Context* c = nullptr;
  if (int rc = get_context(&c)) return rc;
  std::lock_guard<std::mutex> lk(c->mu);
  const int nmax = batched_max_n();
  // small tasks, largest first (longest-processing-time order)
  std::vector<int> small, large;
  for (int b = 0; b < count; ++b) {
    if (n2s[b] == 0) continue;
    ((n2s[b] / 2 <= nmax) ? small : large).push_back(b);
  }
  std::stable_sort(small.begin(), small.end(), [&](int x, int y) { return n2s[x] > n2s[y]; });
  int info_max = 0;
  if (!small.empty()) {
    int sms = 0;
    ZQ_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
    const char* env = getenv("ZQ_BATCH_CTAS_PER_SM");
    const int per_sm = env ? atoi(env) : g_batch_ctas_per_sm;
    int ctas = sms * (per_sm > 0 ? per_sm : 2);
    if (ctas > (int)small.size()) ctas = (int)small.size();
    const size_t tb = batched_task_bytes();
    const size_t task_bytes = align256(tb * small.size());
    const size_t info_bytes = align256(sizeof(int) * small.size() + sizeof(int));
    const size_t ws_bytes = sizeof(double) * (size_t)batched_ws_stride() * ctas;
    const size_t need = task_bytes + info_bytes + ws_bytes;
    BatchBuffers& bb = c->bb;
    if (bb.bytes < need) {
      if (bb.dev) { cudaStreamSynchronize(c->st); cudaFree(bb.dev); bb.dev = nullptr; bb.bytes = 0; }
      ZQ_CUDA(cudaMalloc(&bb.dev, need));
      bb.bytes = need;
    }
    char* base = reinterpret_cast<char*>(bb.dev);
    void* dtasks = base;
    int* dinfo = reinterpret_cast<int*>(base + task_bytes);
    int* dcounter = dinfo + small.size();
    double* dws = reinterpret_cast<double*>(base + task_bytes + info_bytes);
    bb.host_tasks.resize(tb * small.size());
    for (size_t q = 0; q < small.size(); ++q) {
      const int b = small[q];
      batched_fill_task(bb.host_tasks.data() + q * tb, offs[b], eoffs[b], n2s[b] / 2, ld2s[b], (int)q);
    }
    ZQ_CUDA(cudaEventRecord(c->ev_fork, st));
    ZQ_CUDA(cudaStreamWaitEvent(c->st, c->ev_fork, 0));
    ZQ_CUDA(cudaMemcpyAsync(dtasks, bb.host_tasks.data(), tb * small.size(), cudaMemcpyHostToDevice, c->st));
    if (int rc = batched_launch(dtasks, (int)small.size(), dcounter, dD, deig, dws, ctas, dinfo, c->st)) return rc;
    std::vector<int> hinfo(small.size());
    ZQ_CUDA(cudaMemcpyAsync(hinfo.data(), dinfo, sizeof(int) * small.size(), cudaMemcpyDeviceToHost, c->st));
    ZQ_CUDA(cudaStreamSynchronize(c->st));
    for (int v : hinfo) info_max = v > info_max ? v : info_max;
  }
  for (int b : large) {
    if (int rc = solve_device(c, dD + offs[b], ld2s[b], n2s[b] / 2, deig + eoffs[b], true, st)) return rc;
  }
  ZQ_CUDA(cudaStreamSynchronize(st));
  return info_max;
}

}  // namespace zq

using namespace zq;

extern "C" {

int zquatev_c(int n2, double* D, int ld2, double* eig) {
  return zquatev_host(n2, reinterpret_cast<double2*>(D), ld2, eig, true);
}

int zquatev_values(int n2, double* D, int ld2, double* eig) {
  return zquatev_host(n2, reinterpret_cast<double2*>(D), ld2, eig, false);
}

int zquatev_device(int n2, double* dD, int ld2, double* deig, void* stream) {
  if (int rc = check_args(n2, dD, ld2, deig)) return rc;
  if (n2 == 0) return ZQ_OK;
  Context* c = nullptr;
  if (int rc = get_context(&c)) return rc;
  std::lock_guard<std::mutex> lk(c->mu);
  if (path_for(n2 / 2) == 1)
    return refined_device(c, reinterpret_cast<double2*>(dD), ld2, n2 / 2, deig, reinterpret_cast<cudaStream_t>(stream), 1);
  return solve_device(c, reinterpret_cast<double2*>(dD), ld2, n2 / 2, deig, true, reinterpret_cast<cudaStream_t>(stream));
}

int zquatev_fp64_device(int n2, double* dD, int ld2, double* deig, void* stream) {
  if (int rc = check_args(n2, dD, ld2, deig)) return rc;
  if (n2 == 0) return ZQ_OK;
  Context* c = nullptr;
  if (int rc = get_context(&c)) return rc;
  std::lock_guard<std::mutex> lk(c->mu);
  return solve_device(c, reinterpret_cast<double2*>(dD), ld2, n2 / 2, deig, true, reinterpret_cast<cudaStream_t>(stream));
}

int zquatev_fp64_c(int n2, double* D, int ld2, double* eig) {
  return zquatev_host(n2, reinterpret_cast<double2*>(D), ld2, eig, true, 0);
}

int zquatev_refined_c(int n2, double* D, int ld2, double* eig) {
  return zquatev_host(n2, reinterpret_cast<double2*>(D), ld2, eig, true, 1);
}

int zq_set_path(int path) {
  if (path < 0 || path > 2) { set_msg("path must be 0 (FP64), 1 (refined) or 2 (auto)"); return ZQ_ERR_ARG; }
  g_path = path;
  return ZQ_OK;
}

int zquatev_values_device(int n2, double* dD, int ld2, double* deig, void* stream) {
  if (int rc = check_args(n2, dD, ld2, deig)) return rc;
  if (n2 == 0) return ZQ_OK;
  Context* c = nullptr;
  if (int rc = get_context(&c)) return rc;
  std::lock_guard<std::mutex> lk(c->mu);
  return solve_device(c, reinterpret_cast<double2*>(dD), ld2, n2 / 2, deig, false, reinterpret_cast<cudaStream_t>(stream));
}

int zq_stedc_device(int n, const double* d, const double* e, double* lam, double* Z, int ldz, void* stream) {
  if (n < 0) { set_msg("n < 0"); return ZQ_ERR_ARG; }
  if (n == 0) return ZQ_OK;
  if (!d || !lam || !Z || (n > 1 && !e) || ldz < n) { set_msg("bad stedc arguments"); return ZQ_ERR_ARG; }
  Context* c = nullptr;
  if (int rc = get_context(&c)) return rc;
  std::lock_guard<std::mutex> lk(c->mu);
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  if (c->dc_n != n) {
    DcPlan probe;
    probe.build(n);
    Layout L = layout_for(n, NBMAX, g_nbq, probe.num_nodes(), probe.num_descs());
    if (int rc = ensure_ws(c, L.total)) return rc;
    c->dc = probe;
    char* base = reinterpret_cast<char*>(c->ws);
    char* p = base + L.tri + L.small;
    double* dcws = reinterpret_cast<double*>(p); p += L.dc + L.fq;
    DcNode* nodes = reinterpret_cast<DcNode*>(p); p += L.nodes;
    if (int rc = c->dc.upload(dcws, nodes, reinterpret_cast<DgemmDesc*>(p), c->st)) return rc;
    c->dc_n = n;
  }
  ZQ_CUDA(cudaEventRecord(c->ev_fork, st));
  ZQ_CUDA(cudaStreamWaitEvent(c->st, c->ev_fork, 0));
  double* Zi = nullptr;
  if (int rc = c->dc.run(d, e, lam, Zi, c->st)) return rc;
  ZQ_CUDA(cudaMemcpy2DAsync(Z, sizeof(double) * (size_t)ldz, Zi, sizeof(double) * n, sizeof(double) * n, n,
                            cudaMemcpyDeviceToDevice, c->st));
  ZQ_CUDA(cudaEventRecord(c->ev_join, c->st));
  ZQ_CUDA(cudaStreamWaitEvent(st, c->ev_join, 0));
  return ZQ_OK;
}

int zquatev_batched_device(int count, const int* n2s, const int* ld2s, const long long* offs,
                           const long long* eoffs, double* dD, double* deig, void* stream) {
  if (count < 0 || (count > 0 && (!n2s || !ld2s || !offs || !eoffs || !dD || !deig))) {
    set_msg("bad batched arguments");
    return ZQ_ERR_ARG;
  }
  for (int b = 0; b < count; ++b)
    if (int rc = check_args(n2s[b], dD, ld2s[b], deig)) return rc;
  if (count == 0) return ZQ_OK;
  return batched_solve(count, n2s, ld2s, offs, eoffs, reinterpret_cast<double2*>(dD), deig,
                       reinterpret_cast<cudaStream_t>(stream));
}

int zquatev_refined_device(int n2, double* dD, int ld2, double* deig, void* stream, int mode) {
  if (int rc = check_args(n2, dD, ld2, deig)) return rc;
  if (n2 == 0) return ZQ_OK;
  if (mode < 0 || mode > 1) { set_msg("mode must be 0 (FP64 products) or 1 (Ozaki tensor-core products)"); return ZQ_ERR_ARG; }
  Context* c = nullptr;
  if (int rc = get_context(&c)) return rc;
  std::lock_guard<std::mutex> lk(c->mu);
  return refined_device(c, reinterpret_cast<double2*>(dD), ld2, n2 / 2, deig, reinterpret_cast<cudaStream_t>(stream), mode);
}

int zq_refine_stats(int* iters, double* last_correction, int* fell_back) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return ZQ_ERR_CUDA;
  Context* c = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_ctx_mu);
    c = g_ctx[dev];
  }
  if (iters) *iters = c ? c->rb.last_iters : 0;
  if (last_correction) *last_correction = c ? c->rb.last_emax : 0.0;
  if (fell_back) *fell_back = c ? c->rb.last_fallback : 0;
  return ZQ_OK;
}

int zq_profile_enable(int mask) {
  std::lock_guard<std::mutex> lk(g_prof.mu);
  g_prof.mask = mask;
  return ZQ_OK;
}

int zq_profile_read(int cls, double* total_ms, long long* launches) {
  if (cls < 0 || cls >= PC_COUNT || !total_ms || !launches) { set_msg("bad profile class"); return ZQ_ERR_ARG; }
  std::lock_guard<std::mutex> lk(g_prof.mu);
  g_prof.collect();
  *total_ms = g_prof.total_ms[cls];
  *launches = g_prof.launches[cls];
  return ZQ_OK;
}

int zq_profile_reset(void) {
  std::lock_guard<std::mutex> lk(g_prof.mu);
  g_prof.collect();
  for (int i = 0; i < PC_COUNT; ++i) { g_prof.total_ms[i] = 0; g_prof.launches[i] = 0; g_prof_flops[i] = 0; }
  return ZQ_OK;
}

int zq_profile_flops(int cls, double* flops) {
  if (cls < 0 || cls >= PC_COUNT || !flops) { set_msg("bad profile class"); return ZQ_ERR_ARG; }
  std::lock_guard<std::mutex> lk(g_prof.mu);
  *flops = g_prof_flops[cls];
  return ZQ_OK;
}

int zq_set_block_size(int nb) {
  if (nb < 1 || nb > NBMAX) { set_msg("block size must be in [1, 128]"); return ZQ_ERR_ARG; }
  g_nb = nb;
  for (auto& row : g_nb_table)
    for (auto& v : row) v.store(0);  // an explicit width replaces the tuned table
  return ZQ_OK;
}

int zq_get_block_size(void) { return g_nb; }

const char* zq_last_error(void) { return last_error_message(); }

int zq_version(void) { return 100; }

int zq_set_pipeline_wait(long long cycles) {
  zq::set_pipeline_wait_cycles(cycles);
  return ZQ_OK;
}

long long zq_launch_count(void) { return zq::g_launches.load(std::memory_order_relaxed); }

int zq_release_workspace(void) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return ZQ_ERR_CUDA;
  std::lock_guard<std::mutex> lk(g_ctx_mu);
  Context* c = g_ctx[dev];
  if (!c) return ZQ_OK;
  std::lock_guard<std::mutex> lk2(c->mu);
  cudaStreamSynchronize(c->st);
  cudaStreamSynchronize(c->st2);
  if (c->ws) cudaFree(c->ws);
  c->ws = nullptr;
  c->ws_bytes = 0;
  c->dc_n = -1;
  if (c->hbuf) cudaFree(c->hbuf);
  c->hbuf = nullptr;
  c->hbuf_bytes = 0;
  return ZQ_OK;
}

}  // extern "C"

// The reference's own symbol (C++ linkage): ts::zquatev(int, std::complex<double>*, int, double*)
namespace ts {
int zquatev(const int n2, std::complex<double>* const D, const int ld2, double* const eig) {
  return zquatev_c(n2, reinterpret_cast<double*>(D), ld2, eig);
}
}  // namespace ts
