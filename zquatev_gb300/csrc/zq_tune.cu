// Autotuning and the graph-captured batch plan.
//
// * zq_autotune_nb times the quaternion tridiagonalisation (the only stage the
//   panel width changes) for each candidate width on a seeded random matrix of
//   the requested size and stores the fastest in the per-size table that the
//   solves read (one table for the FP64 path, one for the refined path's FP32
//   decomposition). The reference hard-codes nb = 20 (zquatev.cc:64).
// * zq_batch_plan: one batch layout of small matrices (n2 <= 512) solved
//   repeatedly. The tasks are ordered largest first and uploaded once; on the
//   first run the launch shape of the persistent kernel (CTAs per SM) is chosen
//   by timing each candidate on the caller's batch (input restored between
//   candidates); the counter reset and the kernel are then captured in a CUDA
//   graph, and every run replays it with one cudaGraphLaunch.
#include "zq_common.cuh"
#include "zq_context.h"
#include "zq_kernels.h"

#include <type_traits>
#include "../../include/zquatev_gb300.h"

#include <algorithm>
#include <cstdint>
#include <vector>

namespace zq {
namespace {

__device__ __forceinline__ double tune_hash(uint64_t x) {
  // splitmix64 -> uniform in [-1, 1)
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  x ^= x >> 31;
  return (double)(x >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

// [A; B] with A Hermitian, B antisymmetric (lower triangles are what the reduction reads)
template <typename R>
__global__ void k_tune_fill(cplx<R>* M, int n, int64_t ld, uint64_t seed) {
  const int64_t total = (int64_t)n * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % n), j = (int)(t / n);
    const int lo = i > j ? i : j, hi = i > j ? j : i;
    const uint64_t key = seed * 0x100000001B3ull + (uint64_t)lo * (uint64_t)n + (uint64_t)hi;
    double ar = tune_hash(4 * key), ai = tune_hash(4 * key + 1);
    double br = tune_hash(4 * key + 2), bi = tune_hash(4 * key + 3);
    if (i == j) { ai = 0.0; br = 0.0; bi = 0.0; }
    if (i < j) { ai = -ai; br = -br; bi = -bi; }  // A = A^H, B = -B^T
    M[i + (int64_t)j * ld] = mk((R)ar, (R)ai);
    M[n + i + (int64_t)j * ld] = mk((R)br, (R)bi);
  }
}

template <typename R>
int tune_nb(int n, const int* cand, int ncand, double* ms_out, int* best, cudaStream_t st) {
  const size_t mbytes = sizeof(cplx<R>) * (size_t)2 * n * n;
  const size_t wbytes = tridiag_workspace_bytes<R>(n, NBMAX);
  const size_t sbytes = sizeof(double) * (size_t)(6 * n + 16);
  void* mem = nullptr;
  ZQ_CUDA(cudaMallocAsync(&mem, mbytes + wbytes + sbytes + 1024 + 256, st));
  char* p = reinterpret_cast<char*>(mem);
  cplx<R>* M = reinterpret_cast<cplx<R>*>(p);
  void* ws = p + ((mbytes + 255) & ~(size_t)255);
  double* sm = reinterpret_cast<double*>(p + ((mbytes + 255) & ~(size_t)255) + ((wbytes + 255) & ~(size_t)255));
  double* d = sm;
  double* e = sm + n;
  double* tau = sm + 5 * (size_t)n;
  TridiagView<R> v = tridiag_bind<R>(ws, M, n, 2 * n, NBMAX, d, e, tau);
  if (std::is_same<R, float>::value) {
    // time the FP32 reduction as the refined path runs it
    v.tc_err = reinterpret_cast<int*>(p + ((mbytes + 255) & ~(size_t)255) + ((wbytes + 255) & ~(size_t)255) +
                                      ((sbytes + 255) & ~(size_t)255));
    ZQ_CUDA(cudaMemsetAsync(v.tc_err, 0, sizeof(int), st));
  }
  cudaEvent_t e0, e1;
  ZQ_CUDA(cudaEventCreate(&e0));
  ZQ_CUDA(cudaEventCreate(&e1));
  int rc = ZQ_OK;
  double best_ms = 1e300;
  const int blocks = (int)std::min<int64_t>(4096, ((int64_t)n * n + 255) / 256);
  for (int c = -1; c < ncand && rc == ZQ_OK; ++c) {  // c = -1: warm-up with the first candidate
    const int nb = cand[c < 0 ? 0 : c];
    k_tune_fill<R><<<blocks, 256, 0, st>>>(M, n, 2 * n, 12345u);
    count_launch();
    if (cudaGetLastError() != cudaSuccess) { rc = ZQ_ERR_CUDA; break; }
    cudaEventRecord(e0, st);
    rc = tridiagonalize<R>(v, nb, st);
    cudaEventRecord(e1, st);
    if (cudaEventSynchronize(e1) != cudaSuccess) rc = ZQ_ERR_CUDA;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (c >= 0) {
      if (ms_out) ms_out[c] = ms;
      if (ms < best_ms) { best_ms = ms; *best = nb; }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(mem, st);
  if (cudaStreamSynchronize(st) != cudaSuccess && rc == ZQ_OK) rc = ZQ_ERR_CUDA;
  return rc;
}

}  // namespace
}  // namespace zq

// ----------------------------------------------------------------- batch plan
struct zq_batch_plan {
  int device = 0, sms = 0, count = 0, ntask = 0;
  int ctas_per_sm = 0, ctas = 0;
  bool tuned = false;
  double tune_ms[4] = {0, 0, 0, 0};
  int warp_max = -1;               // switch size of the warp variant (tuned)
  double variant_ms[4] = {0, 0, 0, 0};
  long long extent = 0;            // complex elements of D the batch touches
  void* dev = nullptr;             // tasks | info (+ counter) | per-CTA workspace
  size_t task_bytes = 0, info_bytes = 0;
  cudaStream_t cap = nullptr;      // capture stream
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  double2* gD = nullptr;           // pointers baked into the graph
  double* gE = nullptr;
  int gctas = 0;
};

namespace zq {
namespace {

constexpr int PLAN_MAX_CPS = 4;

void* plan_ws(zq_batch_plan* p) { return reinterpret_cast<char*>(p->dev) + p->task_bytes + p->info_bytes; }
int* plan_info(zq_batch_plan* p) { return reinterpret_cast<int*>(reinterpret_cast<char*>(p->dev) + p->task_bytes); }

int plan_launch_direct(zq_batch_plan* p, double2* D, double* E, int ctas, cudaStream_t st, int wmax) {
  int* info = plan_info(p);
  return batched_launch(p->dev, p->ntask, info + p->ntask, D, E, reinterpret_cast<double*>(plan_ws(p)), ctas, info, st,
                        wmax);
}
// candidates of the warp variant's switch size (0: CTA variant for every size)
constexpr int PLAN_WMAX[4] = {0, 16, 24, 32};

int plan_tune(zq_batch_plan* p, double2* D, double* E, cudaStream_t st) {
  // keep the caller's input: every candidate overwrites it
  void* save = nullptr;
  const size_t bytes = sizeof(double2) * (size_t)p->extent;
  ZQ_CUDA(cudaMallocAsync(&save, bytes, st));
  ZQ_CUDA(cudaMemcpyAsync(save, D, bytes, cudaMemcpyDeviceToDevice, st));
  cudaEvent_t e0, e1;
  ZQ_CUDA(cudaEventCreate(&e0));
  ZQ_CUDA(cudaEventCreate(&e1));
  double best = 1e300;
  int rc = ZQ_OK;
  // 1) launch shape (CTAs per SM) with the default switch size
  const int w0 = batched_warp_max();
  for (int cps = 1; cps <= PLAN_MAX_CPS && rc == ZQ_OK; ++cps) {
    const int ctas = std::min(p->ntask, cps * p->sms);
    if (cps > 1 && ctas == std::min(p->ntask, (cps - 1) * p->sms)) break;  // no more CTAs than tasks
    if (cudaMemcpyAsync(D, save, bytes, cudaMemcpyDeviceToDevice, st) != cudaSuccess) { rc = ZQ_ERR_CUDA; break; }
    cudaEventRecord(e0, st);
    rc = plan_launch_direct(p, D, E, ctas, st, w0);
    cudaEventRecord(e1, st);
    if (cudaEventSynchronize(e1) != cudaSuccess) rc = ZQ_ERR_CUDA;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    p->tune_ms[cps - 1] = ms;
    if (ms < best) { best = ms; p->ctas_per_sm = cps; }
  }
  // 2) the per-size variant: largest order solved warp-per-matrix (the rest
  //    one CTA per matrix), at that launch shape
  p->warp_max = w0;
  best = 1e300;
  const int ctas = std::min(p->ntask, p->ctas_per_sm * p->sms);
  for (int q = 0; q < 4 && rc == ZQ_OK; ++q) {
    if (cudaMemcpyAsync(D, save, bytes, cudaMemcpyDeviceToDevice, st) != cudaSuccess) { rc = ZQ_ERR_CUDA; break; }
    cudaEventRecord(e0, st);
    rc = plan_launch_direct(p, D, E, ctas, st, PLAN_WMAX[q]);
    cudaEventRecord(e1, st);
    if (cudaEventSynchronize(e1) != cudaSuccess) rc = ZQ_ERR_CUDA;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    p->variant_ms[q] = ms;
    if (ms < best) { best = ms; p->warp_max = PLAN_WMAX[q]; }
  }
  if (rc == ZQ_OK && cudaMemcpyAsync(D, save, bytes, cudaMemcpyDeviceToDevice, st) != cudaSuccess) rc = ZQ_ERR_CUDA;
  cudaFreeAsync(save, st);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  p->tuned = true;
  return rc;
}

int plan_capture(zq_batch_plan* p, double2* D, double* E) {
  if (p->exec) { cudaGraphExecDestroy(p->exec); p->exec = nullptr; }
  if (p->graph) { cudaGraphDestroy(p->graph); p->graph = nullptr; }
  const int ctas = std::min(p->ntask, p->ctas_per_sm * p->sms);
  ZQ_CUDA(cudaStreamBeginCapture(p->cap, cudaStreamCaptureModeThreadLocal));
  int rc = plan_launch_direct(p, D, E, ctas, p->cap, p->warp_max);
  cudaGraph_t g = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(p->cap, &g);
  count_launch(-1);  // capturing ran nothing; replays are counted
  if (rc != ZQ_OK) { if (g) cudaGraphDestroy(g); return rc; }
  if (ce != cudaSuccess) { set_last_error(ce, "cudaStreamEndCapture", __FILE__, __LINE__); return ZQ_ERR_CUDA; }
  p->graph = g;
  ZQ_CUDA(cudaGraphInstantiate(&p->exec, p->graph, 0));
  p->gD = D; p->gE = E; p->gctas = ctas;
  return ZQ_OK;
}

}  // namespace
}  // namespace zq

using namespace zq;

extern "C" {

int zq_autotune_nb(int n2, int precision, int* best_nb, double* ms) {
  if (n2 < 4 || (n2 & 1) || (precision != 0 && precision != 1) || !best_nb) {
    set_error_message("zq_autotune_nb: n2 even >= 4, precision 0 (FP64) or 1 (FP32)");
    return ZQ_ERR_ARG;
  }
  const int n = n2 / 2;
  static const int cand[4] = {16, 32, 64, 128};
  cudaStream_t st;
  ZQ_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  int best = 32;
  const int rc = precision == 0 ? tune_nb<double>(n, cand, 4, ms, &best, st) : tune_nb<float>(n, cand, 4, ms, &best, st);
  cudaStreamDestroy(st);
  if (rc) return rc;
  nb_table_set(precision, n, best);
  *best_nb = best;
  return ZQ_OK;
}

int zq_tuned_nb(int n2, int precision) {
  if (n2 < 2 || (n2 & 1) || (precision != 0 && precision != 1)) return ZQ_ERR_ARG;
  return nb_table_get(precision, n2 / 2);
}

int zq_set_tuned_nb(int n2, int precision, int nb) {
  if (n2 < 2 || (n2 & 1) || (precision != 0 && precision != 1) || nb < 0 || nb > NBMAX) {
    set_error_message("zq_set_tuned_nb: bad arguments");
    return ZQ_ERR_ARG;
  }
  nb_table_set(precision, n2 / 2, nb);
  return ZQ_OK;
}

zq_batch_plan* zq_batch_plan_create(int count, const int* n2s, const int* ld2s, const long long* offs,
                                    const long long* eoffs, int ctas_per_sm) {
  if (count <= 0 || !n2s || !ld2s || !offs || !eoffs || ctas_per_sm < 0 || ctas_per_sm > PLAN_MAX_CPS) {
    set_error_message("zq_batch_plan_create: bad arguments");
    return nullptr;
  }
  const int nmax = batched_max_n();
  std::vector<int> order;
  long long extent = 0;
  for (int b = 0; b < count; ++b) {
    const int n2 = n2s[b];
    if (n2 < 0 || (n2 & 1) || ld2s[b] < n2 || offs[b] < 0 || eoffs[b] < 0) {
      set_error_message("zq_batch_plan_create: bad n2 / ld2 / offset");
      return nullptr;
    }
    if (n2 / 2 > nmax) { set_error_message("zq_batch_plan_create: every n2 must be <= 512"); return nullptr; }
    if (n2 == 0) continue;
    order.push_back(b);
    extent = std::max(extent, offs[b] + (long long)ld2s[b] * n2);
  }
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return n2s[x] > n2s[y]; });
  zq_batch_plan* p = new zq_batch_plan();
  cudaGetDevice(&p->device);
  cudaDeviceGetAttribute(&p->sms, cudaDevAttrMultiProcessorCount, p->device);
  p->count = count;
  p->ntask = (int)order.size();
  p->extent = extent;
  p->ctas_per_sm = ctas_per_sm;
  p->tuned = ctas_per_sm > 0;
  const size_t tb = batched_task_bytes();
  p->task_bytes = (tb * std::max(1, p->ntask) + 255) & ~(size_t)255;
  p->info_bytes = (sizeof(int) * (p->ntask + 1) + 255) & ~(size_t)255;
  const int max_ctas = std::max(1, std::min(p->ntask, PLAN_MAX_CPS * p->sms));
  const size_t need = p->task_bytes + p->info_bytes + sizeof(double) * (size_t)batched_ws_stride() * max_ctas;
  std::vector<char> ht(tb * std::max(1, p->ntask));
  for (int q = 0; q < p->ntask; ++q) {
    const int b = order[q];
    batched_fill_task(ht.data() + q * tb, offs[b], eoffs[b], n2s[b] / 2, ld2s[b], q);
  }
  if (cudaMalloc(&p->dev, need) != cudaSuccess ||
      cudaStreamCreateWithFlags(&p->cap, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMemcpy(p->dev, ht.data(), tb * p->ntask, cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaGetLastError();
    set_error_message("zq_batch_plan_create: device allocation or upload failed");
    if (p->dev) cudaFree(p->dev);
    if (p->cap) cudaStreamDestroy(p->cap);
    delete p;
    return nullptr;
  }
  return p;
}

int zq_batch_plan_variant(zq_batch_plan* p, int* warp_max_n, double* ms) {
  if (!p) return ZQ_ERR_ARG;
  if (warp_max_n) *warp_max_n = p->warp_max < 0 ? batched_warp_max() : p->warp_max;
  if (ms) for (int i = 0; i < 4; ++i) ms[i] = p->variant_ms[i];
  return ZQ_OK;
}

int zq_set_batch_warp_max(int n) {
  if (n < -1 || n > 32) { set_error_message("zq_set_batch_warp_max: -1 (default) or 0..32"); return ZQ_ERR_ARG; }
  batched_set_warp_max(n);
  return ZQ_OK;
}

int zq_batch_plan_run(zq_batch_plan* p, double* dD, double* deig, void* stream) {
  if (!p || !dD || !deig) { set_error_message("zq_batch_plan_run: null argument"); return ZQ_ERR_ARG; }
  if (p->ntask == 0) return ZQ_OK;
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  double2* D = reinterpret_cast<double2*>(dD);
  if (!p->tuned) {
    if (int rc = plan_tune(p, D, deig, st)) return rc;
  }
  if (!p->exec || p->gD != D || p->gE != deig) {
    // capturing records the launches without running them; the replay below is ordered on `stream`
    if (int rc = plan_capture(p, D, deig)) return rc;
  }
  ZQ_CUDA(cudaGraphLaunch(p->exec, st));
  count_launch();
  return ZQ_OK;
}

int zq_batch_plan_info(zq_batch_plan* p, void* stream) {
  if (!p) return ZQ_ERR_ARG;
  if (p->ntask == 0) return ZQ_OK;
  std::vector<int> h(p->ntask);
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  ZQ_CUDA(cudaMemcpyAsync(h.data(), plan_info(p), sizeof(int) * p->ntask, cudaMemcpyDeviceToHost, st));
  ZQ_CUDA(cudaStreamSynchronize(st));
  int m = 0;
  for (int v : h) m = v > m ? v : m;
  return m;
}

int zq_batch_plan_shape(zq_batch_plan* p, int* ctas_per_sm, int* ctas, double* tune_ms) {
  if (!p) return ZQ_ERR_ARG;
  if (ctas_per_sm) *ctas_per_sm = p->ctas_per_sm;
  if (ctas) *ctas = p->gctas;
  if (tune_ms) for (int i = 0; i < PLAN_MAX_CPS; ++i) tune_ms[i] = p->tune_ms[i];
  return ZQ_OK;
}

int zq_batch_plan_destroy(zq_batch_plan* p) {
  if (!p) return ZQ_OK;
  if (p->cap) cudaStreamSynchronize(p->cap);
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  if (p->dev) { cudaDeviceSynchronize(); cudaFree(p->dev); }
  if (p->cap) cudaStreamDestroy(p->cap);
  delete p;
  return ZQ_OK;
}

}  // extern "C"
