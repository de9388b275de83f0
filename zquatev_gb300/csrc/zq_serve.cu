// Request server: a stream of mixed-size solves on one GPU with admission by
// HBM footprint and continuous batching.
//
// A request is one ts::zquatev call (zquatev.h:54) on host arrays. Its
// footprint is its device matrix (n2 x n2 complex, the reference's in-place
// D) plus eigenvalues plus the workspace its solve needs. Requests are
// admitted in arrival order while the admitted footprints fit the budget; an
// admitted request's matrix is copied into HBM right away (copy stream) and
// stays there until its result is copied back.
//
// Admitted requests run as soon as an execution slot is free:
//  * n2 <= batch_max_n2 (at most 512): batch workers take every such request that is ready
//    when they become free and solve them in one launch of the persistent
//    batched kernel (largest first), so the batch size follows the load;
//  * larger ones: lane workers (one host thread, stream pair and context each)
//    run the drop-in's policy path (refined, FP64 fallback) on workspace taken
//    from the stream-ordered pool for that request.
// Lanes and batches overlap on the device. Each worker is a host thread, since
// the refined path reads its convergence figure back between steps.
#include "zq_common.cuh"
#include "zq_context.h"
#include "zq_kernels.h"
#include "../../include/zquatev_gb300.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <deque>
#include <limits>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

namespace zq {
namespace {

using Clock = std::chrono::steady_clock;

struct Req {
  long long id = 0;
  int n2 = 0, ld2 = 0, n = 0;
  double2* hD = nullptr;
  double* heig = nullptr;
  bool small = false;
  size_t mat_bytes = 0;               // device matrix (ld n2) + eigenvalues
  size_t ws_fp64 = 0, ws_ref = 0;     // lane workspace
  size_t footprint = 0;
  double2* dD = nullptr;
  double* deig = nullptr;
  cudaEvent_t ready = nullptr;        // H2D copy done
  int info = 0;
  int path = -1;                      // 0 FP64, 1 refined, 2 batched, 3 refined then FP64 fallback
  bool done = false;
  double t_submit = 0, t_admit = 0, t_start = 0, t_done = 0;  // ms since the server was created
};

}  // namespace

}  // namespace zq

struct zq_server {
  int device = 0;
  int sms = 0;
  std::chrono::steady_clock::time_point t0;
  size_t budget = 0;
  int max_batch = 0;
  int batch_max_n = 0;                // requests with n <= this go to the batched kernel
  std::mutex mu;
  std::condition_variable cv_admit, cv_lane, cv_batch, cv_done;
  std::deque<zq::Req*> pending, ready_lane, ready_small;
  std::unordered_map<long long, zq::Req*> reqs;
  long long next_id = 0;
  bool stop = false;
  cudaStream_t copy_st = nullptr;
  std::vector<zq::Context*> lanes, batchers;
  std::vector<std::thread> threads;
  // accounting
  size_t reserved = 0, peak_reserved = 0;
  double occ_integral = 0.0, occ_since = -1.0, occ_last = 0.0;
  long long submitted = 0, completed = 0, batches = 0, batched_solves = 0, lane_solves = 0;
  long long refined_solves = 0, fp64_solves = 0, fallbacks = 0;

  double now() const { return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count(); }
  // reserved-bytes integral over time (caller holds mu)
  void occupancy_tick() {
    const double t = now();
    if (occ_since < 0.0) occ_since = t;
    occ_integral += (double)reserved * (t - occ_last);
    occ_last = t;
  }
};

namespace zq {
using Server = ::zq_server;

namespace {

void finish(Server* s, Req* r, int rc, int path) {
  std::lock_guard<std::mutex> lk(s->mu);
  r->info = rc;
  r->path = path;
  r->t_done = s->now();
  r->done = true;
  s->occupancy_tick();
  s->reserved -= r->footprint;
  ++s->completed;
  if (path == 2) ++s->batched_solves;
  else {
    ++s->lane_solves;
    if (path == 1) ++s->refined_solves;
    if (path == 0) ++s->fp64_solves;
    if (path == 3) ++s->fallbacks;
  }
  s->cv_done.notify_all();
  s->cv_admit.notify_one();
}

// Admission in arrival order: the head request waits until its footprint fits.
void admission_loop(Server* s) {
  cudaSetDevice(s->device);
  for (;;) {
    Req* r = nullptr;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_admit.wait(lk, [&] {
        return s->stop || (!s->pending.empty() && s->reserved + s->pending.front()->footprint <= s->budget);
      });
      if (s->stop) return;
      r = s->pending.front();
      s->pending.pop_front();
      s->occupancy_tick();
      s->reserved += r->footprint;
      s->peak_reserved = std::max(s->peak_reserved, s->reserved);
      r->t_admit = s->now();
    }
    int rc = ZQ_OK;
    void* mem = nullptr;
    if (cudaMallocAsync(&mem, r->mat_bytes, s->copy_st) != cudaSuccess) {
      cudaGetLastError();
      set_error_message("server: device matrix allocation failed");
      rc = ZQ_ERR_NOMEM;
    } else {
      r->dD = reinterpret_cast<double2*>(mem);
      r->deig = reinterpret_cast<double*>(reinterpret_cast<char*>(mem) + sizeof(double2) * (size_t)r->n2 * r->n2);
      // only the left half [A; B] is read (zquatev.cc:47-54)
      if (cudaMemcpy2DAsync(r->dD, sizeof(double2) * r->n2, r->hD, sizeof(double2) * (size_t)r->ld2,
                            sizeof(double2) * r->n2, r->n, cudaMemcpyHostToDevice, s->copy_st) != cudaSuccess ||
          cudaEventRecord(r->ready, s->copy_st) != cudaSuccess) {
        cudaGetLastError();
        rc = ZQ_ERR_CUDA;
      }
    }
    if (rc != ZQ_OK) {
      if (mem) { cudaFreeAsync(mem, s->copy_st); cudaStreamSynchronize(s->copy_st); }
      r->dD = nullptr;
      finish(s, r, rc, -1);
      continue;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    if (r->small) { s->ready_small.push_back(r); s->cv_batch.notify_one(); }
    else { s->ready_lane.push_back(r); s->cv_lane.notify_one(); }
  }
}

int copy_back(Req* r, cudaStream_t st) {
  ZQ_CUDA(cudaMemcpy2DAsync(r->hD, sizeof(double2) * (size_t)r->ld2, r->dD, sizeof(double2) * r->n2,
                            sizeof(double2) * r->n2, r->n2, cudaMemcpyDeviceToHost, st));
  ZQ_CUDA(cudaMemcpyAsync(r->heig, r->deig, sizeof(double) * r->n, cudaMemcpyDeviceToHost, st));
  return ZQ_OK;
}

void lane_loop(Server* s, Context* c) {
  cudaSetDevice(s->device);
  for (;;) {
    Req* r = nullptr;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_lane.wait(lk, [&] { return s->stop || !s->ready_lane.empty(); });
      if (s->stop) return;
      r = s->ready_lane.front();
      s->ready_lane.pop_front();
      r->t_start = s->now();
    }
    const int p = path_for(r->n);
    int used = p;
    int rc = ZQ_OK;
    void* ws = nullptr;
    const size_t wsb = r->ws_fp64 + (p == 1 ? r->ws_ref : 0);
    if (cudaMallocAsync(&ws, wsb, c->st) != cudaSuccess) {
      cudaGetLastError();
      set_error_message("server: workspace allocation failed");
      rc = ZQ_ERR_NOMEM;
      ws = nullptr;
    }
    if (rc == ZQ_OK) {
      char* w = reinterpret_cast<char*>(ws);
      context_bind(c, w, r->ws_fp64, p == 1 ? w + r->ws_fp64 : nullptr, p == 1 ? r->ws_ref : 0);
      if (cudaStreamWaitEvent(c->st, r->ready, 0) != cudaSuccess) rc = ZQ_ERR_CUDA;
      if (rc == ZQ_OK)
        rc = (p == 1) ? refined_device(c, r->dD, r->n2, r->n, r->deig, c->st, 1)
                      : solve_device(c, r->dD, r->n2, r->n, r->deig, true, c->st);
      if (rc == ZQ_OK && p == 1 && c->rb.last_fallback) used = 3;
      if (rc == ZQ_OK) rc = copy_back(r, c->st);
      cudaFreeAsync(ws, c->st);
    }
    cudaFreeAsync(r->dD, c->st);
    const cudaError_t e = cudaStreamSynchronize(c->st);
    context_bind(c, nullptr, 0, nullptr, 0);
    if (rc == ZQ_OK && e != cudaSuccess) { set_last_error(e, "server lane", __FILE__, __LINE__); rc = ZQ_ERR_CUDA; }
    finish(s, r, rc, used);
  }
}

void batch_loop(Server* s, Context* c) {
  cudaSetDevice(s->device);
  const size_t tb = batched_task_bytes();
  std::vector<char> htasks;
  std::vector<int> hinfo;
  for (;;) {
    std::vector<Req*> batch;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_batch.wait(lk, [&] { return s->stop || !s->ready_small.empty(); });
      if (s->stop) return;
      while (!s->ready_small.empty() && (int)batch.size() < s->max_batch) {
        batch.push_back(s->ready_small.front());
        s->ready_small.pop_front();
      }
      const double t = s->now();
      for (Req* r : batch) r->t_start = t;
      ++s->batches;
    }
    // longest first: the persistent kernel hands out tasks in this order
    std::stable_sort(batch.begin(), batch.end(), [](const Req* a, const Req* b) { return a->n > b->n; });
    const int k = (int)batch.size();
    const int ctas = std::min(k, 2 * s->sms);
    const size_t task_bytes = (tb * k + 255) & ~(size_t)255;
    const size_t info_bytes = (sizeof(int) * (k + 1) + 255) & ~(size_t)255;
    const size_t need = task_bytes + info_bytes + sizeof(double) * (size_t)batched_ws_stride() * ctas;
    htasks.resize(tb * k);
    hinfo.assign(k, 0);
    for (int q = 0; q < k; ++q) batched_fill_task_ptr(htasks.data() + q * tb, batch[q]->dD, batch[q]->deig, batch[q]->n,
                                                      batch[q]->n2, q);
    int rc = ZQ_OK;
    void* mem = nullptr;
    if (cudaMallocAsync(&mem, need, c->st) != cudaSuccess) {
      cudaGetLastError();
      rc = ZQ_ERR_NOMEM;
      mem = nullptr;
    }
    if (rc == ZQ_OK) {
      char* b = reinterpret_cast<char*>(mem);
      int* dinfo = reinterpret_cast<int*>(b + task_bytes);
      for (Req* r : batch)
        if (cudaStreamWaitEvent(c->st, r->ready, 0) != cudaSuccess) rc = ZQ_ERR_CUDA;
      if (rc == ZQ_OK && cudaMemcpyAsync(b, htasks.data(), tb * k, cudaMemcpyHostToDevice, c->st) != cudaSuccess)
        rc = ZQ_ERR_CUDA;
      if (rc == ZQ_OK)
        rc = batched_launch(b, k, dinfo + k, nullptr, nullptr, reinterpret_cast<double*>(b + task_bytes + info_bytes),
                            ctas, dinfo, c->st);
      if (rc == ZQ_OK && cudaMemcpyAsync(hinfo.data(), dinfo, sizeof(int) * k, cudaMemcpyDeviceToHost, c->st) != cudaSuccess)
        rc = ZQ_ERR_CUDA;
      for (int q = 0; q < k && rc == ZQ_OK; ++q) rc = copy_back(batch[q], c->st);
      cudaFreeAsync(mem, c->st);
    }
    for (Req* r : batch) cudaFreeAsync(r->dD, c->st);
    const cudaError_t e = cudaStreamSynchronize(c->st);
    if (rc == ZQ_OK && e != cudaSuccess) { set_last_error(e, "server batch", __FILE__, __LINE__); rc = ZQ_ERR_CUDA; }
    for (int q = 0; q < k; ++q) finish(s, batch[q], rc != ZQ_OK ? rc : hinfo[q], 2);
  }
}

}  // namespace
}  // namespace zq

using namespace zq;

extern "C" {

long long zq_solve_footprint(int n2, int path) {
  if (n2 < 0 || (n2 & 1) || path < -1 || path > 2) { set_error_message("bad n2 or path"); return ZQ_ERR_ARG; }
  const int n = n2 / 2;
  if (path == -1) path = n <= batched_max_n() ? 2 : path_for(n);
  if (path == 2 && n > batched_max_n()) { set_error_message("batched kernel takes n2 <= 512"); return ZQ_ERR_LIMIT; }
  const size_t mat = sizeof(double2) * (size_t)n2 * n2 + sizeof(double) * (size_t)(n + 32);
  if (path == 2) return (long long)(mat + sizeof(double) * (size_t)batched_ws_stride() + 256);
  size_t f = 0, r = 0;
  solve_workspace_bytes(n, &f, &r);
  return (long long)(mat + f + (path == 1 ? r : 0));
}

zq_server* zq_server_create(long long hbm_budget_bytes, int lanes, int max_batch, int batch_max_n2) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) { set_error_message("no CUDA device"); return nullptr; }
  if (lanes < 1 || lanes > 64 || max_batch < 1 || batch_max_n2 < 0 || batch_max_n2 > 2 * batched_max_n()) {
    set_error_message("lanes must be 1..64, max_batch >= 1, batch_max_n2 in [0, 512]");
    return nullptr;
  }
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) { set_error_message("cudaMemGetInfo failed"); return nullptr; }
  Server* s = new Server();
  s->device = dev;
  s->t0 = Clock::now();
  s->budget = hbm_budget_bytes > 0 ? (size_t)hbm_budget_bytes : (size_t)(0.8 * (double)free_b);
  s->max_batch = max_batch;
  s->batch_max_n = batch_max_n2 / 2;
  cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, dev);
  // keep freed request memory in the stream-ordered pool between requests
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    uint64_t thr = std::numeric_limits<uint64_t>::max();
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  bool ok = cudaStreamCreateWithFlags(&s->copy_st, cudaStreamNonBlocking) == cudaSuccess;
  for (int i = 0; ok && i < lanes; ++i) {
    Context* c = nullptr;
    ok = context_create(dev, &c) == ZQ_OK;
    if (ok) c->coop = false;  // lanes solve beside each other: no cooperative launches
    if (ok) s->lanes.push_back(c);
  }
  for (int i = 0; ok && i < 2; ++i) {
    Context* c = nullptr;
    ok = context_create(dev, &c) == ZQ_OK;
    if (ok) s->batchers.push_back(c);
  }
  if (!ok) {
    for (Context* c : s->lanes) context_destroy(c);
    for (Context* c : s->batchers) context_destroy(c);
    if (s->copy_st) cudaStreamDestroy(s->copy_st);
    delete s;
    return nullptr;
  }
  s->threads.emplace_back(admission_loop, s);
  for (Context* c : s->lanes) s->threads.emplace_back(lane_loop, s, c);
  for (Context* c : s->batchers) s->threads.emplace_back(batch_loop, s, c);
  return s;
}

long long zq_server_submit(zq_server* s, int n2, double* D, int ld2, double* eig) {
  if (!s) { set_error_message("null server"); return ZQ_ERR_ARG; }
  if (n2 < 0 || (n2 & 1)) { set_error_message("n2 must be even and non-negative"); return ZQ_ERR_N2; }
  if (n2 > 0 && !D) { set_error_message("D is null"); return ZQ_ERR_D; }
  if (n2 > 0 && ld2 < n2) { set_error_message("ld2 < n2"); return ZQ_ERR_LD; }
  if (n2 > 0 && !eig) { set_error_message("eig is null"); return ZQ_ERR_EIG; }
  Req* r = new Req();
  r->n2 = n2; r->ld2 = ld2; r->n = n2 / 2;
  r->hD = reinterpret_cast<double2*>(D);
  r->heig = eig;
  r->small = r->n <= s->batch_max_n;
  r->mat_bytes = sizeof(double2) * (size_t)n2 * n2 + sizeof(double) * (size_t)(r->n + 32);
  if (r->small) {
    r->footprint = (size_t)zq_solve_footprint(n2, 2);
  } else {
    solve_workspace_bytes(r->n, &r->ws_fp64, &r->ws_ref);
    r->footprint = r->mat_bytes + r->ws_fp64 + (path_for(r->n) == 1 ? r->ws_ref : 0);
  }
  std::lock_guard<std::mutex> lk(s->mu);
  if (r->footprint > s->budget) {
    delete r;
    set_error_message("request footprint exceeds the server's HBM budget");
    return ZQ_ERR_LIMIT;
  }
  r->id = s->next_id++;
  r->t_submit = s->now();
  ++s->submitted;
  s->reqs[r->id] = r;
  if (n2 == 0) {
    r->done = true;
    r->t_admit = r->t_start = r->t_done = r->t_submit;
    ++s->completed;
    return r->id;
  }
  if (cudaEventCreateWithFlags(&r->ready, cudaEventDisableTiming) != cudaSuccess) {
    s->reqs.erase(r->id);
    delete r;
    set_error_message("cudaEventCreate failed");
    return ZQ_ERR_CUDA;
  }
  s->pending.push_back(r);
  s->cv_admit.notify_one();
  return r->id;
}

int zq_server_test(zq_server* s, long long id) {
  if (!s) return ZQ_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) { set_error_message("unknown request id"); return ZQ_ERR_ARG; }
  return it->second->done ? 1 : 0;
}

int zq_server_wait(zq_server* s, long long id, double* times_ms, int* path) {
  if (!s) return ZQ_ERR_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) { set_error_message("unknown request id"); return ZQ_ERR_ARG; }
  Req* r = it->second;
  s->cv_done.wait(lk, [&] { return r->done; });
  if (times_ms) { times_ms[0] = r->t_submit; times_ms[1] = r->t_admit; times_ms[2] = r->t_start; times_ms[3] = r->t_done; }
  if (path) *path = r->path;
  const int info = r->info;
  s->reqs.erase(it);
  lk.unlock();
  if (r->ready) cudaEventDestroy(r->ready);
  delete r;
  return info;
}

int zq_server_stats_read(zq_server* s, zq_server_stats* out) {
  if (!s || !out) return ZQ_ERR_ARG;
  size_t free_b = 0, total_b = 0;
  cudaMemGetInfo(&free_b, &total_b);
  std::lock_guard<std::mutex> lk(s->mu);
  s->occupancy_tick();
  out->submitted = s->submitted;
  out->completed = s->completed;
  out->batches = s->batches;
  out->batched_solves = s->batched_solves;
  out->lane_solves = s->lane_solves;
  out->refined_solves = s->refined_solves;
  out->fp64_solves = s->fp64_solves;
  out->fallbacks = s->fallbacks;
  out->queued = (long long)s->pending.size();
  out->in_flight = s->submitted - s->completed - (long long)s->pending.size();
  out->lanes = (int)s->lanes.size();
  out->budget_bytes = (double)s->budget;
  out->reserved_bytes = (double)s->reserved;
  out->peak_reserved_bytes = (double)s->peak_reserved;
  const double span = s->occ_last - (s->occ_since < 0.0 ? s->occ_last : s->occ_since);
  out->mean_reserved_bytes = span > 0.0 ? s->occ_integral / span : 0.0;
  out->device_used_bytes = (double)(total_b - free_b);
  return ZQ_OK;
}

int zq_server_destroy(zq_server* s) {
  if (!s) return ZQ_OK;
  {
    std::unique_lock<std::mutex> lk(s->mu);
    s->cv_done.wait(lk, [&] { return s->completed == s->submitted; });
    s->stop = true;
    s->cv_admit.notify_all();
    s->cv_lane.notify_all();
    s->cv_batch.notify_all();
  }
  for (std::thread& t : s->threads) t.join();
  for (Context* c : s->lanes) context_destroy(c);
  for (Context* c : s->batchers) context_destroy(c);
  cudaStreamDestroy(s->copy_st);
  for (auto& kv : s->reqs) {
    if (kv.second->ready) cudaEventDestroy(kv.second->ready);
    delete kv.second;
  }
  delete s;
  return ZQ_OK;
}

}  // extern "C"
