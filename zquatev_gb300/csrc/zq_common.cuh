// Shared device/host helpers for the GB300 quaternion eigensolver.
//
// Storage convention used by every kernel: a quaternion-Hermitian matrix
// H = (A -B*; B A*) is held as its left half [A; B] -- a 2n x n complex,
// column-major array with leading dimension ld (A at rows 0..n-1, B at rows
// n..2n-1), exactly the part of the caller's array the reference reads
// (zquatev.cc:47-54). A quaternion vector u is the pair (ua, ub) of complex
// n-vectors; its partner column J*conj(u) = (-conj(ub), conj(ua)) is implied.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>

namespace zq {

// ----------------------------------------------------------------------------
// complex helpers (double2 / float2)
// ----------------------------------------------------------------------------
template <typename R> struct cplx_of;
template <> struct cplx_of<double> { using type = double2; };
template <> struct cplx_of<float> { using type = float2; };
template <typename R> using cplx = typename cplx_of<R>::type;

__host__ __device__ __forceinline__ double2 mk(double x, double y) { return make_double2(x, y); }
__host__ __device__ __forceinline__ float2 mk(float x, float y) { return make_float2(x, y); }

template <typename Z> __host__ __device__ __forceinline__ Z cadd(Z a, Z b) { return mk(a.x + b.x, a.y + b.y); }
template <typename Z> __host__ __device__ __forceinline__ Z csub(Z a, Z b) { return mk(a.x - b.x, a.y - b.y); }
template <typename Z> __host__ __device__ __forceinline__ Z cneg(Z a) { return mk(-a.x, -a.y); }
template <typename Z> __host__ __device__ __forceinline__ Z cconj(Z a) { return mk(a.x, -a.y); }
template <typename Z> __host__ __device__ __forceinline__ Z cmul(Z a, Z b) {
  return mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// conj(a) * b
template <typename Z> __host__ __device__ __forceinline__ Z cmulc(Z a, Z b) {
  return mk(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
template <typename Z, typename R> __host__ __device__ __forceinline__ Z cscale(Z a, R s) { return mk(a.x * s, a.y * s); }
template <typename Z> __host__ __device__ __forceinline__ auto cabs2(Z a) -> decltype(a.x) { return a.x * a.x + a.y * a.y; }
// acc += a * b
template <typename Z> __host__ __device__ __forceinline__ void cfma(Z& acc, Z a, Z b) {
  acc.x = fma(a.x, b.x, acc.x); acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y); acc.y = fma(a.y, b.x, acc.y);
}
// acc += conj(a) * b
template <typename Z> __host__ __device__ __forceinline__ void cfmac(Z& acc, Z a, Z b) {
  acc.x = fma(a.x, b.x, acc.x); acc.x = fma(a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y); acc.y = fma(-a.y, b.x, acc.y);
}
// acc += a * conj(b)
template <typename Z> __host__ __device__ __forceinline__ void cfmacb(Z& acc, Z a, Z b) {
  acc.x = fma(a.x, b.x, acc.x); acc.x = fma(a.y, b.y, acc.x);
  acc.y = fma(a.y, b.x, acc.y); acc.y = fma(-a.x, b.y, acc.y);
}

template <typename Z> __host__ __device__ __forceinline__ Z czero() { Z z; z.x = 0; z.y = 0; return z; }

// (I, J), I >= J, of lower-triangle tile t in row order (t = I (I + 1) / 2 + J).
// FP32 square root for the estimate, exact integer correction (GB300's FP64
// pipe is 1/64 of its FP32 rate, so no double arithmetic per thread here).
__device__ __forceinline__ void tri_tile(int t, int& I, int& J) {
  int i = (int)((__fsqrt_rn(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
  if (i < 0) i = 0;
  while ((long long)(i + 1) * (i + 2) / 2 <= t) ++i;
  while ((long long)i * (i + 1) / 2 > t) --i;
  I = i;
  J = t - (int)((long long)i * (i + 1) / 2);
}

// Programmatic dependent launch: a kernel launched with launch_pdl may begin
// while the previous kernel on the stream drains; it must execute pdl_wait()
// (griddepcontrol.wait: returns once the preceding grid has completed and its
// memory is visible) before touching anything that grid produced.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// ----------------------------------------------------------------------------
// block reductions
// ----------------------------------------------------------------------------
template <typename T> __device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
template <typename T> __device__ __forceinline__ T warp_max(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
// |v| as the bits of a non-negative double, and max(|Re x|, |Im x|) likewise:
// for non-negative doubles the unsigned order of the bit patterns is the order
// of the values, so running maxima can use integer instructions (GB300's FP64
// pipe is narrow); __longlong_as_double turns the result back into |v|
__device__ __forceinline__ unsigned long long abs_bits(double v) {
  return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
}
__device__ __forceinline__ unsigned long long absmax_bits(double2 x) {
  const unsigned long long a = abs_bits(x.x), b = abs_bits(x.y);
  return a > b ? a : b;
}
__device__ __forceinline__ double bits_to_double(unsigned long long b) { return __longlong_as_double((long long)b); }
// Sum over the block; every thread gets the result. `sh` needs blockDim/32 slots.
template <typename T> __device__ T block_sum(T v, T* sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  T r = 0;
  for (int i = 0; i < nw; ++i) r += sh[i];
  return r;
}
template <typename T> __device__ T block_max(T v, T* sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  v = warp_max(v);
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  T r = sh[0];
  for (int i = 1; i < nw; ++i) r = fmax(r, sh[i]);
  return r;
}

// ----------------------------------------------------------------------------
// error handling (host)
// ----------------------------------------------------------------------------
// Status codes returned through the C ABI. Positive values are the
// tridiagonal solver's non-convergence count, as LAPACK's info (zquatev.cc:99).
enum Status : int {
  ZQ_OK = 0,
  ZQ_ERR_N2 = -1,       // n2 negative or odd (the reference asserts n2 % 2 == 0, zquatev.cc:43)
  ZQ_ERR_D = -2,        // null D with n2 > 0
  ZQ_ERR_LD = -3,       // ld2 < max(1, n2)
  ZQ_ERR_EIG = -4,      // null eig with n2 > 0
  ZQ_ERR_ARG = -5,      // other invalid argument
  ZQ_ERR_CUDA = -100,   // a CUDA runtime call failed
  ZQ_ERR_NOMEM = -101,  // device allocation failed
  ZQ_ERR_NOTFINITE = -102,  // input contains Inf/NaN
  ZQ_ERR_LIMIT = -103,  // size above a fixed limit of the called entry point
  ZQ_ERR_TIMEOUT = -104,  // a device-side wait ran out of time (the kernel stopped and reported it)
};

#define ZQ_CUDA(call)                                                        \
  do {                                                                       \
    cudaError_t _e = (call);                                                 \
    if (_e != cudaSuccess) {                                                 \
      zq::set_last_error(_e, #call, __FILE__, __LINE__);                     \
      return (_e == cudaErrorMemoryAllocation) ? zq::ZQ_ERR_NOMEM : zq::ZQ_ERR_CUDA; \
    }                                                                        \
  } while (0)

// Every kernel launch of the library is followed by this check, which also
// counts the launch (zq_launch_count).
#define ZQ_LAUNCH_CHECK()     \
  do {                        \
    zq::count_launch();       \
    ZQ_CUDA(cudaGetLastError()); \
  } while (0)

void count_launch(int k = 1);

template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

// the same with dynamic shared memory
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl_smem(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                                   Args... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

void set_last_error(cudaError_t e, const char* what, const char* file, int line);
void set_error_message(const char* msg);
const char* last_error_message();

// Optional per-kernel-class timing with CUDA events recorded on the launching
// stream (off unless enabled through zq_profile_enable). Each begin/end pair
// brackets one launch; totals are read back after a synchronisation.
enum ProfClass : int {
  PC_HEMV = 0, PC_TRAIL = 1, PC_PANEL = 2, PC_FORMQ_GEMM = 3, PC_APPLYZ = 4,
  PC_STEDC = 5, PC_TRIDIAG = 6, PC_FORMQ = 7, PC_BATCHED = 8, PC_OZAKI = 9, PC_REFINE = 10, PC_COUNT = 11
};
void prof_begin(int cls, cudaStream_t st);
void prof_end(int cls, cudaStream_t st);
void prof_add_flops(int cls, double flops);

__host__ __device__ inline int ceil_div(int a, int b) { return (a + b - 1) / b; }
__host__ __device__ inline int64_t ceil_div64(int64_t a, int64_t b) { return (a + b - 1) / b; }

}  // namespace zq
