"""Benchmark: quaternion-Hermitian eigensolve on GB300 (one JSON line on rank 0).

Workload (default): one n2 = 8192 (n = 4096) random quaternion-Hermitian
matrix, complex128, A = (X + X^H)/2, B = (Y - Y^T)/2, Re/Im ~ N(0,1), full
eigenvectors. A step is one full solve of that matrix through the drop-in's
default path: an FP32 decomposition refined to FP64 accuracy (Ogita-Aishima,
products on the bf16 tensor cores by Ozaki slicing), with the plain FP64 path
as fallback. The plain FP64 GPU path is timed on the same input beside it
(fp64_path_ms). Inputs (512 MiB left half) are larger than L2, so no extra L2
flush is needed between steps.

  value   device-resident: the input is restored from an HBM master copy
          (device-to-device) and solved through the device C ABI; ms per solve.
  e2e     the reference-facing host call (zquatev_c on pinned host arrays): H2D
          of the left half, solve, D2H of all of D and eig, per solve.
  roofline  the dominant kernel (the Ozaki tensor-core product), timed with
          CUDA events on its launch stream during the timed region, executed
          bf16 flops against MEASURED_PEAKS.json's sustained bf16 figure; the
          FP64 path's kernels are reported against the FP64 DFMA peak measured
          here by a calibration kernel (DMMA issues slower than DFMA).
  cpu_baseline  the reference's CPU code on a bounded n2=1024 sample, scaled by
          n^3 to n2 = 8192: the compiled reference (oracle/_ref) where it loads,
          else the oracle port (numpy/scipy restatement of the reference, the only
          CPU implementation that exists on the GPU host).

--impl reference runs the CPU reference arm (the same choice, all host threads).
Under torchrun (N > 1) every rank solves its own matrix (replicas, no
collectives on the data path); rank 0 prints.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "n2=8192 solve ms; mixed-stream solves/s, p99 ms vs plain FP64 at resid≤1e-12"
# DRAM bytes (read + write) per executed bf16 flop of the Ozaki product kernel,
# from one ncu capture of k_oz_umma<2> (n2 = 4096, second step's P1, 8 slices:
# 6.264 + 1.048 GB / 4.95e12 flop)
OZ_BYTES_PER_FLOP = 7.312e9 / 4.95e12


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--n2", type=int, default=8192)
    p.add_argument("--e2e-steps", type=int, default=3)
    p.add_argument("--no-check", action="store_true")
    p.add_argument("--cpu-sample-n2", type=int, default=0,
                   help="CPU sample size (0: 2048 for the compiled reference, 1024 for the port)")
    p.add_argument("--serve-requests", type=int, default=128, help="requests per serving run (0 skips serving)")
    p.add_argument("--serve-rates", default="0.5,1,2",
                   help="Poisson arrival rates as multiples of the FP64 one-at-a-time capacity")
    p.add_argument("--serve-lanes", type=int, default=4)
    p.add_argument("--batch-count", type=int, default=4096, help="matrices in the batched run (0 skips it)")
    p.add_argument("--profile-path", default="default", choices=["default", "fp64", "batched"])
    p.add_argument("--clustered-n2", type=int, default=0,
                   help="also measure the clustered-spectrum workload (e.g. 16384): refined vs FP64, errors")
    p.add_argument("--profile-n2", type=int, default=0,
                   help="profiling case: run --reps device-resident solves of this size (--profile-path) and exit")
    p.add_argument("--reps", type=int, default=1)
    return p.parse_args()


def workload_config(n2: int, world: int) -> dict:
    """The measured workload, identical on the GPU arm and the reference arm."""
    return {"workload": f"single quaternion-Hermitian solve n2={n2} (n={n2 // 2}): random A=(X+X^H)/2, "
                        "B=(Y-Y^T)/2 (Re, Im ~ N(0,1)), complex128, all eigenvalues and eigenvectors",
            "n2": n2, "parallelism": f"replicas{world}",
            "l2": "inputs (512 MiB left half) larger than L2; restored D2D each step"}


def max_over_ranks(value: float, world: int, device) -> float:
    """The slowest rank's time (all ranks receive it); value itself for one rank."""
    if world <= 1:
        return value
    import torch

    t = torch.tensor([value], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# --------------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None

    def __enter__(self):
        # the sampler's start-up (driver and NVML initialisation) is kept out of
        # the timed region: wait (at most 5 s) for its first sample
        self.first = []
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        if self.proc is not None:
            import select
            ready, _, _ = select.select([self.proc.stdout], [], [], 5.0)
            if ready:
                self.first.append(self.proc.stdout.readline())
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out = ""
            self.lines = [l for l in self.first + out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------- FP64 peak probe
_PEAK_SRC = r"""
extern "C" __global__ void dfma_peak(double* out, int iters, double a, double b) {
  double x0=threadIdx.x, x1=x0+1, x2=x0+2, x3=x0+3, x4=x0+4, x5=x0+5, x6=x0+6, x7=x0+7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0,a,b); x1 = fma(x1,a,b); x2 = fma(x2,a,b); x3 = fma(x3,a,b);
    x4 = fma(x4,a,b); x5 = fma(x5,a,b); x6 = fma(x6,a,b); x7 = fma(x7,a,b);
  }
  out[blockIdx.x*blockDim.x+threadIdx.x] = x0+x1+x2+x3+x4+x5+x6+x7;
}
// FP64 on the tensor cores: independent m8n8k4 DMMA chains per warp (512 flops each)
extern "C" __global__ void dmma_peak(double* out, int iters) {
  const double a = 1.0 + threadIdx.x * 1e-3, b = 0.5;
  double c0 = 0, c1 = 0, c2 = 0, c3 = 0, c4 = 0, c5 = 0, c6 = 0, c7 = 0;
  for (int i = 0; i < iters; ++i) {
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};" : "+d"(c0), "+d"(c1) : "d"(a), "d"(b));
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};" : "+d"(c2), "+d"(c3) : "d"(a), "d"(b));
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};" : "+d"(c4), "+d"(c5) : "d"(a), "d"(b));
    asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};" : "+d"(c6), "+d"(c7) : "d"(a), "d"(b));
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = c0 + c1 + c2 + c3 + c4 + c5 + c6 + c7;
}
// the larger f64 shapes: four independent m16n8kK chains per warp
extern "C" __global__ void dmma_k4(double* out, int iters) {
  const double a = 1.0 + threadIdx.x * 1e-3, b = 0.5;
  double c[4][4] = {};
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int q = 0; q < 4; ++q)
      asm volatile("mma.sync.aligned.m16n8k4.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, {%4,%5}, {%6}, {%0,%1,%2,%3};"
                   : "+d"(c[q][0]), "+d"(c[q][1]), "+d"(c[q][2]), "+d"(c[q][3]) : "d"(a), "d"(a), "d"(b));
  }
  double s = 0;
  for (int q = 0; q < 4; ++q) s += c[q][0] + c[q][1] + c[q][2] + c[q][3];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
extern "C" __global__ void dmma_k8(double* out, int iters) {
  const double a = 1.0 + threadIdx.x * 1e-3, b = 0.5;
  double c[4][4] = {};
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int q = 0; q < 4; ++q)
      asm volatile("mma.sync.aligned.m16n8k8.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
                   : "+d"(c[q][0]), "+d"(c[q][1]), "+d"(c[q][2]), "+d"(c[q][3])
                   : "d"(a), "d"(a), "d"(a), "d"(a), "d"(b), "d"(b));
  }
  double s = 0;
  for (int q = 0; q < 4; ++q) s += c[q][0] + c[q][1] + c[q][2] + c[q][3];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
extern "C" __global__ void dmma_k16(double* out, int iters) {
  const double a = 1.0 + threadIdx.x * 1e-3, b = 0.5;
  double c[4][4] = {};
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int q = 0; q < 4; ++q)
      asm volatile("mma.sync.aligned.m16n8k16.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, {%4,%5,%6,%7,%8,%9,%10,%11}, "
                   "{%12,%13,%14,%15}, {%0,%1,%2,%3};"
                   : "+d"(c[q][0]), "+d"(c[q][1]), "+d"(c[q][2]), "+d"(c[q][3])
                   : "d"(a), "d"(a), "d"(a), "d"(a), "d"(a), "d"(a), "d"(a), "d"(a), "d"(b), "d"(b), "d"(b), "d"(b));
  }
  double s = 0;
  for (int q = 0; q < 4; ++q) s += c[q][0] + c[q][1] + c[q][2] + c[q][3];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
"""


def fp64_peak_tflops() -> float:
    """DFMA throughput of this GPU (TFLOP/s), timed with CUDA events."""
    import torch

    lib = _peak_module()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    blocks, threads, iters = sms * 4, 256, 4096
    out = torch.empty(blocks * threads, dtype=torch.float64, device="cuda")
    best = 0.0
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        lib.run(out, blocks, threads, iters)
        e1.record()
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        best = max(best, 2.0 * 8 * iters * blocks * threads / (ms * 1e9))
    return best


# flops of one warp-wide mma.sync of each f64 shape, and per-iteration MMAs
DMMA_SHAPES = {"m8n8k4": (512, 4), "m16n8k4": (1024, 4), "m16n8k8": (2048, 4), "m16n8k16": (4096, 4)}


def dmma_peak_tflops(shape: str = "m8n8k4") -> float:
    """FP64 tensor-core (DMMA) throughput of this GPU for one mma.sync f64
    shape (TFLOP/s), CUDA events."""
    import torch

    lib = _peak_module()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    flops, per_iter = DMMA_SHAPES[shape]
    blocks, threads, iters = sms * 4, 256, max(256, 2048 * 512 // flops)
    out = torch.empty(blocks * threads, dtype=torch.float64, device="cuda")
    best = 0.0
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        lib.run_dmma(out, blocks, threads, iters, shape)
        e1.record()
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        best = max(best, per_iter * float(flops) * iters * blocks * (threads // 32) / (ms * 1e9))
    return best


def dmma_all_shapes() -> dict:
    return {shape: round(dmma_peak_tflops(shape), 3) for shape in DMMA_SHAPES}


_PEAK_LIB = None


def _peak_module():
    """Compiles the calibration kernel with nvcc into a tiny shared library."""
    global _PEAK_LIB
    if _PEAK_LIB is not None:
        return _PEAK_LIB
    import ctypes
    import tempfile

    import torch

    d = tempfile.mkdtemp(prefix="zqpeak")
    src = os.path.join(d, "peak.cu")
    with open(src, "w") as f:
        f.write(_PEAK_SRC + r"""
extern "C" int launch_peak(double* out, int blocks, int threads, int iters, void* st) {
  dfma_peak<<<blocks, threads, 0, (cudaStream_t)st>>>(out, iters, 0.999, 1e-3);
  return (int)cudaGetLastError();
}
extern "C" int launch_dmma(double* out, int blocks, int threads, int iters, int shape, void* st) {
  cudaStream_t s = (cudaStream_t)st;
  if (shape == 0) dmma_peak<<<blocks, threads, 0, s>>>(out, iters);
  else if (shape == 1) dmma_k4<<<blocks, threads, 0, s>>>(out, iters);
  else if (shape == 2) dmma_k8<<<blocks, threads, 0, s>>>(out, iters);
  else dmma_k16<<<blocks, threads, 0, s>>>(out, iters);
  return (int)cudaGetLastError();
}
""")
    so = os.path.join(d, "peak.so")
    subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-shared", "-Xcompiler", "-fPIC",
                    "-cudart", "shared", src, "-o", so], check=True, capture_output=True)
    lib = ctypes.CDLL(so)
    lib.launch_peak.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    lib.launch_dmma.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                ctypes.c_void_p]

    class _M:
        @staticmethod
        def run(out, blocks, threads, iters):
            lib.launch_peak(out.data_ptr(), blocks, threads, iters, torch.cuda.current_stream().cuda_stream)

        @staticmethod
        def run_dmma(out, blocks, threads, iters, shape="m8n8k4"):
            lib.launch_dmma(out.data_ptr(), blocks, threads, iters, list(DMMA_SHAPES).index(shape),
                            torch.cuda.current_stream().cuda_stream)

    _PEAK_LIB = _M
    return _M


# ------------------------------------------------------------------ CPU legs
def cpu_kind() -> str:
    """"reference" where the unmodified reference compiled from its sources
    (oracle/_ref) loads on this host, else "port" (the numpy/scipy restatement;
    the GPU host has no reference sources)."""
    try:
        from oracle import ref

        if ref.available():
            ref._load()
            return "reference"
    except OSError:
        pass
    return "port"


def cpu_sample_n2(requested: int) -> int:
    """The CPU sample: n^3 scaling from n2 = 2048 is within 5% of the compiled
    reference's directly measured n2 = 8192 time (from 1024 it overstates it
    1.7x); the port grows faster than n^3, so its 1024 sample understates it."""
    if requested > 0:
        return requested
    return 2048 if cpu_kind() == "reference" else 1024


def cpu_sample(n2_sample: int, n2_target: int, threads: int):
    """Times the reference's CPU code on one n2_sample solve — the compiled
    reference where it loads, else the oracle port — and scales by n^3 to
    n2_target."""
    os.environ.setdefault("OPENBLAS_NUM_THREADS", str(threads))
    from oracle import port, ref
    from zquatev_gb300 import inputs

    n = n2_sample // 2
    d = inputs.random_matrix(n, 4321)
    eig = np.zeros(2 * n)
    impl = ref if cpu_kind() == "reference" else port
    if impl is ref:
        d = np.asfortranarray(d)
    t0 = time.perf_counter()
    rc = impl.zquatev(2 * n, d, 2 * n, eig)
    dt = time.perf_counter() - t0
    assert rc == 0
    scale = (n2_target / n2_sample) ** 3
    return dt * 1e3 * scale, dt


# The compiled reference timed directly at the headline size, once, on the
# 8-core x86 development host (OpenBLAS 0.3.31, 8 threads): it cannot be built
# on the GPU host (its sources stay out of this repository), so the bench's
# reference arm extrapolates from a bounded sample and carries this figure
# beside it, labelled.
REFERENCE_MEASURED_N2_8192 = {"n2": 8192, "seconds": 412.0, "impl": "compiled reference (oracle/_ref)",
                              "host": "8-core x86 development host, OpenBLAS 0.3.31, 8 threads",
                              "measured_on_gpu_host": False}


def cpu_baseline_fields(value_ms: float, n2_target: int, n2_sample: int, raw_s: float, threads: int) -> dict:
    """The cpu_baseline object: what was timed, and how it was scaled."""
    kind = cpu_kind()
    scale = (n2_target / n2_sample) ** 3
    return {"value": value_ms, "unit": "ms", "cores": threads, "kind": kind,
            "sample": f"one n2={n2_sample} solve per step through "
                      + ("oracle/_ref (the compiled reference, OpenBLAS)" if kind == "reference"
                         else "oracle/port.py (numpy + scipy OpenBLAS/LAPACK restatement of the reference)")
                      + f" = {raw_s:.2f} s, scaled x{scale:.0f} (n^3) to n2={n2_target}",
            "extrapolated": n2_sample != n2_target, "sample_n2": n2_sample, "sample_s": round(raw_s, 3),
            "scale_n3": scale, "fits_in_driver_run": n2_sample == n2_target,
            "reference_measured_directly": REFERENCE_MEASURED_N2_8192}


def run_reference(args, rank, world):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    os.environ["OPENBLAS_NUM_THREADS"] = str(threads)
    vals, raws = [], []
    for i in range(args.warmup + args.steps):
        ms, raw = cpu_sample(args.cpu_sample_n2, args.n2, threads)
        if i >= args.warmup:
            vals.append(ms)
            raws.append(raw)
    v = float(np.mean(vals))
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "ms", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": v, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
        "config": workload_config(args.n2, world),
        "cpu_baseline": cpu_baseline_fields(v, args.n2, args.cpu_sample_n2, float(np.mean(raws)), threads),
        "e2e": {"value": v, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------ profiling case
def profile_case(n2: int, reps: int, path: str):
    """Small fixed workload for ncu captures: `reps` device-resident solves of
    one random n2 matrix (default path or plain FP64), or one batched launch of
    `reps` x 64 matrices with n2 = n2 (--profile-path batched)."""
    import torch

    from zquatev_gb300 import _lib, build, inputs

    if not build.up_to_date():
        build.build()
    lib = _lib.load()
    n = n2 // 2
    st = torch.cuda.current_stream().cuda_stream
    if path == "batched":
        count = 64 * reps
        d = inputs.random_matrix(n, 11)
        one = torch.from_numpy(np.ascontiguousarray(d.T).reshape(-1))
        buf = one.repeat(count).cuda()
        deig = torch.zeros(count * n, dtype=torch.float64, device="cuda")
        n2s = np.full(count, n2, np.int32)
        offs = (np.arange(count, dtype=np.int64) * n2 * n2)
        eoffs = (np.arange(count, dtype=np.int64) * n)
        rc = lib.zquatev_batched_device(count, n2s.ctypes.data, n2s.ctypes.data, offs.ctypes.data, eoffs.ctypes.data,
                                        buf.data_ptr(), deig.data_ptr(), st)
        torch.cuda.synchronize()
        print(json.dumps({"profile_case": "batched", "n2": n2, "count": count, "rc": rc}))
        return
    d = inputs.random_matrix(n, 11)
    master = torch.from_numpy(np.ascontiguousarray(d.T)).cuda()
    work = torch.empty_like(master)
    deig = torch.zeros(n2, dtype=torch.float64, device="cuda")
    fn = lib.zquatev_device if path == "default" else lib.zquatev_fp64_device
    for _ in range(reps):
        work.copy_(master)
        rc = fn(n2, work.data_ptr(), n2, deig.data_ptr(), st)
        if rc != 0:
            raise RuntimeError(f"rc={rc}: {_lib.last_error()}")
    torch.cuda.synchronize()
    print(json.dumps({"profile_case": path, "n2": n2, "reps": reps}))


# ---------------------------------------------------------- batched solves
def batched_case(count: int, fp64_peak: float, seed: int = 2024) -> dict:
    """4096 independent matrices, n log-uniform in [8, 256], solved by one call
    of the batched entry point (persistent kernel); against the plain FP64
    drop-in looped over a 1-in-16 sample of the same matrices (scaled)."""
    import torch

    from zquatev_gb300 import _lib, inputs

    lib = _lib.load()
    st = torch.cuda.current_stream().cuda_stream
    ns = inputs.log_uniform_sizes(count, 8, 256, seed).astype(np.int64)
    n2s = (2 * ns).astype(np.int32)
    sizes = (2 * ns) ** 2
    offs = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
    eoffs = np.concatenate([[0], np.cumsum(ns)[:-1]]).astype(np.int64)
    host = np.empty(int(sizes.sum()), np.complex128)
    for i, n in enumerate(ns):
        host[offs[i]:offs[i] + sizes[i]] = inputs.random_matrix(int(n), seed * 7 + i).ravel(order="F")
    master = torch.from_numpy(host).cuda()
    work = torch.empty_like(master)
    deig = torch.zeros(int(ns.sum()), dtype=torch.float64, device="cuda")

    from zquatev_gb300 import solver

    plan = solver.BatchPlan(n2s, n2s, offs, eoffs)  # launch shape tuned on the first run, then graph replays
    times = []
    launches = 0
    for i in range(4):
        work.copy_(master)
        torch.cuda.synchronize()
        lc0 = lib.zq_launch_count()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        plan.run(work, deig)
        e1.record()
        torch.cuda.synchronize()
        assert plan.info() == 0
        if i >= 1:
            times.append(e0.elapsed_time(e1))
            launches = lib.zq_launch_count() - lc0
    shape = plan.shape()
    plan.close()
    ms = float(np.median(times))
    # accuracy on a few of the results (GPU residual)
    from zquatev_gb300 import metrics

    worst = 0.0
    for i in list(range(0, count, max(1, count // 16)))[:16]:
        n = int(ns[i])
        d = host[offs[i]:offs[i] + sizes[i]].reshape(2 * n, 2 * n, order="F")
        h = torch.from_numpy(inputs.full_from_blocks(d[:n, :n], d[n:, :n])).cuda()
        v = work[offs[i]:offs[i] + sizes[i]].view(2 * n, 2 * n).T
        worst = max(worst, metrics.torch_residual(h, v, deig[eoffs[i]:eoffs[i] + n]))
    # plain FP64 drop-in, one matrix after the other, on every 16th matrix
    work.copy_(master)
    sample = list(range(0, count, 16))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in sample:
        rc = lib.zquatev_fp64_device(int(n2s[i]), work.data_ptr() + 16 * int(offs[i]), int(n2s[i]),
                                     deig.data_ptr() + 8 * int(eoffs[i]), st)
        assert rc == 0
    torch.cuda.synchronize()
    loop_s = (time.perf_counter() - t0) * count / len(sample)
    flops = float(((64.0 / 3.0 + 16.0) * ns.astype(np.float64) ** 3).sum())
    del master, work
    return {"workload": f"{count} matrices, n log-uniform in [8, 256] (n2 16..512), random as config 0, per-matrix seeds",
            "ms": ms, "solves_per_s": count / (ms * 1e-3), "gpu_launches": int(launches),
            "launch": "one CUDA-graph replay of the persistent kernel (zq_batch_plan)",
            "tuned_shape": shape,
            "fp64_loop_solves_per_s": count / loop_s, "speedup_vs_fp64_loop": loop_s / (ms * 1e-3),
            "fp64_loop_sample": f"{len(sample)} matrices (every 16th), scaled x{count / len(sample):.0f}",
            "algorithmic_tflops": flops / (ms * 1e-3) / 1e12,
            "fp64_frac": flops / (ms * 1e-3) / 1e12 / fp64_peak if fp64_peak else None,
            "max_residual_sampled": worst}


# ------------------------------------------------------- clustered spectrum
def clustered_case(n2: int) -> dict:
    """One matrix H = Q diag(lam) Q^H (Q quaternion-unitary; 80% of lam uniform in
    [-10, 10], 20% in clusters of 8 with gaps 1e-6), solved by the default
    (refined) path and by the plain FP64 path; per-eigenvalue error against the
    constructed spectrum, residual and orthonormality of both (GPU torch FP64 as
    the checker)."""
    import torch

    from zquatev_gb300 import _lib, inputs, metrics, solver

    lib = _lib.load()
    n = n2 // 2
    t0 = time.perf_counter()
    master, lam = inputs.clustered_matrix_device(n, 2023)
    torch.cuda.synchronize()
    gen_s = time.perf_counter() - t0
    lam_sorted = torch.from_numpy(np.sort(lam)).cuda()
    st = torch.cuda.current_stream().cuda_stream
    out = {"workload": f"n2={n2} clustered: H = Q diag(lam) Q^H, 20% of lam in clusters of 8 (gap 1e-6)",
           "generation_s": gen_s}
    for name, fn in (("refined", lib.zquatev_device), ("fp64", lib.zquatev_fp64_device)):
        work = master.clone()
        deig = torch.zeros(n2, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        rc = fn(n2, work.data_ptr(), n2, deig.data_ptr(), st)
        e1.record()
        torch.cuda.synchronize()
        assert rc == 0, _lib.last_error()
        r = {"ms": e0.elapsed_time(e1)}
        if name == "refined":
            it, corr, fb = solver.refine_stats()
            r.update({"refine_iterations": it, "last_correction": corr, "fp64_fallback": fb})
        r["eig_error"] = float((deig[:n] - lam_sorted).abs().max() / lam_sorted.abs().max())
        h = master.T
        v = work.T
        r["residual"] = metrics.torch_residual(h, v, deig[:n])
        r["orthonormality"] = metrics.torch_orthonormality(v)
        out[name] = r
        del work, v
    out["speedup"] = out["fp64"]["ms"] / out["refined"]["ms"]
    del master
    torch.cuda.empty_cache()
    return out


# --------------------------------------------------------------- serving
def serving_requests(count: int, seed: int = 4242):
    """Mixed stream: n log-uniform in [32, 2048]; 70% random (as config 0),
    30% clustered spectra (as config 3: 20% of the values in clusters of 8
    with gaps 1e-6)."""
    from zquatev_gb300 import inputs

    rng = np.random.default_rng(seed)
    ns = inputs.log_uniform_sizes(count, 32, 2048, seed)
    clustered = rng.random(count) < 0.3
    mats = []
    for i, (n, cl) in enumerate(zip(ns, clustered)):
        n = int(n)
        if cl:
            dm, _ = inputs.clustered_matrix_device(n, seed + i)
            mats.append(np.asfortranarray(dm.cpu().numpy().T))
            del dm
        else:
            mats.append(inputs.random_matrix(n, seed + i))
    return mats, clustered


def _fresh(mats):
    return [(np.array(d, order="F", copy=True), np.zeros(d.shape[1])) for d in mats]


def serve_server(mats, arrivals, lanes: int):
    from zquatev_gb300.serve import Server

    bufs = _fresh(mats)
    with Server(lanes=lanes) as srv:
        ids = []
        t0 = time.perf_counter()
        for d, (o, e), a in zip(mats, bufs, arrivals):
            wait = a - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(wait)
            ids.append(srv.submit(d.shape[1], o, d.shape[0], e))
        res = [srv.wait(i) for i in ids]
        st = srv.stats()
    assert all(info == 0 for info, _ in res), [info for info, _ in res]
    lat = np.array([t["done"] - t["submit"] for _, t in res])
    span = max(t["done"] for _, t in res) - min(t["submit"] for _, t in res)
    paths = {}
    for _, t in res:
        paths[t["path"]] = paths.get(t["path"], 0) + 1
    return bufs, {"solves_per_s": len(mats) / (span * 1e-3), "p50_ms": float(np.percentile(lat, 50)),
                  "p99_ms": float(np.percentile(lat, 99)), "mean_ms": float(lat.mean()),
                  "hbm_mean_reserved_gb": st["mean_reserved_bytes"] / 1e9,
                  "hbm_peak_reserved_gb": st["peak_reserved_bytes"] / 1e9,
                  "batches": st["batches"], "paths": paths}


def serve_fp64_serial(mats, arrivals):
    """The same stream served one request at a time, in arrival order, by the
    plain FP64 drop-in (zquatev_fp64_c on the host arrays)."""
    from zquatev_gb300 import _lib, solver

    lib = _lib.load()
    bufs = _fresh(mats)
    lat, done = [], []
    busy = 0.0
    t0 = time.perf_counter()
    for (o, e), a in zip(bufs, arrivals):
        now = time.perf_counter() - t0
        if now < a:
            time.sleep(a - now)
        s0 = time.perf_counter()
        rc = solver.zquatev_fp64(o.shape[1], o, o.shape[0], e)
        t = time.perf_counter() - t0
        assert rc == 0
        busy_i = time.perf_counter() - s0
        busy += busy_i * lib.zq_solve_footprint(o.shape[1], 0)
        lat.append((t - a) * 1e3)
        done.append(t)
    lat = np.array(lat)
    span = done[-1] - arrivals[0]
    return bufs, {"solves_per_s": len(mats) / span, "p50_ms": float(np.percentile(lat, 50)),
                  "p99_ms": float(np.percentile(lat, 99)), "mean_ms": float(lat.mean()),
                  "hbm_mean_reserved_gb": busy / span / 1e9,
                  "hbm_peak_reserved_gb": max(lib.zq_solve_footprint(d.shape[1], 0) for d, _ in bufs) / 1e9}


def serving_case(count: int, rates: list[float], lanes: int) -> dict:
    import torch

    from zquatev_gb300 import inputs, metrics

    t_gen = time.perf_counter()
    mats, clustered = serving_requests(count)
    t_gen = time.perf_counter() - t_gen
    # capacity of the one-at-a-time FP64 drop-in: everything arriving at t = 0
    zero = np.zeros(count)
    _, fp_sat = serve_fp64_serial(mats, zero)
    bufs, sv_sat = serve_server(mats, zero, lanes)
    # accuracy of every served result (GPU residual, FP64 torch as the checker)
    worst_res, worst_eig = 0.0, 0.0
    for d, (o, e) in zip(mats, bufs):
        n = d.shape[1] // 2
        h = torch.from_numpy(inputs.full_from_blocks(d[:n, :n], d[n:, :n])).cuda()
        v = torch.from_numpy(np.ascontiguousarray(o.T)).cuda().T
        ev = torch.from_numpy(e[:n]).cuda()
        worst_res = max(worst_res, metrics.torch_residual(h, v, ev))
        w = torch.linalg.eigvalsh(h)[::2]
        worst_eig = max(worst_eig, float((ev - w).abs().max() / w.abs().max()))
        del h, v, w
    mu = fp_sat["solves_per_s"]
    runs = []
    rng = np.random.default_rng(99)
    for r in rates:
        lam = r * mu
        arr = np.cumsum(rng.exponential(1.0 / lam, count))
        arr -= arr[0]
        _, fp = serve_fp64_serial(mats, arr)
        _, sv = serve_server(mats, arr, lanes)
        runs.append({"rate_per_s": lam, "rate_x_fp64_capacity": r, "server": sv, "fp64_serial": fp})
    sizes = [d.shape[1] for d in mats]
    return {"workload": f"{count} requests, n log-uniform in [32, 2048] (n2 {min(sizes)}..{max(sizes)}), "
                        f"{int(clustered.sum())} clustered (config 3 style) + {count - int(clustered.sum())} random, "
                        "Poisson arrivals; host arrays in, host arrays out",
            "lanes": lanes, "generation_s": t_gen,
            "saturation": {"server": sv_sat, "fp64_serial": fp_sat,
                           "speedup": sv_sat["solves_per_s"] / fp_sat["solves_per_s"]},
            "rates": runs, "max_residual": worst_res, "max_eig_error": worst_eig}


# --------------------------------------------------------------- GPU arm
def measured_peaks() -> dict:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return json.load(f)
    except Exception:
        return {}


def main():
    args = parse()
    rank, world, local = dist_info()
    if args.profile_n2:
        profile_case(args.profile_n2, args.reps, args.profile_path)
        return
    args.cpu_sample_n2 = cpu_sample_n2(args.cpu_sample_n2)
    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    import ctypes

    import torch

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from zquatev_gb300 import _lib, build, inputs, metrics, solver

    if not build.up_to_date():
        build.build()
    lib = _lib.load()
    n2 = args.n2
    n = n2 // 2
    dev = torch.device("cuda", local)

    # synthetic input (per-rank seed), master copy resident in HBM
    d_host = inputs.random_matrix(n, 1000 + rank)
    master = torch.from_numpy(np.ascontiguousarray(d_host.T)).to(dev)      # (n2, n2) = column-major D
    work = torch.empty_like(master)
    deig = torch.zeros(n2, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step(fn="zquatev_device"):
        work[:n].copy_(master[:n])  # restore the left half (columns 0..n-1 of D)
        rc = getattr(lib, fn)(n2, work.data_ptr(), n2, deig.data_ptr(), stream.cuda_stream)
        if rc != 0:
            raise RuntimeError(f"{fn} rc={rc}: {_lib.last_error()}")

    # panel widths: the project's autotuner at this size, for both precisions
    tuned_nb = {}
    for prec in ("fp32", "fp64"):
        best, ms = solver.autotune_nb(n2, prec)
        tuned_nb[prec] = {"nb": best, "candidates": {str(c): round(m, 2) for c, m in zip((16, 32, 64, 128), ms)}}

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # timed region: K steps of the drop-in's default path (refined, FP64 fallback)
    all_classes = sum(1 << c for c in (0, 1, 3, 4, 5, 6, 7, 9, 10))
    # inside the timed region only the Ozaki product and the whole refinement are
    # bracketed with events (a few pairs per step); per-column event records of
    # the tridiagonalisation classes would perturb the step they measure
    timed_classes = (1 << 9) | (1 << 10)
    lib.zq_profile_reset()
    lib.zq_profile_enable(timed_classes)
    barrier()
    torch.cuda.synchronize()
    launches0 = lib.zq_launch_count()
    with ClockSampler(local) as clk:
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
    barrier()
    launches = lib.zq_launch_count() - launches0
    lib.zq_profile_enable(0)
    ms_total = max_over_ranks(e0.elapsed_time(e1), world, dev)
    ms_step = ms_total / args.steps
    prof = {k: _lib.profile_read(k) for k in ("ozaki", "refine", "tridiag", "stedc", "formq", "apply_z")}
    oz_flops = _lib.profile_flops("ozaki") / args.steps
    iters, last_corr, fell_back = solver.refine_stats()

    # end to end through the host C ABI (H2D + solve + D2H inside), from and to
    # pinned host arrays (one untimed call first: it maps the device copy of D
    # in the stream-ordered pool). Measured right after the device-resident
    # steps, before the FP64 comparisons heat the GPU, with its own clock record.
    pinned_d = torch.empty((n2, n2), dtype=torch.complex128, pin_memory=True)
    dh = pinned_d.numpy().T  # column-major (Fortran) view, ld2 = n2
    eh = torch.zeros(n2, dtype=torch.float64, pin_memory=True).numpy()
    e2e_ms = []
    with ClockSampler(local) as e2e_clk:
        for i in range(args.e2e_steps + 1):
            dh[...] = d_host
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            rc = solver.zquatev(n2, dh, n2, eh)
            t1 = time.perf_counter()
            assert rc == 0, _lib.last_error()
            if i > 0:
                e2e_ms.append((t1 - t0) * 1e3)
    e2e = float(np.mean(e2e_ms))

    # accuracy of the last device solve (GPU residual; FP64 torch matmul as checker)
    acc = {}
    if not args.no_check:
        h = torch.from_numpy(inputs.full_from_blocks(d_host[:n, :n], d_host[n:, :n])).to(dev)
        v = work.T  # column-major view
        acc = {"residual": metrics.torch_residual(h, v, deig[:n]), "orthonormality": metrics.torch_orthonormality(v),
               "refine_iterations": iters, "last_correction": last_corr, "fp64_fallback": fell_back}
        w = torch.linalg.eigvalsh(h)[::2]
        acc["eig_error"] = float((deig[:n] - w).abs().max() / w.abs().max())
        del h, w

    # the plain FP64 GPU path on the same input (the comparison the target names):
    # timed without instrumentation, then once more with every kernel class
    # bracketed for its per-class roofline figures
    torch.cuda.synchronize()
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    step("zquatev_fp64_device")
    f1.record(stream)
    torch.cuda.synchronize()
    fp64_ms = f0.elapsed_time(f1)
    lib.zq_profile_reset()
    lib.zq_profile_enable(all_classes)
    step("zquatev_fp64_device")
    torch.cuda.synchronize()
    lib.zq_profile_enable(0)
    fprof = {k: _lib.profile_read(k) for k in ("hemv", "trail", "formq_gemm", "apply_z", "stedc", "tridiag", "formq")}



    peaks = measured_peaks()
    bf16_peak = peaks.get("bf16_tflops_sustained") or peaks.get("bf16_tflops")
    peak_src = "MEASURED_PEAKS.json bf16_tflops_sustained (kernel timed inside a long step)"
    if not bf16_peak:
        bf16_peak, peak_src = 1700.0, "fallback 1.7 PFLOP/s sustained (MEASURED_PEAKS.json absent)"
    oz_ms = prof["ozaki"][0] / args.steps
    oz_launches = prof["ozaki"][1] / args.steps
    achieved = oz_flops / (oz_ms * 1e-3) / 1e12 if oz_ms > 0 else None
    fp64_peak = fp64_peak_tflops()
    # FP64-path kernel classes against the FP64 (DFMA) pipe, executed flops per solve
    F = {"trail": (32.0 / 3.0) * n ** 3, "hemv": (32.0 / 3.0) * n ** 3, "formq_gemm": 16.0 * n ** 3,
         "apply_z": 8.0 * n ** 3}
    fp64_roof = {k: {"ms": round(fprof[k][0], 2), "tflops": round(F[k] / (fprof[k][0] * 1e-3) / 1e12, 3),
                     "frac": round(F[k] / (fprof[k][0] * 1e-3) / 1e12 / fp64_peak, 3)}
                 for k in F if fprof[k][0] > 0}

    del master, work
    torch.cuda.empty_cache()
    batched = batched_case(args.batch_count, fp64_peak) if (rank == 0 and args.batch_count > 0) else None
    clustered = clustered_case(args.clustered_n2) if (rank == 0 and args.clustered_n2 > 0) else None
    serving = None
    if rank == 0 and args.serve_requests > 0:
        serving = serving_case(args.serve_requests, [float(x) for x in args.serve_rates.split(",")], args.serve_lanes)

    if rank == 0:
        cpu_ms, cpu_raw = cpu_sample(args.cpu_sample_n2, n2, os.cpu_count() or 1)
        clocks = clk.summary()
        line = {
            "metric": METRIC,
            "value": ms_step,
            "unit": "ms",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": ms_step,
            "higher_is_better": False,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f64 (FP32 decomposition + bf16-Ozaki-refined to FP64 accuracy)",
            "data": "synthetic",
            "config": workload_config(n2, world),
            "path": "drop-in default: FP32 decomposition + Ozaki-product refinement to FP64 accuracy",
            "nb_tuned": tuned_nb,
            "fp64_path_ms": fp64_ms,
            "speedup_vs_fp64_path": fp64_ms / ms_step if ms_step > 0 else None,
            "e2e": {"value": e2e, "unit": "ms", "h2d_bytes_per_step": n2 * n * 16,
                    "d2h_bytes_per_step": n2 * n2 * 16 + n * 8, "host_memory": "pinned",
                    "samples_ms": [round(x, 1) for x in e2e_ms], "clocks": e2e_clk.summary()},
            "gpu_launches": None,
            "roofline": {"bound": "tensor", "kernel": "k_oz_umma<2> (bf16 2-SM tcgen05.mma cta_group::2, M=256 N=256 per CTA pair; TMEM accumulators; TMA; Ozaki slices)",
                         "achieved": achieved, "peak": bf16_peak, "unit": "TFLOP/s",
                         "frac": (achieved / bf16_peak) if achieved else None,
                         "traffic": (OZ_BYTES_PER_FLOP * oz_flops / oz_launches
                                     if (oz_launches and OZ_BYTES_PER_FLOP) else None),
                         "traffic_source": "profiles/k_oz_umma_n2-4096.md: dram read+write per executed flop of one "
                                           "captured launch (n2=4096), scaled by this step's executed flops per launch",
                         "peak_source": peak_src, "launches_per_step": oz_launches, "ms_per_step": oz_ms},
            "stage_ms": {"refine": round(prof["refine"][0] / args.steps, 2), "ozaki": round(oz_ms, 2),
                         "fp32_decomposition": round(ms_step - prof["refine"][0] / args.steps, 2)},
            "fp64_path_roofline": {"pipe": "fp64 DFMA", "peak_tflops_measured": round(fp64_peak, 3),
                                   "dmma_tflops_measured": dmma_all_shapes(),
                                   "kernels": fp64_roof},
            "accuracy": acc,
            "cpu_baseline": cpu_baseline_fields(cpu_ms, n2, args.cpu_sample_n2, cpu_raw, os.cpu_count() or 1),
            "clocks": clocks,
        }
        line["gpu_launches"] = int(launches)
        if serving is not None:
            ref_rate = min(serving["rates"], key=lambda r: abs(r["rate_x_fp64_capacity"] - 1.0))
            line["mixed_stream"] = {
                "solves_per_s": serving["saturation"]["server"]["solves_per_s"],
                "fp64_serial_solves_per_s": serving["saturation"]["fp64_serial"]["solves_per_s"],
                "p99_ms": ref_rate["server"]["p99_ms"], "fp64_serial_p99_ms": ref_rate["fp64_serial"]["p99_ms"],
                "p99_at_rate_per_s": ref_rate["rate_per_s"], "max_residual": serving["max_residual"]}
            line["serving"] = serving
        if batched is not None:
            line["batched"] = batched
        if clustered is not None:
            line["clustered"] = clustered
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
