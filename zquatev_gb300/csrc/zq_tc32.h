// FP32-accurate tensor-core products (zq_tc32.cu): C = alpha * sum_s A_s B_s
// + beta * C over up to four segments, complex (float2) or real operands.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace zq {

// One operand of one segment. For A: element (r, k) with r an output row; for
// B: element (k, c) with c an output column, addressed as "row" c.
struct Tc32Src {
  const float* p;  // base; complex operands are interleaved (re, im) pairs
  int64_t ld;      // leading dimension in elements (complex or real)
  int kfast;       // 1: element (r, k) at p[k + r * ld]; 0: at p[r + k * ld]
  int conj;        // complex: use the conjugate
  float sign;      // +1 or -1
  int vec;         // filled by tc32_gemm: 16-byte loads allowed
};
struct Tc32Seg {
  Tc32Src a;       // A_s: m x k
  Tc32Src b;       // B_s: k x n (columns < nsplit when b2 is used)
  Tc32Src b2;      // optional: columns c >= nsplit come from b2 at column c - nsplit
  int nsplit;
  int k;
};
struct Tc32Args {
  int cplx;              // 1 complex, 0 real
  int m, n;              // output rows and columns
  int nseg;
  Tc32Seg seg[4];
  int kb_total;          // filled by tc32_gemm
  int kb_first[5];
  float2 alpha, beta;    // real products use .x
  float* C;
  int64_t ldc;
  int ctrans;            // 1: the product's (i, j) is stored at C[j + i * ldc]
  int tri;               // 0 every tile; 1 lower tiles, elements i >= j; 2 lower tiles, i > j
  float* P;              // split-K partials (splits * m * n elements), or null
  int splits;
  int* err;              // device flag raised when a pipeline wait runs out (may be null)
  long long wait;        // filled by tc32_gemm
};

int tc32_gemm(const Tc32Args& g, cudaStream_t st);
int tc32_smem_bytes();

}  // namespace zq
