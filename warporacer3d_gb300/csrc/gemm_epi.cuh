// Epilogues for the generic tcgen05 GEMM (gemm_tc.cuh). Each is called with
// one row m of the 128 x BN tile and 16 consecutive columns n .. n + 15.
#pragma once
#include <cuda_bf16.h>

#include "tc.cuh"

namespace racer {

// C[m * ldc + n] = v (row-major FP32).
struct EpiRowF32 {
  float* C;
  int ldc, M, N;
  __device__ void operator()(int m, int n, const float* v, int z) const {
    if (m >= M) return;
#pragma unroll
    for (int j = 0; j < 16; ++j)
      if (n + j < N) C[(long)m * ldc + n + j] = v[j];
  }
};

// Split-K partial: P[z][m][n] for split z.
struct EpiSplitF32 {
  float* P;
  long mn;
  int M, N;
  __device__ void operator()(int m, int n, const float* v, int z) const {
    if (m >= M) return;
    float* row = P + z * mn + (long)m * N;
#pragma unroll
    for (int j = 0; j < 16; ++j)
      if (n + j < N) row[n + j] = v[j];
  }
};

}  // namespace racer
