// Plain BF16 GEMM entry point over the generic tcgen05 kernel (gemm_tc.cuh):
// C[M, N] (FP32, row-major, ldc) = A[M, K] . B[N, K]^T with A and B BF16
// row-major (K contiguous). With splits > 1 the K range is split across CTAs
// and the partial tiles are summed in a fixed order by a second kernel.
#include <cuda_bf16.h>

#include <string>

#include "../../include/racer.h"
#include "common.cuh"
#include "gemm_tc.cuh"
#include "gemm_epi.cuh"
#include "tma.h"

namespace racer {
namespace {

__global__ void k_sum_splits(const float* P, int splits, long mn, int M, int N, float* C, int ldc) {
  long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long)M * N) return;
  int m = (int)(e / N), n = (int)(e % N);
  float acc = 0.0f;
  for (int z = 0; z < splits; ++z) acc += P[(long)z * mn + (long)m * N + n];
  C[(long)m * ldc + n] = acc;
}

}  // namespace
}  // namespace racer

using namespace racer;

extern "C" int racer_gemm_bf16(const void* a_dev, const void* b_dev, float* c_dev, int M, int N, int K, int lda,
                               int ldb, int ldc, int splits, float* scratch_dev, int* err_dev, void* stream) {
  if (!a_dev || !b_dev || !c_dev || !err_dev || M < 1 || N < 1 || K < 1 || lda < K || ldb < K || ldc < N ||
      (lda % 8) || (ldb % 8) || splits < 1 || (splits > 1 && !scratch_dev)) {
    racer_host::set_error("racer_gemm_bf16: bad argument (leading dimensions must be multiples of 8)");
    return 1;
  }
  const int BN = N <= 64 ? 64 : (N <= 128 ? 128 : 256);
  CUtensorMap ta, tb;
  int rc = make_tmap_bf16(&ta, a_dev, M, K, lda, 128);
  if (!rc) rc = make_tmap_bf16(&tb, b_dev, N, K, ldb, BN);
  if (rc) return rc;
  const int kblocks = (K + 63) / 64;
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e;
  int per = (kblocks + splits - 1) / splits;
  int used = (kblocks + per - 1) / per;
  if (used <= 1) {
    EpiRowF32 epi{c_dev, ldc, M, N};
    e = BN == 64 ? gemm_launch<64>(ta, tb, M, N, kblocks, 1, epi, err_dev, st)
                 : (BN == 128 ? gemm_launch<128>(ta, tb, M, N, kblocks, 1, epi, err_dev, st)
                              : gemm_launch<256>(ta, tb, M, N, kblocks, 1, epi, err_dev, st));
  } else {
    EpiSplitF32 epi{scratch_dev, (long)M * N, M, N};
    e = BN == 64 ? gemm_launch<64>(ta, tb, M, N, kblocks, used, epi, err_dev, st)
                 : (BN == 128 ? gemm_launch<128>(ta, tb, M, N, kblocks, used, epi, err_dev, st)
                              : gemm_launch<256>(ta, tb, M, N, kblocks, used, epi, err_dev, st));
    if (e == cudaSuccess) {
      long count = (long)M * N;
      k_sum_splits<<<(unsigned)((count + 255) / 256), 256, 0, st>>>(scratch_dev, used, count, M, N, c_dev, ldc);
      e = cudaGetLastError();
    }
  }
  if (e != cudaSuccess) {
    racer_host::set_error(std::string("racer_gemm_bf16: ") + cudaGetErrorString(e));
    return 2;
  }
  return 0;
}
