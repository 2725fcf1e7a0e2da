// Policy MLP GEMMs in FP32 on the CUDA cores (racer/ppo.mojo:108-138):
// forward C = tanh(W x) with feature-major activations, and the backward
// passes (dgrad through tanh, weight gradients with a deterministic split-K
// reduction over the batch).
#include "common.cuh"
#include "kernels.h"

namespace racer {
namespace {

constexpr int BM = 64, BN = 64, BK = 16;

// C[M, N] (+)= op(A)[M, K] @ op(B)[K, N]; op(A)(m, k) = ta ? A[k*lda + m] : A[m*lda + k],
// op(B)(k, n) = tb ? B[n*ldb + k] : B[k*ldb + n]. Block (bx, by, z) computes a 64x64
// tile over the K range of split z and writes it to C + z * split_stride.
__global__ void __launch_bounds__(256) k_sgemm(const float* __restrict__ A, int lda, int ta,
                                               const float* __restrict__ B, int ldb, int tb, float* __restrict__ C,
                                               int ldc, long split_stride, int M, int N, int K, int kper,
                                               int squash) {
  __shared__ float As[BK][BM + 4];
  __shared__ float Bs[BK][BN + 4];
  int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  int k0 = blockIdx.z * kper, k1 = min(K, k0 + kper);
  float acc[4][4] = {};
  for (int kb = k0; kb < k1; kb += BK) {
    for (int e = threadIdx.x; e < BK * BM; e += 256) {
      int kk, mm;
      if (ta) { mm = e % BM; kk = e / BM; } else { kk = e % BK; mm = e / BK; }
      int m = m0 + mm, k = kb + kk;
      float v = 0.0f;
      if (m < M && k < k1) v = ta ? A[(long)k * lda + m] : A[(long)m * lda + k];
      As[kk][mm] = v;
    }
    for (int e = threadIdx.x; e < BK * BN; e += 256) {
      int kk, nn;
      if (tb) { kk = e % BK; nn = e / BK; } else { nn = e % BN; kk = e / BN; }
      int n = n0 + nn, k = kb + kk;
      float v = 0.0f;
      if (n < N && k < k1) v = tb ? B[(long)n * ldb + k] : B[(long)k * ldb + n];
      Bs[kk][nn] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) a[r] = As[kk][ty * 4 + r];
#pragma unroll
      for (int c = 0; c < 4; ++c) b[c] = Bs[kk][tx * 4 + c];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[r][c] += a[r] * b[c];
    }
    __syncthreads();
  }
  float* Cz = C + blockIdx.z * split_stride;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    int m = m0 + ty * 4 + r;
    if (m >= M) continue;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      int n = n0 + tx * 4 + c;
      if (n < N) Cz[(long)m * ldc + n] = squash ? tanhf(acc[r][c]) : acc[r][c];
    }
  }
}

// C[m, n] = sum over splits of P[z][m][n] (fixed order).
__global__ void k_split_reduce(const float* P, int splits, int M, int N, float* C, int ldc) {
  long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long)M * N) return;
  int m = (int)(e / N), nn = (int)(e % N);
  float acc = 0.0f;
  for (int z = 0; z < splits; ++z) acc += P[(long)z * M * N + e];
  C[(long)m * ldc + nn] = acc;
}

// d2 = (W2^T d3) * (1 - h2^2): one thread per sample column.
__global__ void k_dgrad2(int in, const float* theta, const float* d3, const float* h2, float* d2, int cols) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= cols) return;
  const float* w2 = theta + H * in + H * HA;
  float e0 = d3[j], e1 = d3[(long)cols + j], e2 = d3[2L * cols + j];
  for (int k = 0; k < HA; ++k) {
    float acc = w2[k] * e0 + w2[HA + k] * e1 + w2[2 * HA + k] * e2;
    float a = h2[(long)k * cols + j];
    d2[(long)k * cols + j] = acc * (1.0f - a * a);
  }
}

// out *= (1 - h^2), element-wise over [rows, cols].
__global__ void k_tanh_mask(float* out, const float* h, long count) {
  long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= count) return;
  float a = h[e];
  out[e] = out[e] * (1.0f - a * a);
}

int splits_for(int K, int tiles) {
  // enough blocks to fill the GPU, at least 512 K per split
  int want = std::max(1, SPLIT_CTAS / std::max(1, tiles));
  int most = std::max(1, K / 512);
  return std::min(want, most);
}

void sgemm(const float* A, int lda, int ta, const float* B, int ldb, int tb, float* C, int ldc, int M, int N, int K,
           int squash, float* scratch, cudaStream_t st) {
  dim3 grid((N + BN - 1) / BN, (M + BM - 1) / BM, 1);
  int splits = scratch ? splits_for(K, grid.x * grid.y) : 1;
  if (splits <= 1) {
    k_sgemm<<<grid, 256, 0, st>>>(A, lda, ta, B, ldb, tb, C, ldc, 0, M, N, K, K, squash);
    return;
  }
  int kper = ((K + splits - 1) / splits + BK - 1) / BK * BK;
  splits = (K + kper - 1) / kper;
  grid.z = splits;
  k_sgemm<<<grid, 256, 0, st>>>(A, lda, ta, B, ldb, tb, scratch, N, (long)M * N, M, N, K, kper, 0);
  long count = (long)M * N;
  k_split_reduce<<<(unsigned)((count + 255) / 256), 256, 0, st>>>(scratch, splits, M, N, C, ldc);
}

}  // namespace

void launch_sgemm(const float* A, int lda, const float* B, int ldb, float* C, int ldc, int M, int N, int K,
                  int squash, cudaStream_t st) {
  sgemm(A, lda, 0, B, ldb, 0, C, ldc, M, N, K, squash, nullptr, st);
}

// Split-K partials: splits * tiles <= SPLIT_CTAS and every tile is at most 64 x 64.
static_assert(BM == 64 && BN == 64, "BACKWARD_SCRATCH_FLOATS assumes 64 x 64 tiles");
size_t backward_scratch_floats(int in, int cols) {
  (void)in;
  (void)cols;
  return BACKWARD_SCRATCH_FLOATS;
}

// Floats of split-K partials one weight-gradient GEMM [M, N] over K uses (0 when unsplit).
static size_t split_need(int M, int N, int K) {
  int tiles = ((N + BN - 1) / BN) * ((M + BM - 1) / BM);
  int splits = splits_for(K, tiles);
  if (splits <= 1) return 0;
  int kper = ((K + splits - 1) / splits + BK - 1) / BK * BK;
  splits = (K + kper - 1) / kper;
  return (size_t)splits * M * N;
}

size_t backward_scratch_needed(int in, int cols) {
  return std::max(split_need(H, in, cols), std::max(split_need(H, HA, cols), split_need(OUT, HA, cols)));
}

// racer/ppo.mojo:113-138: d3 [3, cols] -> d2, d1 [HA, cols], grad[W0|W1|W2].
void launch_backward(int in, const float* theta, const float* x, int cols, const float* h1, const float* h2,
                     const float* d3, float* d2, float* d1, float* grad, float* scratch, cudaStream_t st) {
  const int w1 = H * in, w2 = w1 + H * HA;
  k_dgrad2<<<(cols + 127) / 128, 128, 0, st>>>(in, theta, d3, h2, d2, cols);
  // d1 = W1^T[HA, H] d2[:H] then * (1 - h1^2)
  sgemm(theta + w1, HA, 1, d2, cols, 0, d1, cols, HA, cols, H, 0, nullptr, st);
  long count = (long)HA * cols;
  k_tanh_mask<<<(unsigned)((count + 255) / 256), 256, 0, st>>>(d1, h1, count);
  // weight gradients, split-K over the batch
  sgemm(d1, cols, 0, x, cols, 1, grad, in, H, in, cols, 0, scratch, st);
  sgemm(d2, cols, 0, h1, cols, 1, grad + w1, HA, H, HA, cols, 0, scratch, st);
  sgemm(d3, cols, 0, h2, cols, 1, grad + w2, HA, OUT, HA, cols, 0, scratch, st);
}

}  // namespace racer
