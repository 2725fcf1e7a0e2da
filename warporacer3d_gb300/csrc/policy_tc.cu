// Policy backward (racer/ppo.mojo:113-138) with BF16 operands and FP32
// accumulation, FP32 outputs in the reference's layouts.
//
//   d2 = (W2^T d3) * (1 - h2^2)                   k_dgrad (CUDA cores: K = 3)
//   d1 = (W1^T d2[:64]) * (1 - h1^2)              k_dgrad, same thread: K = 64 per sample, W1 in shared
//                                                 memory; operands rounded to BF16 like a tensor-core product
//   gW0[r, k] = sum_b d1[r, b] x[k, b]            GEMM D[k, r] = xb[k, :] . d1f[r, :], split-K over b
//   gW1[r, j] = sum_b d2[r, b] h1[j, b]           GEMM D[j, r] = h1b[j, :] . d2f[r, :], split-K
//   gW2[r, j] = sum_b d3[r, b] h2[j, b]           GEMM D[j, r] = h2b[j, :] . d3f[r, :], split-K
//
// The three weight gradients (K = batch) run on the tcgen05 tensor cores
// through the generic TMA-fed kernel of gemm_tc.cuh; their split-K partials
// are summed in a fixed order and written straight into the theta layout
// W0 [64, IN] | W1 [64, 65] | W2 [3, 65]. The data-gradient products have
// K <= 64 and N <= 65 per sample: memory-bound, so they stay on the CUDA
// cores, fused with the tanh derivatives and the BF16 operand copies.
#include <cuda_bf16.h>

#include <string>

#include "common.cuh"
#include "gemm_epi.cuh"
#include "gemm_tc.cuh"
#include "policy_tc.h"
#include "tma.h"

using bf16 = __nv_bfloat16;

namespace racer {
namespace {

// dst[r * ld + c] = bf16(src[r * cols + c]) for r < rows (blockIdx.y), c < cols;
// four columns per thread when rows of both stay 16/8-byte aligned.
__global__ void k_rows_bf16(const float* __restrict__ src, int rows, int cols, bf16* dst, int ld) {
  const int r = blockIdx.y;
  const float* s = src + (long)r * cols;
  bf16* d = dst + (long)r * ld;
  const int c = (blockIdx.x * blockDim.x + threadIdx.x) * 4;
  if (c >= cols) return;
  if ((cols & 3) == 0 && (ld & 3) == 0) {
    const float4 v = *reinterpret_cast<const float4*>(s + c);
    uint2 o;
    o.x = tc::pack_bf16(v.x, v.y);
    o.y = tc::pack_bf16(v.z, v.w);
    *reinterpret_cast<uint2*>(d + c) = o;
  } else {
    for (int q = c; q < c + 4 && q < cols; ++q) d[q] = __float2bfloat16_rn(s[q]);
  }
}

__device__ __forceinline__ float bf16_round(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

// Per sample j (one thread): d2 = (W2^T d3) * (1 - h2^2) and
// d1 = (W1^T bf16(d2[:64])) * (1 - h1^2) with W1 rounded to BF16 (the
// operands a tensor-core product would see; FP32 accumulation), written as
// FP32 d2, d1 [65, cols] plus the BF16 operand copies of the weight-gradient
// GEMMs d2f, d1f [64, ld] and d3f [16, ld] (feature-major).
constexpr int DGRAD_THREADS = 128;
constexpr int DGRAD_SMEM = (HA * H + HA * DGRAD_THREADS) * 4;

__global__ void __launch_bounds__(DGRAD_THREADS) k_dgrad(int in, const float* __restrict__ theta,
                                                         const float* __restrict__ d3, const float* __restrict__ h1,
                                                         const float* __restrict__ h2, float* d2, float* d1, int cols,
                                                         bf16* d1f, bf16* d2f, bf16* d3f, int ld) {
  extern __shared__ __align__(16) float dg_smem[];
  float(*w1t)[H] = reinterpret_cast<float(*)[H]>(dg_smem);                          // w1t[k][r] = bf16(W1[r][k])
  float(*h1s)[DGRAD_THREADS] = reinterpret_cast<float(*)[DGRAD_THREADS]>(dg_smem + HA * H);  // this thread's h1
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  // every h1 load of this sample in flight at once; each thread reads back only its own column
  if (j < cols) {
#pragma unroll
    for (int k = 0; k < HA; ++k) h1s[k][threadIdx.x] = h1[(long)k * cols + j];
  }
  const float* w1 = theta + H * in;
  for (int e = threadIdx.x; e < H * HA; e += blockDim.x) {
    const int r = e / HA, k = e % HA;
    w1t[k][r] = bf16_round(w1[e]);
  }
  __syncthreads();
  if (j >= cols) return;
  const float* w2 = theta + H * in + H * HA;
  const float e0 = d3[j], e1 = d3[(long)cols + j], e2 = d3[2L * cols + j];
  d3f[j] = __float2bfloat16_rn(e0);
  d3f[(long)ld + j] = __float2bfloat16_rn(e1);
  d3f[2L * ld + j] = __float2bfloat16_rn(e2);
  float b[H];
#pragma unroll
  for (int k = 0; k < HA; ++k) {
    const float acc = w2[k] * e0 + w2[HA + k] * e1 + w2[2 * HA + k] * e2;
    const float a = h2[(long)k * cols + j];
    const float v = acc * (1.0f - a * a);
    d2[(long)k * cols + j] = v;
    if (k < H) {
      const bf16 vb = __float2bfloat16_rn(v);
      d2f[(long)k * ld + j] = vb;
      b[k] = __bfloat162float(vb);
    }
  }
  constexpr int KU = 5;  // 65 = 13 x 5 output units per pass: five independent loads of h1 in flight
#pragma unroll 1
  for (int k0 = 0; k0 < HA; k0 += KU) {
    float acc[KU], a[KU];
#pragma unroll
    for (int u = 0; u < KU; ++u) {
      a[u] = h1s[k0 + u][threadIdx.x];
      acc[u] = 0.0f;
    }
#pragma unroll
    for (int q = 0; q < H / 4; ++q) {
#pragma unroll
      for (int u = 0; u < KU; ++u) {
        const float4 c = reinterpret_cast<const float4*>(w1t[k0 + u])[q];
        acc[u] += c.x * b[4 * q] + c.y * b[4 * q + 1] + c.z * b[4 * q + 2] + c.w * b[4 * q + 3];
      }
    }
#pragma unroll
    for (int u = 0; u < KU; ++u) {
      const int k = k0 + u;
      const float g = acc[u] * (1.0f - a[u] * a[u]);
      d1[(long)k * cols + j] = g;
      if (k < H) d1f[(long)k * ld + j] = __float2bfloat16_rn(g);
    }
  }
}

// grad[n * ldg + m] = sum_z P[z][m][n] for m < mreal, n < nreal (the GEMM row
// m is the weight's input index, column n its output row). One warp per
// element: lane l sums the partials z = l, l + 32, ... in order, then a fixed
// shuffle tree adds the lanes (deterministic).
__global__ void k_wgrad_reduce(const float* __restrict__ P, int splits, int mrows, int nreal, int mreal,
                               float* grad, int ldg) {
  const long total = (long)mreal * nreal;
  const int lane = threadIdx.x & 31;
  const long warps = ((long)gridDim.x * blockDim.x) >> 5;
  for (long e = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; e < total; e += warps) {
    const int m = (int)(e / nreal), n = (int)(e % nreal);
    float acc = 0.0f;
    for (int z = lane; z < splits; z += 32) acc += P[((long)z * mrows + m) * nreal + n];
#pragma unroll
    for (int off = 16; off; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    if (lane == 0) grad[(long)n * ldg + m] = acc;
  }
}

template <typename T>
int walloc(T** p, size_t count) {
  RACER_TRY(cudaMalloc((void**)p, count * sizeof(T) + 64));
  RACER_TRY(cudaMemset(*p, 0, count * sizeof(T) + 64));
  return 0;
}

constexpr int MAX_SPLIT_TILES = 296;

}  // namespace

struct BackwardWork {
  int in = 0, cols = 0, ld = 0;
  bf16 *xb = nullptr, *h1b = nullptr, *h2b = nullptr, *d2f = nullptr, *d3f = nullptr, *d1f = nullptr;
  float* scratch = nullptr;
  CUtensorMap txb, th1b, th2b, td2f, td3f, td1f;
};

int backward_work_new(int in, int cols, BackwardWork** out) {
  BackwardWork* w = new BackwardWork();
  w->in = in;
  w->cols = cols;
  w->ld = (cols + 7) / 8 * 8;
  const size_t ld = w->ld;
  int rc = 0;
  if ((rc = walloc(&w->xb, (size_t)in * ld)) || (rc = walloc(&w->h1b, (size_t)HA * ld)) ||
      (rc = walloc(&w->h2b, (size_t)HA * ld)) || (rc = walloc(&w->d2f, (size_t)H * ld)) ||
      (rc = walloc(&w->d3f, (size_t)16 * ld)) || (rc = walloc(&w->d1f, (size_t)H * ld)) ||
      (rc = walloc(&w->scratch, (size_t)MAX_SPLIT_TILES * 128 * 64))) {
    backward_work_delete(w);
    return rc;
  }
  if ((rc = make_tmap_bf16(&w->txb, w->xb, in, ld, ld, 128)) || (rc = make_tmap_bf16(&w->th1b, w->h1b, HA, ld, ld, 128)) ||
      (rc = make_tmap_bf16(&w->th2b, w->h2b, HA, ld, ld, 128)) || (rc = make_tmap_bf16(&w->td2f, w->d2f, H, ld, ld, 64)) ||
      (rc = make_tmap_bf16(&w->td3f, w->d3f, 16, ld, ld, 16)) || (rc = make_tmap_bf16(&w->td1f, w->d1f, H, ld, ld, 64))) {
    backward_work_delete(w);
    return rc;
  }
  *out = w;
  return 0;
}

void backward_work_delete(BackwardWork* w) {
  if (!w) return;
  for (bf16* p : {w->xb, w->h1b, w->h2b, w->d2f, w->d3f, w->d1f}) cudaFree(p);
  cudaFree(w->scratch);
  delete w;
}

int backward_work_cols(const BackwardWork* w) { return w ? w->cols : 0; }

#define BW_CHECK(expr)                                                                           \
  do {                                                                                           \
    cudaError_t e_ = (expr);                                                                     \
    if (e_ != cudaSuccess) {                                                                     \
      racer_host::set_error(std::string("policy backward: ") + #expr + ": " + cudaGetErrorString(e_)); \
      return 2;                                                                                  \
    }                                                                                            \
  } while (0)

namespace {
// split-K weight gradient D[mrows, nreal] over the batch into grad (see k_wgrad_reduce)
template <int BN>
int wgrad(BackwardWork* w, const CUtensorMap& ta, const CUtensorMap& tb, int mrows, int nreal, int mreal, float* grad,
          int ldg, int* err, cudaStream_t st) {
  const int kblocks = w->ld / 64 + (w->ld % 64 ? 1 : 0);
  const int tiles = (mrows + 127) / 128;
  int splits = std::max(1, std::min(kblocks, MAX_SPLIT_TILES / tiles));
  const int per = (kblocks + splits - 1) / splits;
  splits = (kblocks + per - 1) / per;
  EpiSplitF32 epi{w->scratch, (long)mrows * nreal, mrows, nreal};
  BW_CHECK(gemm_launch<BN>(ta, tb, mrows, nreal, kblocks, splits, epi, err, st));
  const long total = (long)mreal * nreal;
  k_wgrad_reduce<<<(unsigned)std::min<long>((total + 7) / 8, 4096), 256, 0, st>>>(w->scratch, splits, mrows, nreal,
                                                                                     mreal, grad, ldg);
  BW_CHECK(cudaGetLastError());
  return 0;
}
}  // namespace

int backward_refresh(BackwardWork* w, const float* theta, cudaStream_t st) {
  (void)w, (void)theta, (void)st;  // the backward reads W1 from theta directly
  return 0;
}

int backward_tc(BackwardWork* w, const float* theta, const float* x, const float* h1, const float* h2,
                const float* d3, float* d2, float* d1, float* grad, int* err, cudaStream_t st) {
  const int in = w->in, cols = w->cols, ld = w->ld;
  const unsigned gx = (unsigned)((cols + 1023) / 1024);
  k_rows_bf16<<<dim3(gx, in), 256, 0, st>>>(x, in, cols, w->xb, ld);
  k_rows_bf16<<<dim3(gx, HA), 256, 0, st>>>(h1, HA, cols, w->h1b, ld);
  k_rows_bf16<<<dim3(gx, HA), 256, 0, st>>>(h2, HA, cols, w->h2b, ld);
  static bool dgrad_configured = false;
  if (!dgrad_configured) {
    BW_CHECK(cudaFuncSetAttribute(k_dgrad, cudaFuncAttributeMaxDynamicSharedMemorySize, DGRAD_SMEM));
    dgrad_configured = true;
  }
  k_dgrad<<<(cols + DGRAD_THREADS - 1) / DGRAD_THREADS, DGRAD_THREADS, DGRAD_SMEM, st>>>(
      in, theta, d3, h1, h2, d2, d1, cols, w->d1f, w->d2f, w->d3f, ld);
  BW_CHECK(cudaGetLastError());
  int rc;
  if ((rc = wgrad<64>(w, w->txb, w->td1f, in, H, in, grad, in, err, st))) return rc;
  if ((rc = wgrad<64>(w, w->th1b, w->td2f, HA, H, HA, grad + H * in, HA, err, st))) return rc;
  if ((rc = wgrad<16>(w, w->th2b, w->td3f, HA, OUT, HA, grad + H * in + H * HA, HA, err, st))) return rc;
  return 0;
}

}  // namespace racer
