// Policy backward on the tcgen05 tensor cores (racer/ppo.mojo:113-138):
// BF16 operands, FP32 accumulation, FP32 outputs in the reference's layouts.
//
//   d2 = (W2^T d3) * (1 - h2^2)                   k_dgrad2_tc (K = 3: CUDA cores)
//   d1 = (W1^T d2[:64]) * (1 - h1^2)              GEMM D[b, j] = d2s[b, :] . W1t[j, :], epilogue EpiDgrad1
//   gW0[r, k] = sum_b d1[r, b] x[k, b]            GEMM D[k, r] = xb[k, :] . d1f[r, :], split-K over b
//   gW1[r, j] = sum_b d2[r, b] h1[j, b]           GEMM D[j, r] = h1b[j, :] . d2f[r, :], split-K
//   gW2[r, j] = sum_b d3[r, b] h2[j, b]           GEMM D[j, r] = h2b[j, :] . d3f[r, :], split-K
//
// Every GEMM is the generic TMA-fed kernel of gemm_tc.cuh; the weight
// gradients' split-K partials are summed in a fixed order and written
// straight into the theta layout W0 [64, IN] | W1 [64, 65] | W2 [3, 65].
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

// dst[r * ld + c] = bf16(src[r * cols + c]) for r < rows, c < cols.
__global__ void k_rows_bf16(const float* __restrict__ src, int rows, int cols, bf16* dst, int ld) {
  const long total = (long)rows * cols;
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const long r = e / cols, c = e % cols;
    dst[r * ld + c] = __float2bfloat16_rn(src[e]);
  }
}

// d2 = (W2^T d3) * (1 - h2^2) per sample j, with BF16 copies: d2s [cols, 64]
// sample-major, d2f [64, ld] and d3f [16, ld] feature-major.
__global__ void k_dgrad2_tc(int in, const float* __restrict__ theta, const float* __restrict__ d3,
                            const float* __restrict__ h2, float* d2, int cols, bf16* d2s, bf16* d2f, bf16* d3f,
                            int ld) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= cols) return;
  const float* w2 = theta + H * in + H * HA;
  const float e0 = d3[j], e1 = d3[(long)cols + j], e2 = d3[2L * cols + j];
  d3f[j] = __float2bfloat16_rn(e0);
  d3f[(long)ld + j] = __float2bfloat16_rn(e1);
  d3f[2L * ld + j] = __float2bfloat16_rn(e2);
  uint32_t packed[H / 2];
#pragma unroll
  for (int k = 0; k < HA; ++k) {
    const float acc = w2[k] * e0 + w2[HA + k] * e1 + w2[2 * HA + k] * e2;
    const float a = h2[(long)k * cols + j];
    const float v = acc * (1.0f - a * a);
    d2[(long)k * cols + j] = v;
    if (k < H) {
      d2f[(long)k * ld + j] = __float2bfloat16_rn(v);
      __nv_bfloat16 b = __float2bfloat16_rn(v);
      uint16_t bits = *reinterpret_cast<uint16_t*>(&b);
      if (k & 1)
        packed[k >> 1] |= (uint32_t)bits << 16;
      else
        packed[k >> 1] = bits;
    }
  }
  uint4* row = reinterpret_cast<uint4*>(d2s + (long)j * H);
#pragma unroll
  for (int q = 0; q < H / 8; ++q)
    row[q] = make_uint4(packed[4 * q], packed[4 * q + 1], packed[4 * q + 2], packed[4 * q + 3]);
}

// d1[j, m] = v * (1 - h1[j, m]^2) for j < 65 (FP32, feature-major) and its BF16
// copy d1f[j, m] for j < 64. Row m is the sample, column n the input unit j.
struct EpiDgrad1 {
  const float* h1;
  int cols;
  float* d1;
  bf16* d1f;
  int ld;
  __device__ void operator()(int m, int n, const float* v, int z) const {
    (void)z;
    if (m >= cols) return;
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const int j = n + q;
      if (j < HA) {
        const float a = h1[(long)j * cols + m];
        const float g = v[q] * (1.0f - a * a);
        d1[(long)j * cols + m] = g;
        if (j < H) d1f[(long)j * ld + m] = __float2bfloat16_rn(g);
      }
    }
  }
};

// grad[off + n * ldg + m] = sum_z P[z][m][n] for m < mreal, n < nreal (the
// GEMM row m is the weight's input index, column n its output row).
__global__ void k_wgrad_reduce(const float* __restrict__ P, int splits, int mrows, int nreal, int mreal,
                               float* grad, int ldg) {
  const long total = (long)mreal * nreal;
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const int n = (int)(e / mreal), m = (int)(e % mreal);
    float acc = 0.0f;
    for (int z = 0; z < splits; ++z) acc += P[((long)z * mrows + m) * nreal + n];
    grad[(long)n * ldg + m] = acc;
  }
}

// W1^T as BF16 [128, 64]: row j (input unit, zero past 64) holds W1[0..63, j].
__global__ void k_pack_w1t(const float* __restrict__ theta, int in, bf16* w1t) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= 128 * H) return;
  const int j = e / H, r = e % H;
  w1t[e] = __float2bfloat16_rn(j < HA ? theta[H * in + r * HA + j] : 0.0f);
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
  bf16 *xb = nullptr, *h1b = nullptr, *h2b = nullptr, *d2s = nullptr, *d2f = nullptr, *d3f = nullptr, *d1f = nullptr,
       *w1t = nullptr;
  float* scratch = nullptr;
  CUtensorMap txb, th1b, th2b, td2s, td2f, td3f, td1f, tw1t;
};

int backward_work_new(int in, int cols, BackwardWork** out) {
  BackwardWork* w = new BackwardWork();
  w->in = in;
  w->cols = cols;
  w->ld = (cols + 7) / 8 * 8;
  const size_t ld = w->ld;
  int rc = 0;
  if ((rc = walloc(&w->xb, (size_t)in * ld)) || (rc = walloc(&w->h1b, (size_t)HA * ld)) ||
      (rc = walloc(&w->h2b, (size_t)HA * ld)) || (rc = walloc(&w->d2s, (size_t)cols * H)) ||
      (rc = walloc(&w->d2f, (size_t)H * ld)) || (rc = walloc(&w->d3f, (size_t)16 * ld)) ||
      (rc = walloc(&w->d1f, (size_t)H * ld)) || (rc = walloc(&w->w1t, (size_t)128 * H)) ||
      (rc = walloc(&w->scratch, (size_t)MAX_SPLIT_TILES * 128 * 64))) {
    backward_work_delete(w);
    return rc;
  }
  if ((rc = make_tmap_bf16(&w->txb, w->xb, in, ld, ld, 128)) || (rc = make_tmap_bf16(&w->th1b, w->h1b, HA, ld, ld, 128)) ||
      (rc = make_tmap_bf16(&w->th2b, w->h2b, HA, ld, ld, 128)) || (rc = make_tmap_bf16(&w->td2s, w->d2s, cols, H, H, 128)) ||
      (rc = make_tmap_bf16(&w->td2f, w->d2f, H, ld, ld, 64)) || (rc = make_tmap_bf16(&w->td3f, w->d3f, 16, ld, ld, 16)) ||
      (rc = make_tmap_bf16(&w->td1f, w->d1f, H, ld, ld, 64)) || (rc = make_tmap_bf16(&w->tw1t, w->w1t, 128, H, H, 128))) {
    backward_work_delete(w);
    return rc;
  }
  *out = w;
  return 0;
}

void backward_work_delete(BackwardWork* w) {
  if (!w) return;
  for (bf16* p : {w->xb, w->h1b, w->h2b, w->d2s, w->d2f, w->d3f, w->d1f, w->w1t}) cudaFree(p);
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
  k_wgrad_reduce<<<(unsigned)std::min<long>((total + 255) / 256, 1024), 256, 0, st>>>(w->scratch, splits, mrows,
                                                                                        nreal, mreal, grad, ldg);
  BW_CHECK(cudaGetLastError());
  return 0;
}
}  // namespace

int backward_refresh(BackwardWork* w, const float* theta, cudaStream_t st) {
  k_pack_w1t<<<(128 * H + 255) / 256, 256, 0, st>>>(theta, w->in, w->w1t);
  BW_CHECK(cudaGetLastError());
  return 0;
}

int backward_tc(BackwardWork* w, const float* theta, const float* x, const float* h1, const float* h2,
                const float* d3, float* d2, float* d1, float* grad, int* err, cudaStream_t st) {
  const int in = w->in, cols = w->cols, ld = w->ld;
  k_rows_bf16<<<592, 256, 0, st>>>(x, in, cols, w->xb, ld);
  k_rows_bf16<<<592, 256, 0, st>>>(h1, HA, cols, w->h1b, ld);
  k_rows_bf16<<<592, 256, 0, st>>>(h2, HA, cols, w->h2b, ld);
  k_dgrad2_tc<<<(cols + 127) / 128, 128, 0, st>>>(in, theta, d3, h2, d2, cols, w->d2s, w->d2f, w->d3f, ld);
  BW_CHECK(cudaGetLastError());
  BW_CHECK(gemm_launch<128>(w->td2s, w->tw1t, cols, HA, 1, 1, EpiDgrad1{h1, cols, d1, w->d1f, ld}, err, st));
  int rc;
  if ((rc = wgrad<64>(w, w->txb, w->td1f, in, H, in, grad, in, err, st))) return rc;
  if ((rc = wgrad<64>(w, w->th1b, w->td2f, HA, H, HA, grad + H * in, HA, err, st))) return rc;
  if ((rc = wgrad<16>(w, w->th2b, w->td3f, HA, OUT, HA, grad + H * in + H * HA, HA, err, st))) return rc;
  return 0;
}

}  // namespace racer
