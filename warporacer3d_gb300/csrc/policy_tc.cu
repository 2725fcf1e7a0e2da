// Policy backward (racer/ppo.mojo:113-138) with BF16 operands and FP32
// accumulation, FP32 outputs in the reference's layouts.
//
//   d2 = (W2^T d3) * (1 - h2^2)                   k_dgrad_tc, per sample on the CUDA cores (K = 3)
//   d1 = (W1^T d2[:64]) * (1 - h1^2)              k_dgrad_tc, per tile of 128 samples on tcgen05 (K = 64)
//   gW0[r, k] = sum_b d1[r, b] x[k, b]            GEMM D[k, r] = xb[k, :] . d1f[r, :], split-K over b
//   gW1[r, j] = sum_b d2[r, b] h1[j, b]           GEMM D[j, r] = h1b[j, :] . d2f[r, :], split-K
//   gW2[r, j] = sum_b d3[r, b] h2[j, b]           GEMM D[j, r] = h2b[j, :] . d3f[r, :], split-K
//
// The three weight gradients (K = batch) run on the tcgen05 tensor cores
// through the generic TMA-fed kernel of gemm_tc.cuh; their split-K partials
// are summed in a fixed order and written straight into the theta layout
// W0 [64, IN] | W1 [64, 65] | W2 [3, 65]. The data gradients are memory-bound
// (K <= 64): one small kernel per 128 samples fuses them with the tanh
// derivatives and the BF16 operand copies of the weight-gradient GEMMs (d1,
// d2, d3 and the h1, h2 it reads anyway; x is converted on its own).
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

// W1^T as a 128B-swizzled K-major BF16 image: row j (input unit, < 64) holds
// W1[0..63][j], the B operand of the d1 product.
__global__ void k_pack_w1ts(const float* __restrict__ theta, int in, bf16* w1ts) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= H * H) return;
  const int j = e / H, r = e % H;
  w1ts[tc::sw128_offset(j, r) / 2] = __float2bfloat16_rn(theta[H * in + r * HA + j]);
}

// Data gradients per tile of 128 samples: each thread computes its sample's
// d2 = (W2^T d3) * (1 - h2^2) (K = 3, CUDA cores) and writes bf16(d2[:64]) as
// its row of a 128B-swizzled A tile; one thread issues the
// four K = 16 MMAs D[128, 64] = A . W1^T into TMEM (64 columns per CTA), and
// each thread reads its row back for d1 = D * (1 - h1^2).
// Row 64 of d1 is zero (h1's row 64 is the constant 1).
__global__ void __launch_bounds__(128, 4)
    k_dgrad_tc(int in, const float* __restrict__ theta, const uint4* __restrict__ w1ts, const float* __restrict__ d3,
               const float* __restrict__ h1, const float* __restrict__ h2, float* __restrict__ d2,
               float* __restrict__ d1, int cols, bf16* __restrict__ d1f, bf16* __restrict__ d2f,
               bf16* __restrict__ d3f, bf16* __restrict__ h1b, bf16* __restrict__ h2b, int ld, int* err,
               int write_f32) {
  __shared__ __align__(1024) uint8_t A[128 * 128];
  __shared__ __align__(1024) uint8_t B[H * 128];
  __shared__ uint64_t done;
  __shared__ uint32_t tslot;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int j = blockIdx.x * 128 + tid;
  const bool live = j < cols;
  if (tid == 0) {
    tc::mbar_init(&done, 1);
    tc::fence_barrier_init();
  }
  if (warp == 0) {
    tc::tmem_alloc(&tslot, 64);
    tc::tmem_relinquish();
  }
  for (int e = tid; e < H * 128 / 16; e += 128) reinterpret_cast<uint4*>(B)[e] = __ldg(w1ts + e);
  const float* w2 = theta + H * in + H * HA;
  float e0 = 0.0f, e1 = 0.0f, e2 = 0.0f;
  if (live) {
    e0 = d3[j], e1 = d3[(long)cols + j], e2 = d3[2L * cols + j];
    d3f[j] = __float2bfloat16_rn(e0);
    d3f[(long)ld + j] = __float2bfloat16_rn(e1);
    d3f[2L * ld + j] = __float2bfloat16_rn(e2);
  }
  float hv[HA];  // every h2 load of this sample issued before any store
#pragma unroll
  for (int k = 0; k < HA; ++k) hv[k] = live ? h2[(long)k * cols + j] : 0.0f;
  uint32_t packed[H / 2];
#pragma unroll
  for (int k = 0; k < HA; ++k) {
    const float acc = w2[k] * e0 + w2[HA + k] * e1 + w2[2 * HA + k] * e2;
    const float a = hv[k];
    const float v = acc * (1.0f - a * a);
    if (live) {
      if (write_f32) d2[(long)k * cols + j] = v;
      h2b[(long)k * ld + j] = __float2bfloat16_rn(a);  // the weight-gradient operand of layer 2
    }
    if (k < H) {
      const bf16 vb = __float2bfloat16_rn(v);
      if (live) d2f[(long)k * ld + j] = vb;
      const uint32_t bits = *reinterpret_cast<const uint16_t*>(&vb);
      packed[k >> 1] = (k & 1) ? (packed[k >> 1] | (bits << 16)) : bits;
    }
  }
#pragma unroll
  for (int q = 0; q < 8; ++q)
    *reinterpret_cast<uint4*>(A + tid * 128 + ((q ^ (tid & 7)) << 4)) =
        make_uint4(packed[4 * q], packed[4 * q + 1], packed[4 * q + 2], packed[4 * q + 3]);
  tc::fence_proxy_async_smem();
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = tslot;
  if (tid == 0) {
    const uint32_t a = tc::smem_u32(A), b = tc::smem_u32(B), idesc = tc::idesc_bf16(128, H);
#pragma unroll
    for (int k = 0; k < 4; ++k)
      tc::mma_bf16(tmem, tc::sdesc_sw128(a + 32 * k), tc::sdesc_sw128(b + 32 * k), idesc, k ? 1u : 0u);
    tc::mma_commit(&done);
  }
  bool ok = tc::mbar_wait(&done, 0);
  tc::tc_fence_after();
  float acc[H];
  const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll
  for (int q = 0; q < 4; ++q) tc::tmem_ld16(trow + 16 * q, acc + 16 * q);
  tc::tmem_wait_ld();
  if (live) {
#pragma unroll
    for (int k0 = 0; k0 < H; k0 += 32) {  // 32 loads of h1 in flight, then their stores
      float hh[32];
#pragma unroll
      for (int k = 0; k < 32; ++k) hh[k] = h1[(long)(k0 + k) * cols + j];
#pragma unroll
      for (int k = 0; k < 32; ++k) {
        const float g = acc[k0 + k] * (1.0f - hh[k] * hh[k]);
        if (write_f32) d1[(long)(k0 + k) * cols + j] = g;
        d1f[(long)(k0 + k) * ld + j] = __float2bfloat16_rn(g);
        h1b[(long)(k0 + k) * ld + j] = __float2bfloat16_rn(hh[k]);  // the weight-gradient operand of layer 1
      }
    }
    if (write_f32) d1[(long)H * cols + j] = 0.0f;
    h1b[(long)H * ld + j] = __float2bfloat16_rn(h1[(long)H * cols + j]);
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 64);
  if (!ok) atomicExch(err, 1);
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
  bf16* w1ts = nullptr;  // swizzled W1^T image for k_dgrad_tc
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
      (rc = walloc(&w->w1ts, (size_t)H * H)) ||
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
  for (bf16* p : {w->xb, w->h1b, w->h2b, w->d2f, w->d3f, w->d1f, w->w1ts}) cudaFree(p);
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
  k_pack_w1ts<<<(H * H + 255) / 256, 256, 0, st>>>(theta, w->in, w->w1ts);
  BW_CHECK(cudaGetLastError());
  return 0;
}

int backward_tc(BackwardWork* w, const float* theta, const float* x, const float* h1, const float* h2,
                const float* d3, float* d2, float* d1, float* grad, int* err, cudaStream_t st,
                const CUtensorMap* xb_map, bool dgrads_f32) {
  const int in = w->in, cols = w->cols, ld = w->ld;
  const unsigned gx = (unsigned)((cols + 1023) / 1024);
  if (!xb_map) k_rows_bf16<<<dim3(gx, in), 256, 0, st>>>(x, in, cols, w->xb, ld);
  // the BF16 copies of h1 and h2 are written by k_dgrad_tc, which reads them anyway
  k_dgrad_tc<<<(cols + 127) / 128, 128, 0, st>>>(in, theta, reinterpret_cast<const uint4*>(w->w1ts), d3, h1, h2, d2,
                                                 d1, cols, w->d1f, w->d2f, w->d3f, w->h1b, w->h2b, ld, err,
                                                 dgrads_f32 ? 1 : 0);
  BW_CHECK(cudaGetLastError());
  int rc;
  if ((rc = wgrad<64>(w, xb_map ? *xb_map : w->txb, w->td1f, in, H, in, grad, in, err, st))) return rc;
  if ((rc = wgrad<64>(w, w->th1b, w->td2f, HA, H, HA, grad + H * in, HA, err, st))) return rc;
  if ((rc = wgrad<16>(w, w->th2b, w->td3f, HA, OUT, HA, grad + H * in + H * HA, HA, err, st))) return rc;
  return 0;
}

}  // namespace racer
