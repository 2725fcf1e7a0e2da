// Learned lidar surrogate: a per-track MLP from the lidar's ray frame to all
// beam ranges, trained on the GPU against the exact sphere tracer. Two
// output frames:
//
// Car frame (racer_surrogate_create): one output per beam.
//   inputs  f = encode(x', y', z, sin h, cos h, layer): the frame itself, a
//           constant 1 and fixed Fourier features (k_features), 64 values;
//           (x, y, z) is the lidar origin, x', y' scaled to [-1, 1] over the map
//   h1 = tanh(W1 f)            W1 [H, 64] (the constant input is its bias)
//   h2 = tanh(W2 h1 + b2)      W2 [H, H]
//   h3 = tanh(W3 h2 + b3)      W3 [H, H]
//   y  = W4 h3 + b4            W4 [beams, H]; y = range / RANGE per beam
//
// World frame (racer_surrogate_create_frame, frame 1): the same three tanh
// layers predict the range profile around the lidar origin at K = 4 (beams -
// 1) / 3 fixed world angles 2 pi k / K, the beam spacing, so a full circle
// holds K of them; beam b of a car with heading h reads world sample
// (k0 + b) mod K, k0 the integer part of (h - FOV / 2) K / (2 pi). The ray's
// direction depends on the world angle alone (the body plane's tilt is the
// surface gradient along that angle), so the network no longer has to learn
// the rotation by the heading; the fractional part of that angle (the phase)
// is an input. The position enters through trainable feature grids per layer
// (five resolutions from 20 cells down to 1.25 cells, eight features per
// vertex, bilinear; a dense version of the multiresolution grids of Mueller
// et al., SIGGRAPH 2022) beside a few fixed Fourier features:
//   f = [grid features (40), x', y', z, layer 0, layer 1, 1,
//        sin/cos(2^k pi x'), sin/cos(2^k pi y') for k < 4, sin/cos(2 pi phase)]
//   y  = W4 h3 + b4            W4 [K, H]: the world profile
// Training backpropagates into the grids through dL/df = W1^T dL/dh1 (one
// more GEMM) and a bilinear scatter; the grids take Adam at a higher rate.
//
// Car frame with feature grids (frame 2): the car frame's outputs (one per
// beam) from the same feature grids at the origin beside the frame itself,
// heading harmonics up to 5 and two Fourier octaves of x and y
// (k_features_cargrid); trained and served like the car frame, the grids
// like the world frame's.
// Inference writes the clamped world profile as FP16 rows per car and a
// gather kernel turns them into the beam rows of obs.
//
// Activations are sample-major BF16 for the forward GEMMs and also written
// feature-major (batch contiguous) for the weight-gradient GEMMs; every GEMM
// is the generic tcgen05 kernel (BF16 operands by TMA, FP32 accumulation in
// TMEM) with an epilogue that applies tanh/bias, the loss gradient, the tanh
// derivative or the split-K partial store. Master weights and Adam are FP32.
//
// Training poses are uniform over the drivable cells (clearance > 0) of every
// layer with uniform heading; their labels come from the exact tracer
// (k_pose_frames + k_lidar) batch by batch. Training walks the pose set in
// order, epoch after epoch, so each batch's labels are kept after their first
// tracing (label cache, FP32, up to 32 GB) and copied back in later epochs: the
// same bits without tracing the same poses again.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/racer.h"
#include "common.cuh"
#include "gemm_epi.cuh"
#include "gemm_tc.cuh"
#include "surrogate_fused.cuh"
#include "kernels.h"
#include "objects.h"
#include "philox.h"
#include "tma.h"

using bf16 = __nv_bfloat16;

namespace racer {
namespace {

constexpr int NIN = 64;  // encoded inputs (see k_features)
// World frame: feature grids of GRID_LEVELS resolutions (GRID_CELLS0 cells,
// halving), GRID_F features per vertex; the grids' Adam rate is GRID_LR_SCALE
// times the network's, with beta2 0.99 and epsilon 1e-15.
constexpr int GRID_LEVELS = 5, GRID_F = 8;
constexpr float GRID_CELLS0 = 20.0f, GRID_LR_SCALE = 3.0f;

struct Norm {
  float xc, inv_xs, yc, inv_ys;
};

// The world frame's feature grids: level l has gy[l] x gx[l] vertices per
// layer, spaced r = GRID_CELLS0 / 2^l cells from the map's corner (x0, y0),
// GRID_F floats per vertex, at offset off[l] of the grid block.
struct GridGeom {
  int gx[GRID_LEVELS], gy[GRID_LEVELS];
  long off[GRID_LEVELS];
  float inv_r[GRID_LEVELS];
  float x0, y0;
};

// Bilinear cell of level l at (ox, oy) on `layer`: first corner's offset and
// the weights' fractions (points off the grid clamp to its edge).
__device__ __forceinline__ long grid_cell(const GridGeom& g, int l, float ox, float oy, int layer, float* fu,
                                          float* fv) {
  const float u = fminf(fmaxf((ox - g.x0) * g.inv_r[l], 0.0f), (float)(g.gx[l] - 2));
  const float v = fminf(fmaxf((oy - g.y0) * g.inv_r[l], 0.0f), (float)(g.gy[l] - 2));
  const int iu = min((int)u, g.gx[l] - 3), iv = min((int)v, g.gy[l] - 3);
  *fu = u - (float)iu;
  *fv = v - (float)iv;
  return g.off[l] + (((long)layer * g.gy[l] + iv) * g.gx[l] + iu) * GRID_F;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// H = tanh(v + bias) -> sample-major hs [M, lds] and feature-major hf [N, ldf] (either may be null).
struct EpiTanhOut {
  bf16* hs;
  int lds;
  bf16* hf;
  int ldf;
  const float* bias;
  int M, N;
  __device__ void operator()(int m, int n, const float* v, int z) const {
    if (m >= M) return;
    float h[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) h[j] = (n + j < N) ? tc::tanh_fast(v[j] + (bias ? bias[n + j] : 0.0f)) : 0.0f;
    if (hs && n < N) {  // N is a multiple of 16: a chunk is wholly inside or outside
      uint4 a = make_uint4(tc::pack_bf16(h[0], h[1]), tc::pack_bf16(h[2], h[3]), tc::pack_bf16(h[4], h[5]),
                           tc::pack_bf16(h[6], h[7]));
      uint4 b = make_uint4(tc::pack_bf16(h[8], h[9]), tc::pack_bf16(h[10], h[11]), tc::pack_bf16(h[12], h[13]),
                           tc::pack_bf16(h[14], h[15]));
      uint4* dst = reinterpret_cast<uint4*>(hs + (long)m * lds + n);
      dst[0] = a;
      dst[1] = b;
    }
    if (hf) {
#pragma unroll
      for (int j = 0; j < 16; ++j)
        if (n + j < N) hf[(long)(n + j) * ldf + m] = __float2bfloat16_rn(h[j]);
    }
  }
};

// Output layer in training: y = v + b4, e = y - target, g = scale * e (MSE gradient).
// Writes g sample-major [M, ldgs] and feature-major [npad rows, ldgf] (zero past N),
// accumulates the bias gradient and the sums of e^2 and |e|.
struct EpiLoss {
  const float* target;  // [N, ldt] feature-major
  int ldt;
  const float* bias;
  int M, N;
  float scale;
  bf16* gs;
  int ldgs;
  bf16* gf;
  int ldgf;
  float* dbias;
  double* sums;
  int npad;     // columns stored (a multiple of 16; past N they are zero)
  float huber;  // > 0: Huber loss with this threshold (range units), its gradient e clamped to +-huber
  __device__ void operator()(int m, int n, const float* v, int z) const {
    const bool row = m < M;
    float g[16], se = 0.0f, ae = 0.0f;
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      g[j] = 0.0f;
      if (row && n + j < N) {
        float e = (v[j] + bias[n + j]) - target[(long)(n + j) * ldt + m];
        se += e * e;
        ae += fabsf(e);
        g[j] = scale * (huber > 0.0f ? fminf(fmaxf(e, -huber), huber) : e);
      }
    }
    if (row && n < npad) {
      uint4 a = make_uint4(tc::pack_bf16(g[0], g[1]), tc::pack_bf16(g[2], g[3]), tc::pack_bf16(g[4], g[5]),
                           tc::pack_bf16(g[6], g[7]));
      uint4 b = make_uint4(tc::pack_bf16(g[8], g[9]), tc::pack_bf16(g[10], g[11]), tc::pack_bf16(g[12], g[13]),
                           tc::pack_bf16(g[14], g[15]));
      uint4* dst = reinterpret_cast<uint4*>(gs + (long)m * ldgs + n);
      dst[0] = a;
      dst[1] = b;
#pragma unroll
      for (int j = 0; j < 16; ++j) gf[(long)(n + j) * ldgf + m] = __float2bfloat16_rn(g[j]);
    }
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      float s = warp_sum(g[j]);
      if ((threadIdx.x & 31) == 0 && n + j < N) atomicAdd(dbias + n + j, s);
    }
    se = warp_sum(se);
    ae = warp_sum(ae);
    if ((threadIdx.x & 31) == 0) {
      atomicAdd(sums, (double)se);
      atomicAdd(sums + 1, (double)ae);
    }
  }
};

// Back through tanh: g = v * (1 - h^2) with h from hs [M, ldh]; writes gs (optional) and gf,
// accumulates the bias gradient (optional).
struct EpiDTanh {
  const bf16* hs;
  int ldh;
  bf16* gs;
  int ldgs;
  bf16* gf;
  int ldgf;
  float* dbias;
  int M, N;
  __device__ void operator()(int m, int n, const float* v, int z) const {
    const bool row = m < M;
    float g[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      g[j] = 0.0f;
      if (row && n + j < N) {
        float h = __bfloat162float(hs[(long)m * ldh + n + j]);
        g[j] = v[j] * (1.0f - h * h);
      }
    }
    if (row && n < N) {
      if (gs) {
        uint4 a = make_uint4(tc::pack_bf16(g[0], g[1]), tc::pack_bf16(g[2], g[3]), tc::pack_bf16(g[4], g[5]),
                             tc::pack_bf16(g[6], g[7]));
        uint4 b = make_uint4(tc::pack_bf16(g[8], g[9]), tc::pack_bf16(g[10], g[11]), tc::pack_bf16(g[12], g[13]),
                             tc::pack_bf16(g[14], g[15]));
        uint4* dst = reinterpret_cast<uint4*>(gs + (long)m * ldgs + n);
        dst[0] = a;
        dst[1] = b;
      }
#pragma unroll
      for (int j = 0; j < 16; ++j)
        if (n + j < N) gf[(long)(n + j) * ldgf + m] = __float2bfloat16_rn(g[j]);
    }
    if (dbias) {
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        float s = warp_sum(g[j]);
        if ((threadIdx.x & 31) == 0 && n + j < N) atomicAdd(dbias + n + j, s);
      }
    }
  }
};

// Inference output: out[(n) * ldo + m] = clamp(v + b4, 0, 1) (feature-major, the obs rows of the
// beams), and the smallest predicted range of each row into minr (as ordered uint bits).
struct EpiInfer {
  float* out;
  int ldo;
  const float* bias;
  int M, N;
  unsigned* minr;
  __device__ void operator()(int m, int n, const float* v, int z) const {
    if (m >= M) return;
    float lo = 1.0f;
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      if (n + j < N) {
        const float y = __saturatef(v[j] + bias[n + j]);  // as the fused kernel: [0, 1], NaN to 0
        out[(long)(n + j) * ldo + m] = y;
        lo = fminf(lo, y);
      }
    }
    if (minr) atomicMin(minr + m, __float_as_uint(lo));
  }
};

// World frame, training: y[m * ldy + n] = v + b4 for n < N (unclamped, FP32), 0 past N.
struct EpiWorldTrain {
  float* y;
  int ldy;
  const float* bias;
  int M, N;
  __device__ void operator()(int m, int n, const float* v, int z) const {
    if (m >= M || n >= ldy) return;  // n is a multiple of 16, ldy of 64
    float4* dst = reinterpret_cast<float4*>(y + (long)m * ldy + n);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      float t[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int o = n + 4 * q + j;
        t[j] = o < N ? v[4 * q + j] + bias[o] : 0.0f;
      }
      dst[q] = make_float4(t[0], t[1], t[2], t[3]);
    }
  }
};

// World frame, layered inference: the world profile of row m into out [M, ldo]
// (FP16) and the row's smallest range in its field of view into minr.
struct EpiWorldInfer {
  __half* out;
  int ldo;
  const float* bias;
  int M, N;  // N = K world samples
  const float4* ray;  // the rows' ray frames [2, M]
  int beams;
  unsigned* minr;
  __device__ void operator()(int m, int n, const float* v, int z) const {
    if (m >= M || n >= ldo) return;  // n is a multiple of 16, ldo of 64
    float ph;
    const float4 r0 = ray[m], r1 = ray[M + m];
    const int k0 = world_phase(r1.x, r0.w, N, &ph);
    float bb[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) bb[j] = n + j < N ? bias[n + j] : 0.0f;
    const float lo = world_store16(v, bb, n, N, k0, beams, out + (long)m * ldo, 1.0f);
    if (minr) atomicMin(minr + m, __float_as_uint(lo));
  }
};

// ray frames [2, count] -> encoded inputs, sample-major x [count, 64] and feature-major xf [64, count]:
//   0..7    x', y', z, sin h, cos h, [layer 0], [layer 1], 1
//   8..47   sin/cos(2^k pi x'), sin/cos(2^k pi y') for k = 0..9  (Fourier features,
//           Tancik et al. 2020: a plain MLP on raw coordinates fits the
//           high-frequency range field far too slowly)
//   48..55  sin/cos(j h) for j = 2..5
//   56..59  sin/cos(pi z), sin/cos(2 pi z)
//   60..63  0
__device__ __forceinline__ void encode(float xn, float yn, float z, float sh, float ch, float layer, float* f) {
  f[0] = xn;
  f[1] = yn;
  f[2] = z;
  f[3] = sh;
  f[4] = ch;
  f[5] = layer == 0.0f ? 1.0f : 0.0f;
  f[6] = layer == 1.0f ? 1.0f : 0.0f;
  f[7] = 1.0f;
  float scale = 1.0f;
#pragma unroll
  for (int k = 0; k < 10; ++k) {
    sincospif(scale * xn, &f[8 + 4 * k], &f[9 + 4 * k]);
    sincospif(scale * yn, &f[10 + 4 * k], &f[11 + 4 * k]);
    scale *= 2.0f;
  }
  const float h = atan2f(sh, ch);
#pragma unroll
  for (int j = 2; j <= 5; ++j) sincosf((float)j * h, &f[48 + 2 * (j - 2)], &f[49 + 2 * (j - 2)]);
  sincospif(z, &f[56], &f[57]);
  sincospif(2.0f * z, &f[58], &f[59]);
  f[60] = f[61] = f[62] = f[63] = 0.0f;
}

__global__ void k_features(const float4* __restrict__ ray, int count, Norm nm, bf16* x, bf16* xf) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float4 r0 = ray[i], r1 = ray[count + i];
  float f[NIN];
  encode((r0.x - nm.xc) * nm.inv_xs, (r0.y - nm.yc) * nm.inv_ys, r0.z, r1.x, r0.w, r1.w, f);
  uint4* row = reinterpret_cast<uint4*>(x + (long)i * NIN);
#pragma unroll
  for (int q = 0; q < NIN / 8; ++q)
    row[q] = make_uint4(tc::pack_bf16(f[8 * q], f[8 * q + 1]), tc::pack_bf16(f[8 * q + 2], f[8 * q + 3]),
                        tc::pack_bf16(f[8 * q + 4], f[8 * q + 5]), tc::pack_bf16(f[8 * q + 6], f[8 * q + 7]));
  if (xf)
#pragma unroll
    for (int k = 0; k < NIN; ++k) xf[(long)k * count + i] = __float2bfloat16_rn(f[k]);
}

// The feature grids of `layer` at (ox, oy), level by level, into f[0 .. 39].
__device__ __forceinline__ void grid_features(const GridGeom& gg, const float* __restrict__ grid, float ox, float oy,
                                              int layer, float* f) {
#pragma unroll
  for (int l = 0; l < GRID_LEVELS; ++l) {
    float fu, fv;
    const long c = grid_cell(gg, l, ox, oy, layer, &fu, &fv);
    const long dy = (long)gg.gx[l] * GRID_F;
    const float w00 = (1.0f - fu) * (1.0f - fv), w10 = fu * (1.0f - fv), w01 = (1.0f - fu) * fv, w11 = fu * fv;
#pragma unroll
    for (int q = 0; q < GRID_F / 4; ++q) {
      const float4 a = __ldg(reinterpret_cast<const float4*>(grid + c) + q);
      const float4 b = __ldg(reinterpret_cast<const float4*>(grid + c + GRID_F) + q);
      const float4 d = __ldg(reinterpret_cast<const float4*>(grid + c + dy) + q);
      const float4 e = __ldg(reinterpret_cast<const float4*>(grid + c + dy + GRID_F) + q);
      float* o = f + GRID_F * l + 4 * q;
      o[0] = w00 * a.x + w10 * b.x + w01 * d.x + w11 * e.x;
      o[1] = w00 * a.y + w10 * b.y + w01 * d.y + w11 * e.y;
      o[2] = w00 * a.z + w10 * b.z + w01 * d.z + w11 * e.z;
      o[3] = w00 * a.w + w10 * b.w + w01 * d.w + w11 * e.w;
    }
  }
}

__device__ __forceinline__ void store_inputs(const float* f, int i, int count, bf16* x, bf16* xf) {
  uint4* row = reinterpret_cast<uint4*>(x + (long)i * NIN);
#pragma unroll
  for (int q = 0; q < NIN / 8; ++q)
    row[q] = make_uint4(tc::pack_bf16(f[8 * q], f[8 * q + 1]), tc::pack_bf16(f[8 * q + 2], f[8 * q + 3]),
                        tc::pack_bf16(f[8 * q + 4], f[8 * q + 5]), tc::pack_bf16(f[8 * q + 6], f[8 * q + 7]));
  if (xf)
#pragma unroll
    for (int k = 0; k < NIN; ++k) xf[(long)k * count + i] = __float2bfloat16_rn(f[k]);
}

// Car frame with feature grids (frame 2): ray frames [2, count] -> encoded inputs:
//   0..39   the feature grids of the origin's layer at (x, y), level by level
//   40..47  x', y', z, sin h, cos h, [layer 0], [layer 1], 1
//   48..55  sin/cos(j h) for j = 2..5
//   56..63  sin/cos(2^k pi x'), sin/cos(2^k pi y') for k = 0, 1
__global__ void k_features_cargrid(const float4* __restrict__ ray, int count, Norm nm, GridGeom gg,
                                   const float* __restrict__ grid, bf16* x, bf16* xf) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float4 r0 = ray[i], r1 = ray[count + i];
  const int layer = r1.w == 1.0f ? 1 : 0;
  float f[NIN];
  grid_features(gg, grid, r0.x, r0.y, layer, f);
  const float xn = (r0.x - nm.xc) * nm.inv_xs, yn = (r0.y - nm.yc) * nm.inv_ys;
  f[40] = xn;
  f[41] = yn;
  f[42] = r0.z;
  f[43] = r1.x;
  f[44] = r0.w;
  f[45] = layer == 0 ? 1.0f : 0.0f;
  f[46] = layer == 1 ? 1.0f : 0.0f;
  f[47] = 1.0f;
  const float h = atan2f(r1.x, r0.w);
#pragma unroll
  for (int j = 2; j <= 5; ++j) sincosf((float)j * h, &f[48 + 2 * (j - 2)], &f[49 + 2 * (j - 2)]);
  sincospif(xn, &f[56], &f[57]);
  sincospif(yn, &f[58], &f[59]);
  sincospif(2.0f * xn, &f[60], &f[61]);
  sincospif(2.0f * yn, &f[62], &f[63]);
  store_inputs(f, i, count, x, xf);
}

// World frame: ray frames [2, count] -> encoded inputs (see the top of this file):
//   0..39   the feature grids of the origin's layer at (x, y), level by level
//   40..45  x', y', z, [layer 0], [layer 1], 1
//   46..61  sin/cos(2^k pi x'), sin/cos(2^k pi y') for k = 0..3
//   62, 63  sin/cos(2 pi phase)
__global__ void k_features_world(const float4* __restrict__ ray, int count, Norm nm, GridGeom gg,
                                 const float* __restrict__ grid, int K, bf16* x, bf16* xf) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float4 r0 = ray[i], r1 = ray[count + i];
  const int layer = r1.w == 1.0f ? 1 : 0;
  float f[NIN];
  grid_features(gg, grid, r0.x, r0.y, layer, f);
  const float xn = (r0.x - nm.xc) * nm.inv_xs, yn = (r0.y - nm.yc) * nm.inv_ys;
  f[40] = xn;
  f[41] = yn;
  f[42] = r0.z;
  f[43] = layer == 0 ? 1.0f : 0.0f;
  f[44] = layer == 1 ? 1.0f : 0.0f;
  f[45] = 1.0f;
  float scale = 1.0f;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    sincospif(scale * xn, &f[46 + 4 * k], &f[47 + 4 * k]);
    sincospif(scale * yn, &f[48 + 4 * k], &f[49 + 4 * k]);
    scale *= 2.0f;
  }
  float phase;
  world_phase(r1.x, r0.w, K, &phase);
  sincospif(2.0f * phase, &f[62], &f[63]);
  store_inputs(f, i, count, x, xf);
}

// World frame, training loss: one thread per sample m and 64 world samples
// (blockIdx.y: columns 64 y .. 64 y + 63). Beam b's prediction is
// y[m][(k0 + b) mod K] (y from EpiWorldTrain, ldy = npad); the loss gradient
// (scale times the error, clamped to +-huber when huber > 0) goes to that
// world sample, and every world sample no beam reads gets 0. Writes the
// gradient sample-major gs [B, npad] and feature-major gf [npad, B] (BF16),
// sums the output bias gradient and the sums of e^2 and |e| (range units).
__global__ void __launch_bounds__(128) k_world_loss(const float* __restrict__ y, const float* __restrict__ target,
                                                    const float4* __restrict__ ray, int B, int beams, int K, int npad,
                                                    float scale, float huber, bf16* gs, bf16* gf, float* dbias,
                                                    double* sums) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  const bool row = m < B;
  int k0 = 0;
  if (row) {
    float ph;
    k0 = world_phase(ray[B + m].x, ray[m].w, K, &ph);
  }
  float se = 0.0f, ae = 0.0f;
  const int c0 = 64 * blockIdx.y;
  for (int w0 = c0; w0 < c0 + 64 && w0 < npad; w0 += 8) {
    float g[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int w = w0 + j;
      g[j] = 0.0f;
      int b = w - k0;
      if (b < 0) b += K;
      if (row && w < K && b < beams) {
        const float e = y[(long)m * npad + w] - target[(long)b * B + m];
        se += e * e;
        ae += fabsf(e);
        g[j] = scale * (huber > 0.0f ? fminf(fmaxf(e, -huber), huber) : e);
      }
    }
    if (row) {
      *reinterpret_cast<uint4*>(gs + (long)m * npad + w0) =
          make_uint4(tc::pack_bf16(g[0], g[1]), tc::pack_bf16(g[2], g[3]), tc::pack_bf16(g[4], g[5]),
                     tc::pack_bf16(g[6], g[7]));
#pragma unroll
      for (int j = 0; j < 8; ++j) gf[(long)(w0 + j) * B + m] = __float2bfloat16_rn(g[j]);
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const float t = warp_sum(g[j]);
      if ((threadIdx.x & 31) == 0 && w0 + j < K) atomicAdd(dbias + w0 + j, t);
    }
  }
  se = warp_sum(se);
  ae = warp_sum(ae);
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(sums, (double)se);
    atomicAdd(sums + 1, (double)ae);
  }
}

// World frame: gradient of the feature grids from dL/df (dx [B, 64], FP32):
// each sample's bilinear weights scatter its first 40 input gradients onto the
// four corners of its cell at every level (16-byte atomic adds).
__global__ void k_grid_grad(const float4* __restrict__ ray, int B, GridGeom gg, const float* __restrict__ dx,
                            float* ggrad) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= B) return;
  const float4 r0 = ray[m], r1 = ray[B + m];
  const int layer = r1.w == 1.0f ? 1 : 0;
#pragma unroll
  for (int l = 0; l < GRID_LEVELS; ++l) {
    float fu, fv;
    const long c = grid_cell(gg, l, r0.x, r0.y, layer, &fu, &fv);
    const long dy = (long)gg.gx[l] * GRID_F;
    const float w[4] = {(1.0f - fu) * (1.0f - fv), fu * (1.0f - fv), (1.0f - fu) * fv, fu * fv};
    const long corner[4] = {c, c + GRID_F, c + dy, c + dy + GRID_F};
#pragma unroll
    for (int q = 0; q < GRID_F / 4; ++q) {
      const float4 d = *reinterpret_cast<const float4*>(dx + (long)m * NIN + GRID_F * l + 4 * q);
#pragma unroll
      for (int k = 0; k < 4; ++k)
        atomicAdd(reinterpret_cast<float4*>(ggrad + corner[k]) + q,
                  make_float4(w[k] * d.x, w[k] * d.y, w[k] * d.z, w[k] * d.w));
    }
  }
}

// World frame, inference: beam rows pred[b * ldp + m] (FP32, the obs layout)
// from the world profiles wout [n, ldw] (FP16): beam b of car m is
// wout[m][(k0(m) + b) mod K]. A block stages, for each of its 16 cars, the
// 16-byte pieces of the row that cover the car's window k0 .. k0 + beams - 1
// (wrapping at K, a multiple of 8) in shared memory, unwrapped (coalesced
// loads along each row), then each warp writes beam rows of those 16 cars, two
// rows per store instruction (64 contiguous bytes each). The window's
// elements are the only ones read; the rest of a piece may hold anything
// (world_store16 skips groups outside every window). Small blocks (35 KB of
// shared memory at 1081 beams) let several per SM overlap loads and stores.
constexpr int WR_CARS = 16, WR_THREADS = 256;
// Words (2 halves) per staged row: the window plus a partial piece at each end,
// rounded to an odd count so that rows start in different banks.
__host__ __device__ constexpr int world_rotate_words(int beams) { return (((beams + 15) / 8 * 8) / 2) | 1; }

__global__ void __launch_bounds__(WR_THREADS) k_world_rotate(const __half* __restrict__ wout, int ldw,
                                                             const float4* __restrict__ ray, int n, int beams, int K,
                                                             float* pred, long ldp) {
  extern __shared__ __align__(16) uint8_t wr_smem[];
  uint32_t* rows = reinterpret_cast<uint32_t*>(wr_smem);
  __shared__ int k0s[WR_CARS];
  const int words = world_rotate_words(beams), m0 = blockIdx.x * WR_CARS;
  if (threadIdx.x < WR_CARS) {
    int k0 = -1;  // -1: no car
    const int m = m0 + threadIdx.x;
    if (m < n) {
      float ph;
      k0 = world_phase(ray[n + m].x, ray[m].w, K, &ph);
    }
    k0s[threadIdx.x] = k0;
  }
  __syncthreads();
  const int pieces = (beams + 14) / 8 + 1;  // covers (k0 & 7) + beams halves
  const int kp = K / 8;                     // pieces per row
  for (int i = threadIdx.x; i < WR_CARS * pieces; i += WR_THREADS) {
    const int r = i / pieces, p = i % pieces;
    if (k0s[r] < 0 || 8 * p >= (k0s[r] & 7) + beams) continue;
    int q = (k0s[r] >> 3) + p;
    if (q >= kp) q -= kp;
    const uint4 v = __ldcs(reinterpret_cast<const uint4*>(wout + (long)(m0 + r) * ldw) + q);
    uint32_t* dst = rows + (long)r * words + 4 * p;
    dst[0] = v.x, dst[1] = v.y, dst[2] = v.z, dst[3] = v.w;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, car = lane & 15, m = m0 + car;
  if (k0s[car] < 0) return;
  const __half* mine = reinterpret_cast<const __half*>(rows + (long)car * words) + (k0s[car] & 7);
  for (int b = 2 * (threadIdx.x >> 5) + (lane >> 4); b < beams; b += 2 * (WR_THREADS / 32))
    pred[(long)b * ldp + m] = __half2float(mine[b]);
}

// The world frame's largest beam count (the gather's shared memory: 16 windows of it, 131 KB).
constexpr int WORLD_MAX_BEAMS = 4093;

// The gather kernel's shared-memory limit, once per device.
cudaError_t world_rotate_configure() {
  static unsigned long long configured = 0;
  return once_per_device(&configured, [] {
    return cudaFuncSetAttribute(k_world_rotate, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                WR_CARS * world_rotate_words(WORLD_MAX_BEAMS) * 4);
  });
}

// Each sample's first world sample (racer_surrogate_batch_inputs).
__global__ void k_world_k0(const float4* __restrict__ ray, int B, int K, int* k0) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= B) return;
  float ph;
  k0[m] = world_phase(ray[B + m].x, ray[m].w, K, &ph);
}

// Poses uniform over drivable (cell, layer) pairs, jittered inside the cell, heading uniform.
__global__ void k_sample_poses(const int2* cells, int ncells, int count, uint64_t seed, TrackDev t, float4* poses) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  float u[4];
  philox::uniform4(seed, (uint64_t)i, 7, u);
  int k = min((int)(u[0] * (float)ncells), ncells - 1);
  int2 c = cells[k];
  int ix = c.x % t.nx, iy = c.x / t.nx;
  float x = t.x0 + ((float)ix + u[1] - 0.5f) * t.cell;
  float y = t.y0 + ((float)iy + u[2] - 0.5f) * t.cell;
  float h = (2.0f * u[3] - 1.0f) * PI_F;
  poses[i] = make_float4(x, y, h, (float)c.y);
}

// Sum of split-K partials into a row-major [Mreal, N] gradient block.
__global__ void k_reduce_splits(const float* P, int splits, long mn, int N, int Mreal, float* out) {
  long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long)Mreal * N) return;
  float acc = 0.0f;
  for (int z = 0; z < splits; ++z) acc += P[(long)z * mn + e];
  out[e] = acc;
}

// Parameter block: W1 [H, 64] | W2 [H, H] | b2 | W3 [H, H] | b3 | W4 [nout, H] |
// b4 [nout] | (world frame) the feature grids from g, 8-float aligned.
struct Layout {
  int H, beams, npad;  // npad: nout rounded up to 64
  int world;           // 0: car frame (nout = beams), 1: world frame (nout = K world samples)
  int grid;            // 1: the first 40 inputs are the trainable feature grids (world frame, frame 2)
  int nout;
  long w1, w2, b2, w3, b3, w4, b4, g, total;
};

// theta -> BF16 operand images (row-major and transposed), zero past `nout` rows/cols of W4;
// w1t = W1^T [64, H] (the input-gradient GEMM of the world frame; may be null).
__global__ void k_refresh(const float* __restrict__ th, Layout L, bf16* w1b, bf16* w2b, bf16* w3b, bf16* w4b,
                          bf16* w2t, bf16* w3t, bf16* w4t, bf16* w1t) {
  const int H = L.H;
  const long n1 = (long)H * NIN, n2 = (long)H * H, n4 = (long)L.npad * H;
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < n1 + 2 * n2 + n4;
       e += (long)gridDim.x * blockDim.x) {
    if (e < n1) {
      const bf16 v = __float2bfloat16_rn(th[L.w1 + e]);
      w1b[e] = v;
      if (w1t) w1t[(e % NIN) * H + e / NIN] = v;
    } else if (e < n1 + n2) {
      long f = e - n1;
      int o = (int)(f / H), i = (int)(f % H);
      bf16 v = __float2bfloat16_rn(th[L.w2 + f]);
      w2b[f] = v;
      w2t[(long)i * H + o] = v;
    } else if (e < n1 + 2 * n2) {
      long f = e - n1 - n2;
      int o = (int)(f / H), i = (int)(f % H);
      bf16 v = __float2bfloat16_rn(th[L.w3 + f]);
      w3b[f] = v;
      w3t[(long)i * H + o] = v;
    } else {
      long f = e - n1 - 2 * n2;
      int o = (int)(f / H), i = (int)(f % H);
      bf16 v = __float2bfloat16_rn(o < L.nout ? th[L.w4 + (long)o * H + i] : 0.0f);
      w4b[f] = v;
      w4t[(long)i * L.npad + o] = v;
    }
  }
}

__global__ void k_init_params(float* th, Layout L, uint64_t seed) {
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < L.total; e += (long)gridDim.x * blockDim.x) {
    float z[4];
    philox::normal4(seed, (uint64_t)e, 11, z);
    float v = 0.0f;
    if (e < L.w2) v = z[0] * rsqrtf((float)NIN);
    else if (e < L.b2) v = z[0] * rsqrtf((float)L.H);
    else if (e < L.w3) v = 0.0f;
    else if (e < L.b3) v = z[0] * rsqrtf((float)L.H);
    else if (e < L.w4) v = 0.0f;
    else if (e < L.b4) v = z[0] * rsqrtf((float)L.H) * 0.5f;
    else if (e < L.b4 + L.nout) v = 0.3f;  // output bias: a typical normalised range
    else v = z[0] * 1e-4f;  // feature grids (world frame): small, as for learned grid encodings
    th[e] = v;
  }
}

// Adam (beta1 0.9) over p parameters; c1, c2 the bias corrections 1 - beta^t.
__global__ void k_adam_s(long p, float lr, float beta2, float eps, float c1, float c2, float* th, const float* g,
                         float* m1, float* m2) {
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < p; i += (long)gridDim.x * blockDim.x) {
    float gi = g[i];
    float a = 0.9f * m1[i] + 0.1f * gi;
    float b = beta2 * m2[i] + (1.0f - beta2) * gi * gi;
    m1[i] = a;
    m2[i] = b;
    th[i] -= lr * (a / c1) / (sqrtf(b / c2) + eps);
  }
}

// |pred - exact| statistics over [beams, count] (both feature-major rows of ranges / RANGE):
// sums[0] += sum |e|, sums[1] += sum e^2, max in bits, count of |e| > 5 cm.
// FP32 per-thread partial sums (a few thousand terms each; FP64 arithmetic is
// slow on this GPU), combined in FP64 once per thread.
__device__ __forceinline__ void compare_one(float p, float x, float& a, float& s, float& mx, unsigned& ov) {
  const float e = fabsf(p - x) * RANGE;
  a += e;
  s += e * e;
  mx = fmaxf(mx, e);
  ov += e > 0.05f;
}

// Error statistics of pred against exact (ranges in obs units): sums of |e|
// and e^2, the largest e and the count over 5 cm. 16-byte loads when both
// arrays are 16-byte aligned (unrolled, so several loads are in flight).
__global__ void k_compare(const float* __restrict__ pred, const float* __restrict__ exact, long total, double* sums,
                          unsigned* maxbits, unsigned long long* over) {
  float a = 0.0f, s = 0.0f, mx = 0.0f;
  unsigned ov = 0;
  const long stride = (long)gridDim.x * blockDim.x, i0 = (long)blockIdx.x * blockDim.x + threadIdx.x;
  long tail = 0;
  if ((((uintptr_t)pred | (uintptr_t)exact) & 15) == 0) {
    const long quads = total / 4;
    const float4* p4 = reinterpret_cast<const float4*>(pred);
    const float4* x4 = reinterpret_cast<const float4*>(exact);
#pragma unroll 4
    for (long q = i0; q < quads; q += stride) {
      const float4 p = __ldcs(p4 + q), x = __ldcs(x4 + q);
      compare_one(p.x, x.x, a, s, mx, ov);
      compare_one(p.y, x.y, a, s, mx, ov);
      compare_one(p.z, x.z, a, s, mx, ov);
      compare_one(p.w, x.w, a, s, mx, ov);
    }
    tail = quads * 4;
  }
  for (long i = tail + i0; i < total; i += stride) compare_one(pred[i], exact[i], a, s, mx, ov);
  a = warp_sum(a);
  s = warp_sum(s);
  for (int o = 16; o > 0; o >>= 1) {
    mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    ov += __shfl_xor_sync(0xffffffffu, ov, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(sums, (double)a);
    atomicAdd(sums + 1, (double)s);
    atomicMax(maxbits, __float_as_uint(mx));
    atomicAdd(over, (unsigned long long)ov);
  }
}

}  // namespace
}  // namespace racer

using namespace racer;

struct SurrogateActs {  // activation buffers and tensor maps for one row count M
  int M = 0;
  bf16 *x = nullptr, *xf = nullptr, *h1s = nullptr, *h2s = nullptr, *h3s = nullptr;
  bf16 *h1f = nullptr, *h2f = nullptr, *h3f = nullptr;
  bf16 *g4s = nullptr, *g4f = nullptr, *g3s = nullptr, *g3f = nullptr, *g2s = nullptr, *g2f = nullptr,
       *g1f = nullptr, *g1s = nullptr;
  CUtensorMap tx, th1, th2, th3, tg4s, tg3s, tg2s, tg1s;    // A operands (M rows)
  CUtensorMap tg4f, tg3f, tg2f, tg1f, th3f, th2f, th1f, txf;  // weight-gradient operands (K = M)
};

struct racer_surrogate {
  racer_sim* sim = nullptr;
  Layout L{};
  Norm nm{};
  int batch = 0;
  float huber = 0.0f;  // training loss: 0 = squared error, > 0 = Huber threshold (range / 10 m units)
  int fused = 1;       // rollout inference in one fused kernel (hidden width 512)
  cudaStream_t st = nullptr;
  float *theta = nullptr, *grad = nullptr, *m1 = nullptr, *m2 = nullptr;
  bf16 *w1b = nullptr, *w2b = nullptr, *w3b = nullptr, *w4b = nullptr, *w2t = nullptr, *w3t = nullptr,
       *w4t = nullptr, *w1t = nullptr;
  CUtensorMap tw1, tw2, tw3, tw4, tw2t, tw3t, tw4t, tw1t;  // B operands
  // world frame: grid geometry, world outputs of a training batch (FP32 [batch, npad]), the
  // input gradient (FP32 [batch, 64]), world profiles of a batch and of the sim's cars (FP16)
  GridGeom gg{};
  float* wy = nullptr;
  float* dx = nullptr;
  __half* wbatch = nullptr;
  __half* wout = nullptr;
  int2* cells = nullptr;
  int ncells = 0;
  float4* poses = nullptr;
  int npose = 0;
  float4* ray = nullptr;   // [2, batch]
  float* label = nullptr;  // [4 + beams, batch] (rows 4.. are the exact ranges / RANGE)
  float* lcache = nullptr;   // [npose / batch][beams][batch] labels of the pose set, when cached
  std::vector<uint8_t> lcached;  // per batch of the pose set: its labels are in lcache
  bool use_cache = true;
  float* pred = nullptr;   // [beams, batch]
  float* scratch = nullptr;
  size_t scratch_floats = 0;
  double* sums = nullptr;    // loss sums / compare sums
  unsigned* maxbits = nullptr;
  unsigned long long* over = nullptr;
  int* err = nullptr;
  SurrogateActs train;
  int step = 0;
  // rollout inference for the sim's cars (allocated on first use)
  SurrogateActs infer;
  unsigned* minr = nullptr;  // [n] smallest predicted range per car (uint bits)
  int* list = nullptr;       // [n] fallback cars
  int* list_count = nullptr;
  unsigned* list_units = nullptr;  // unit counter of the fallback lidar
  float* exact = nullptr;    // [4 + beams, n] audit ranges
  double* rsums = nullptr;   // audit sum |e|, sum e^2 (metres)
  unsigned* rmax = nullptr;
  unsigned long long* rcount = nullptr;  // [0] beams over 5 cm, [1] fallback cars
  double audited_beams = 0, car_steps = 0;
  // spot check between audits (racer_surrogate_set_spot_check): every spot_stride-th beam traced
  // exactly, cars off by more than spot_tol (range / RANGE units) fall back to the exact tracer
  int spot_stride = 0;
  float spot_tol = 0.025f;
};

namespace {

template <typename T>
int salloc(T** p, size_t count) {
  RACER_TRY(cudaMalloc((void**)p, count * sizeof(T) + 64));
  RACER_TRY(cudaMemset(*p, 0, count * sizeof(T) + 64));
  return 0;
}

int make_acts(racer_surrogate* s, SurrogateActs* a, int M, bool training) {
  const int H = s->L.H, NP = s->L.npad;
  a->M = M;
  int rc = 0;
  if ((rc = salloc(&a->x, (size_t)M * NIN)) || (rc = salloc(&a->h1s, (size_t)M * H)) ||
      (rc = salloc(&a->h2s, (size_t)M * H)) || (rc = salloc(&a->h3s, (size_t)M * H)))
    return rc;
  if ((rc = make_tmap_bf16(&a->tx, a->x, M, NIN, NIN, 128)) || (rc = make_tmap_bf16(&a->th1, a->h1s, M, H, H, 128)) ||
      (rc = make_tmap_bf16(&a->th2, a->h2s, M, H, H, 128)))
    return rc;
  if ((rc = make_tmap_bf16(&a->th3, a->h3s, M, H, H, 128))) return rc;
  if (!training) return 0;
  if ((M % 8) != 0) {
    racer_host::set_error("surrogate: the training batch must be a multiple of 8");
    return 1;
  }
  if ((rc = salloc(&a->xf, (size_t)NIN * M)) || (rc = salloc(&a->h1f, (size_t)H * M)) ||
      (rc = salloc(&a->h2f, (size_t)H * M)) || (rc = salloc(&a->h3f, (size_t)H * M)) ||
      (rc = salloc(&a->g4s, (size_t)M * NP)) || (rc = salloc(&a->g4f, (size_t)NP * M)) ||
      (rc = salloc(&a->g3s, (size_t)M * H)) || (rc = salloc(&a->g3f, (size_t)H * M)) ||
      (rc = salloc(&a->g2s, (size_t)M * H)) || (rc = salloc(&a->g2f, (size_t)H * M)) ||
      (rc = salloc(&a->g1f, (size_t)H * M)) || (rc = salloc(&a->g1s, (size_t)M * H)))
    return rc;
  if ((rc = make_tmap_bf16(&a->tg4s, a->g4s, M, NP, NP, 128)) || (rc = make_tmap_bf16(&a->tg3s, a->g3s, M, H, H, 128)) ||
      (rc = make_tmap_bf16(&a->tg2s, a->g2s, M, H, H, 128)) || (rc = make_tmap_bf16(&a->tg1s, a->g1s, M, H, H, 128)) ||
      (rc = make_tmap_bf16(&a->tg4f, a->g4f, NP, M, M, 128)) ||
      (rc = make_tmap_bf16(&a->tg3f, a->g3f, H, M, M, 128)) || (rc = make_tmap_bf16(&a->tg2f, a->g2f, H, M, M, 128)) ||
      (rc = make_tmap_bf16(&a->tg1f, a->g1f, H, M, M, 128)) || (rc = make_tmap_bf16(&a->th3f, a->h3f, H, M, M, 256)) ||
      (rc = make_tmap_bf16(&a->th2f, a->h2f, H, M, M, 256)) || (rc = make_tmap_bf16(&a->th1f, a->h1f, H, M, M, 256)) ||
      (rc = make_tmap_bf16(&a->txf, a->xf, NIN, M, M, 64)))
    return rc;
  return 0;
}

void free_acts(SurrogateActs* a) {
  for (bf16* p : {a->x, a->xf, a->h1s, a->h2s, a->h3s, a->h1f, a->h2f, a->h3f, a->g4s, a->g4f, a->g3s, a->g3f, a->g2s,
                  a->g2f, a->g1f, a->g1s})
    cudaFree(p);
}

#define SURR_CHECK(expr)                                                                  \
  do {                                                                                    \
    cudaError_t e_ = (expr);                                                              \
    if (e_ != cudaSuccess) {                                                              \
      racer_host::set_error(std::string("surrogate: ") + #expr + ": " + cudaGetErrorString(e_)); \
      return 2;                                                                           \
    }                                                                                     \
  } while (0)

// Forward of M rows already featurised in a->x; the last layer uses `out` (inference).
int forward(racer_surrogate* s, SurrogateActs* a, bool training, const EpiInfer* out) {
  const int H = s->L.H, M = a->M;
  const float* th = s->theta;
  cudaStream_t st = s->st;
  SURR_CHECK(gemm_launch<256>(a->tx, s->tw1, M, H, 1, 1, EpiTanhOut{a->h1s, H, training ? a->h1f : nullptr, M, nullptr, M, H},
                              s->err, st));
  SURR_CHECK(gemm_launch<256>(a->th1, s->tw2, M, H, H / 64, 1,
                              EpiTanhOut{a->h2s, H, training ? a->h2f : nullptr, M, th + s->L.b2, M, H}, s->err, st));
  SURR_CHECK(gemm_launch<256>(a->th2, s->tw3, M, H, H / 64, 1,
                              EpiTanhOut{a->h3s, H, training ? a->h3f : nullptr, M, th + s->L.b3, M, H}, s->err, st));
  if (out) SURR_CHECK(gemm_launch<256>(a->th3, s->tw4, M, s->L.beams, H / 64, 1, *out, s->err, st));
  return 0;
}

// World frame, layered inference of M rows featurised in a->x with ray frames
// `ray` [2, M]: world profiles into wout [M, npad] (FP16); minr (optional)
// gets each row's smallest predicted range.
int world_profiles(racer_surrogate* s, SurrogateActs* a, const float4* ray, __half* wout, unsigned* minr) {
  int rc = forward(s, a, false, nullptr);
  if (rc) return rc;
  const int H = s->L.H, M = a->M;
  EpiWorldInfer epi{wout, s->L.npad, s->theta + s->L.b4, M, s->L.nout, ray, s->L.beams, minr};
  SURR_CHECK(gemm_launch<256>(a->th3, s->tw4, M, s->L.nout, H / 64, 1, epi, s->err, s->st));
  return 0;
}

// Beam rows pred [beams, ldp] of M cars from their world profiles (k_world_rotate).
int world_rotate(racer_surrogate* s, const __half* wout, const float4* ray, int M, float* pred, long ldp,
                 cudaStream_t st) {
  if (s->L.beams > WORLD_MAX_BEAMS) {
    racer_host::set_error("surrogate: the world frame serves at most 4093 beams");
    return 1;
  }
  SURR_CHECK(world_rotate_configure());
  const int smem = WR_CARS * world_rotate_words(s->L.beams) * 4;
  k_world_rotate<<<(M + WR_CARS - 1) / WR_CARS, WR_THREADS, smem, st>>>(wout, s->L.npad, ray, M, s->L.beams,
                                                                        s->L.nout, pred, ldp);
  SURR_CHECK(cudaGetLastError());
  return 0;
}

// BN must equal the row box of tb's tensor map (256 for the hidden activations, 64 for the inputs).
template <int BN>
int wgrad(racer_surrogate* s, const CUtensorMap& ta, const CUtensorMap& tb, int Mpad, int Mreal, int N, long off) {
  const int kblocks = (s->batch + 63) / 64;
  const int tiles = ((Mpad + 127) / 128) * ((N + BN - 1) / BN);
  int splits = std::max(1, std::min(kblocks, 2 * 148 / std::max(1, tiles)));
  const int per = (kblocks + splits - 1) / splits;
  splits = (kblocks + per - 1) / per;
  if ((size_t)splits * Mpad * N > s->scratch_floats) {
    racer_host::set_error("surrogate: split-K scratch too small");
    return 1;
  }
  EpiSplitF32 epi{s->scratch, (long)Mpad * N, Mpad, N};
  SURR_CHECK(gemm_launch<BN>(ta, tb, Mpad, N, kblocks, splits, epi, s->err, s->st));
  long count = (long)Mreal * N;
  k_reduce_splits<<<(unsigned)((count + 255) / 256), 256, 0, s->st>>>(s->scratch, splits, (long)Mpad * N, N, Mreal,
                                                                       s->grad + off);
  SURR_CHECK(cudaGetLastError());
  return 0;
}

// Encoded inputs of `count` ray frames (sample-major x; feature-major xf if given).
int featurise(racer_surrogate* s, const float4* ray, int count, bf16* x, bf16* xf, cudaStream_t st) {
  if (s->L.world)
    k_features_world<<<(count + 127) / 128, 128, 0, st>>>(ray, count, s->nm, s->gg, s->theta + s->L.g, s->L.nout, x,
                                                          xf);
  else if (s->L.grid)
    k_features_cargrid<<<(count + 127) / 128, 128, 0, st>>>(ray, count, s->nm, s->gg, s->theta + s->L.g, x, xf);
  else
    k_features<<<(count + 127) / 128, 128, 0, st>>>(ray, count, s->nm, x, xf);
  SURR_CHECK(cudaGetLastError());
  return 0;
}

// Labels and features for batch rows taken from the pose set starting at `first`.
// Frames, exact labels and encoded inputs of the batch at pose `first`; with
// `cached`, the labels come from (or go to) the label cache of the pose set.
int prepare(racer_surrogate* s, SurrogateActs* a, long first, bool cached = false) {
  racer_sim* sim = s->sim;
  const int B = a->M;
  const float4* poses = s->poses + first;
  launch_pose_frames(sim->t, poses, B, s->ray, s->st);
  const long b = first / B;
  const size_t block = (size_t)sim->beams * B;
  float* slot = cached && s->lcache && first % B == 0 ? s->lcache + b * block : nullptr;
  if (slot && s->lcached[b]) {
    SURR_CHECK(cudaMemcpyAsync(s->label + 4L * B, slot, block * sizeof(float), cudaMemcpyDeviceToDevice, s->st));
  } else {
    launch_lidar(sim->t, s->ray, s->label, B, sim->beams, sim->beam_dir, nullptr, s->st);
    if (slot) {
      SURR_CHECK(cudaMemcpyAsync(slot, s->label + 4L * B, block * sizeof(float), cudaMemcpyDeviceToDevice, s->st));
      s->lcached[b] = 1;
    }
  }
  return featurise(s, s->ray, B, a->x, a->xf, s->st);
}

// Gradient of the mean squared error over the batch into s->grad; loss sums into s->sums.
int gradient(racer_surrogate* s, long first) {
  SurrogateActs* a = &s->train;
  const int H = s->L.H, B = a->M, NP = s->L.npad, beams = s->L.beams;
  int rc = prepare(s, a, first, true);
  if (rc) return rc;
  SURR_CHECK(cudaMemsetAsync(s->grad + s->L.b2, 0, H * sizeof(float), s->st));
  SURR_CHECK(cudaMemsetAsync(s->grad + s->L.b3, 0, H * sizeof(float), s->st));
  const int nout = s->L.nout;
  SURR_CHECK(cudaMemsetAsync(s->grad + s->L.b4, 0, nout * sizeof(float), s->st));
  SURR_CHECK(cudaMemsetAsync(s->sums, 0, 2 * sizeof(double), s->st));
  if (s->L.grid)
    SURR_CHECK(cudaMemsetAsync(s->grad + s->L.g, 0, (s->L.total - s->L.g) * sizeof(float), s->st));
  if ((rc = forward(s, a, true, nullptr))) return rc;
  const float scale = 2.0f / ((float)B * (float)beams);
  if (s->L.world) {
    SURR_CHECK(gemm_launch<256>(a->th3, s->tw4, B, NP, H / 64, 1, EpiWorldTrain{s->wy, NP, s->theta + s->L.b4, B, nout},
                                s->err, s->st));
    k_world_loss<<<dim3(B / 128, NP / 64), 128, 0, s->st>>>(s->wy, s->label + 4L * B, s->ray, B, beams, nout, NP,
                                                            scale, s->huber, a->g4s, a->g4f, s->grad + s->L.b4,
                                                            s->sums);
    SURR_CHECK(cudaGetLastError());
  } else {
    EpiLoss loss{s->label + 4L * B, B, s->theta + s->L.b4, B, beams, scale,
                 a->g4s, NP, a->g4f, B, s->grad + s->L.b4, s->sums, NP, s->huber};
    SURR_CHECK(gemm_launch<256>(a->th3, s->tw4, B, NP, H / 64, 1, loss, s->err, s->st));
  }
  SURR_CHECK(gemm_launch<256>(a->tg4s, s->tw4t, B, H, NP / 64, 1,
                              EpiDTanh{a->h3s, H, a->g3s, H, a->g3f, B, s->grad + s->L.b3, B, H}, s->err, s->st));
  SURR_CHECK(gemm_launch<256>(a->tg3s, s->tw3t, B, H, H / 64, 1,
                              EpiDTanh{a->h2s, H, a->g2s, H, a->g2f, B, s->grad + s->L.b2, B, H}, s->err, s->st));
  SURR_CHECK(gemm_launch<256>(a->tg2s, s->tw2t, B, H, H / 64, 1,
                              EpiDTanh{a->h1s, H, s->L.grid ? a->g1s : nullptr, H, a->g1f, B, nullptr, B, H}, s->err,
                              s->st));
  if ((rc = wgrad<256>(s, a->tg4f, a->th3f, NP, nout, H, s->L.w4))) return rc;
  if ((rc = wgrad<256>(s, a->tg3f, a->th2f, H, H, H, s->L.w3))) return rc;
  if ((rc = wgrad<256>(s, a->tg2f, a->th1f, H, H, H, s->L.w2))) return rc;
  if ((rc = wgrad<64>(s, a->tg1f, a->txf, H, H, NIN, s->L.w1))) return rc;
  if (s->L.grid) {  // dL/df = g1 W1, then onto the grids
    SURR_CHECK(gemm_launch<64>(a->tg1s, s->tw1t, B, NIN, H / 64, 1, EpiRowF32{s->dx, NIN, B, NIN}, s->err, s->st));
    k_grid_grad<<<B / 128, 128, 0, s->st>>>(s->ray, B, s->gg, s->dx, s->grad + s->L.g);
    SURR_CHECK(cudaGetLastError());
  }
  return 0;
}

int refresh(racer_surrogate* s) {
  k_refresh<<<296, 256, 0, s->st>>>(s->theta, s->L, s->w1b, s->w2b, s->w3b, s->w4b, s->w2t, s->w3t, s->w4t, s->w1t);
  SURR_CHECK(cudaGetLastError());
  return 0;
}

}  // namespace

extern "C" {

int racer_surrogate_create(racer_sim* sim, int hidden, int batch, uint64_t seed, racer_surrogate** out) {
  return racer_surrogate_create_frame(sim, hidden, batch, seed, 0, out);
}

int racer_surrogate_create_frame(racer_sim* sim, int hidden, int batch, uint64_t seed, int frame,
                                 racer_surrogate** out) {
  using racer_host::set_error;
  if (!sim || !out || (hidden != 128 && hidden != 256 && hidden != 512) || batch < 128 || (batch % 128)) {
    set_error("racer_surrogate_create: hidden must be 128, 256 or 512 and batch a positive multiple of 128");
    return 1;
  }
  if (frame < 0 || frame > 2) {
    set_error("racer_surrogate_create_frame: frame must be 0 (car), 1 (world) or 2 (car, feature grids)");
    return 1;
  }
  if (frame == 1 && ((sim->beams - 1) % 12 != 0 || sim->beams < 13 || sim->beams > WORLD_MAX_BEAMS)) {
    set_error("racer_surrogate_create_frame: the world frame needs beams - 1 a multiple of 12 (the beam spacing "
              "then divides the circle into a multiple of 16 world samples) and at most 4093 beams");
    return 1;
  }
  if (sim->seg.count != 1) {
    set_error("racer_surrogate_create: a surrogate learns one track; the sim holds several");
    return 1;
  }
  if (sim->t.layers > 2) {
    set_error("racer_surrogate_create: the surrogate's inputs encode at most two layers");
    return 1;
  }
  racer_surrogate* s = new racer_surrogate();
  s->sim = sim;
  s->st = sim->st;
  s->batch = batch;
  Layout& L = s->L;
  L.H = hidden;
  L.beams = sim->beams;
  L.world = frame == 1;
  L.grid = frame != 0;
  L.nout = L.world ? 4 * (sim->beams - 1) / 3 : sim->beams;
  L.npad = (L.nout + 63) / 64 * 64;
  L.w1 = 0;
  L.w2 = L.w1 + (long)hidden * NIN;
  L.b2 = L.w2 + (long)hidden * hidden;
  L.w3 = L.b2 + hidden;
  L.b3 = L.w3 + (long)hidden * hidden;
  L.w4 = L.b3 + hidden;
  L.b4 = L.w4 + (long)L.nout * hidden;
  L.g = L.grid ? (L.b4 + L.nout + 7) / 8 * 8 : L.b4 + L.nout;  // grids 32-byte aligned
  L.total = L.g;
  const TrackDev& t = sim->t;
  if (L.grid) {  // feature grids over the map, per layer
    GridGeom& g = s->gg;
    g.x0 = t.x0, g.y0 = t.y0;
    long off = 0;
    for (int l = 0; l < GRID_LEVELS; ++l) {
      const float r = GRID_CELLS0 * t.cell / (float)(1 << l);
      g.inv_r[l] = 1.0f / r;
      g.gx[l] = (int)std::ceil((double)t.nx * t.cell / r) + 2;
      g.gy[l] = (int)std::ceil((double)t.ny * t.cell / r) + 2;
      g.off[l] = off;
      off += (long)t.layers * g.gx[l] * g.gy[l] * GRID_F;
    }
    L.total = L.g + off;
  }
  const float hx = 0.5f * (float)(t.nx - 1) * t.cell, hy = 0.5f * (float)(t.ny - 1) * t.cell;
  s->nm = Norm{t.x0 + hx, 1.0f / hx, t.y0 + hy, 1.0f / hy};
  const int H = hidden, NP = L.npad;
  int rc = 0;
  if ((L.grid && ((rc = salloc(&s->w1t, (size_t)NIN * H)) || (rc = salloc(&s->dx, (size_t)batch * NIN)) ||
                   (rc = make_tmap_bf16(&s->tw1t, s->w1t, NIN, H, H, 64)))) ||
      (L.world && ((rc = salloc(&s->wy, (size_t)batch * NP)) || (rc = salloc(&s->wbatch, (size_t)batch * NP))))) {
    racer_surrogate_destroy(s);
    return rc;
  }
  s->scratch_floats = (size_t)2 * 148 * 128 * 256 + (size_t)NP * H;
  if ((rc = salloc(&s->theta, L.total)) || (rc = salloc(&s->grad, L.total)) || (rc = salloc(&s->m1, L.total)) ||
      (rc = salloc(&s->m2, L.total)) || (rc = salloc(&s->w1b, (size_t)H * NIN)) || (rc = salloc(&s->w2b, (size_t)H * H)) ||
      (rc = salloc(&s->w3b, (size_t)H * H)) || (rc = salloc(&s->w4b, (size_t)NP * H)) ||
      (rc = salloc(&s->w2t, (size_t)H * H)) || (rc = salloc(&s->w3t, (size_t)H * H)) ||
      (rc = salloc(&s->w4t, (size_t)H * NP)) || (rc = salloc(&s->ray, 2 * (size_t)batch)) ||
      (rc = salloc(&s->label, (size_t)(4 + sim->beams) * batch)) || (rc = salloc(&s->pred, (size_t)sim->beams * batch)) ||
      (rc = salloc(&s->scratch, s->scratch_floats)) || (rc = salloc(&s->sums, 4)) || (rc = salloc(&s->maxbits, 1)) ||
      (rc = salloc(&s->over, 1)) || (rc = salloc(&s->err, 1))) {
    racer_surrogate_destroy(s);
    return rc;
  }
  if ((rc = make_tmap_bf16(&s->tw1, s->w1b, H, NIN, NIN, 256)) || (rc = make_tmap_bf16(&s->tw2, s->w2b, H, H, H, 256)) ||
      (rc = make_tmap_bf16(&s->tw3, s->w3b, H, H, H, 256)) || (rc = make_tmap_bf16(&s->tw4, s->w4b, NP, H, H, 256)) ||
      (rc = make_tmap_bf16(&s->tw2t, s->w2t, H, H, H, 256)) || (rc = make_tmap_bf16(&s->tw3t, s->w3t, H, H, H, 256)) ||
      (rc = make_tmap_bf16(&s->tw4t, s->w4t, H, NP, NP, 256)) || (rc = make_acts(s, &s->train, batch, true))) {
    racer_surrogate_destroy(s);
    return rc;
  }
  // drivable (cell, layer) pairs from the track's clearance grids
  std::vector<float> clear((size_t)t.nx * t.ny);
  std::vector<int2> cells;
  for (int l = 0; l < t.layers; ++l) {
    cudaMemcpy(clear.data(), sim->d_track + 12 + (size_t)(3 * l) * t.nx * t.ny, clear.size() * sizeof(float),
               cudaMemcpyDeviceToHost);
    for (size_t k = 0; k < clear.size(); ++k)
      if (clear[k] > 0.0f) cells.push_back(make_int2((int)k, l));
  }
  if (cells.empty()) {
    set_error("racer_surrogate_create: the track has no drivable cell");
    racer_surrogate_destroy(s);
    return 1;
  }
  s->ncells = (int)cells.size();
  if ((rc = salloc(&s->cells, cells.size()))) {
    racer_surrogate_destroy(s);
    return rc;
  }
  cudaMemcpy(s->cells, cells.data(), cells.size() * sizeof(int2), cudaMemcpyHostToDevice);
  k_init_params<<<296, 256, 0, s->st>>>(s->theta, L, seed);
  if ((rc = refresh(s))) {
    racer_surrogate_destroy(s);
    return rc;
  }
  RACER_TRY(cudaStreamSynchronize(s->st));
  *out = s;
  return 0;
}

int racer_surrogate_destroy(racer_surrogate* s) {
  if (!s) return 0;
  for (void* p : {(void*)s->w1t, (void*)s->wy, (void*)s->dx, (void*)s->wbatch, (void*)s->wout})
    cudaFree(p);
  for (void* p : {(void*)s->theta, (void*)s->grad, (void*)s->m1, (void*)s->m2, (void*)s->w1b, (void*)s->w2b,
                  (void*)s->w3b, (void*)s->w4b, (void*)s->w2t, (void*)s->w3t, (void*)s->w4t, (void*)s->cells,
                  (void*)s->poses, (void*)s->ray, (void*)s->label, (void*)s->lcache, (void*)s->pred, (void*)s->scratch,
                  (void*)s->sums,
                  (void*)s->maxbits, (void*)s->over, (void*)s->err})
    cudaFree(p);
  free_acts(&s->train);
  free_acts(&s->infer);
  for (void* p : {(void*)s->minr, (void*)s->list, (void*)s->list_count, (void*)s->list_units, (void*)s->exact,
                  (void*)s->rsums, (void*)s->rmax, (void*)s->rcount})
    cudaFree(p);
  delete s;
  return 0;
}

int racer_surrogate_params(racer_surrogate* s, float** theta, float** grad, long* count, int* hidden) {
  if (!s) {
    racer_host::set_error("racer_surrogate_params: null surrogate");
    return 1;
  }
  if (theta) *theta = s->theta;
  if (grad) *grad = s->grad;
  if (count) *count = s->L.total;
  if (hidden) *hidden = s->L.H;
  return 0;
}

int racer_surrogate_grid(racer_surrogate* s, int* gx, int* gy, float* spacing_m, long* offset) {
  if (!s || !s->L.grid) {
    racer_host::set_error("racer_surrogate_grid: the surrogate has no feature grids");
    return 1;
  }
  for (int l = 0; l < GRID_LEVELS; ++l) {
    if (gx) gx[l] = s->gg.gx[l];
    if (gy) gy[l] = s->gg.gy[l];
    if (spacing_m) spacing_m[l] = 1.0f / s->gg.inv_r[l];
    if (offset) offset[l] = s->L.g + s->gg.off[l];
  }
  return 0;
}

int racer_surrogate_batch_inputs(racer_surrogate* s, float* inputs, int* k0) {
  if (!s) {
    racer_host::set_error("racer_surrogate_batch_inputs: null surrogate");
    return 1;
  }
  const int B = s->batch;
  if (inputs) {
    std::vector<uint16_t> raw((size_t)B * NIN);
    RACER_TRY(cudaMemcpyAsync(raw.data(), s->train.x, raw.size() * sizeof(uint16_t), cudaMemcpyDeviceToHost, s->st));
    RACER_TRY(cudaStreamSynchronize(s->st));
    for (size_t i = 0; i < raw.size(); ++i) {
      const uint32_t u = (uint32_t)raw[i] << 16;
      memcpy(inputs + i, &u, sizeof u);
    }
  }
  if (k0 && s->L.world) {
    int* d = nullptr;
    RACER_TRY(cudaMalloc((void**)&d, (size_t)B * sizeof(int)));
    k_world_k0<<<(B + 127) / 128, 128, 0, s->st>>>(s->ray, B, s->L.nout, d);
    cudaError_t e = cudaMemcpyAsync(k0, d, (size_t)B * sizeof(int), cudaMemcpyDeviceToHost, s->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
    cudaFree(d);
    RACER_TRY(e);
  }
  return 0;
}

int racer_surrogate_batch_predict(racer_surrogate* s, float* pred) {
  if (!s || !pred || !s->poses) {
    racer_host::set_error("racer_surrogate_batch_predict: set poses and run a gradient first");
    return 1;
  }
  SurrogateActs* a = &s->train;
  const int B = s->batch;
  int rc;
  if (s->L.world) {
    rc = world_profiles(s, a, s->ray, s->wbatch, nullptr);
    if (!rc) rc = world_rotate(s, s->wbatch, s->ray, B, pred, B, s->st);
  } else {
    EpiInfer inf{pred, B, s->theta + s->L.b4, B, s->L.beams, nullptr};
    rc = forward(s, a, false, &inf);
  }
  if (rc) return rc;
  RACER_TRY(cudaStreamSynchronize(s->st));
  return 0;
}

// The training set: `count` poses (a multiple of the batch) drawn with `seed`.
int racer_surrogate_set_poses(racer_surrogate* s, long count, uint64_t seed) {
  if (!s || count < s->batch || (count % s->batch)) {
    racer_host::set_error("racer_surrogate_set_poses: count must be a positive multiple of the batch");
    return 1;
  }
  cudaFree(s->poses);
  s->poses = nullptr;
  cudaFree(s->lcache);
  s->lcache = nullptr;
  s->lcached.assign(0, 0);
  if (int rc = salloc(&s->poses, (size_t)count)) return rc;
  s->npose = (int)count;
  const size_t cache_bytes = (size_t)count * s->L.beams * sizeof(float);
  if (s->use_cache && cache_bytes <= (32ull << 30)) {  // else trace every batch every epoch
    if (cudaMalloc((void**)&s->lcache, cache_bytes) == cudaSuccess) {
      s->lcached.assign(count / s->batch, 0);
    } else {
      cudaGetLastError();
      s->lcache = nullptr;
    }
  }
  k_sample_poses<<<(unsigned)((count + 255) / 256), 256, 0, s->st>>>(s->cells, s->ncells, (int)count, seed, s->sim->t,
                                                                       s->poses);
  RACER_TRY(cudaGetLastError());
  return 0;
}

// Use the surrogate with another sim of the same track (a trained surrogate
// serving several sims, one after the other): the track's header, array
// length and beam count must match the sim it was built for.
int racer_surrogate_bind(racer_surrogate* s, racer_sim* sim) {
  using racer_host::set_error;
  if (!s || !sim) {
    set_error("racer_surrogate_bind: null argument");
    return 1;
  }
  if (sim == s->sim) return 0;
  const TrackDev &a = s->sim->t, &b = sim->t;
  if (sim->seg.count != 1 || sim->beams != s->L.beams || sim->track_len != s->sim->track_len || a.nx != b.nx ||
      a.ny != b.ny || a.layers != b.layers || a.x0 != b.x0 || a.y0 != b.y0 || a.cell != b.cell ||
      a.waypoints != b.waypoints) {
    set_error("racer_surrogate_bind: the sim's track or beam count differs from the surrogate's");
    return 1;
  }
  RACER_TRY(cudaStreamSynchronize(s->st));
  // the old sim's learned-lidar graphs read this surrogate's inference buffers
  for (auto& kv : s->sim->surrogate_graphs) cudaGraphExecDestroy(kv.second);
  s->sim->surrogate_graphs.clear();
  if (s->infer.M && s->infer.M != sim->n) {  // inference buffers are sized for the cars
    free_acts(&s->infer);
    s->infer = SurrogateActs();
    for (void* p : {(void*)s->minr, (void*)s->list, (void*)s->list_count, (void*)s->list_units, (void*)s->exact,
                    (void*)s->wout})
      cudaFree(p);
    s->minr = nullptr, s->list = nullptr, s->list_count = nullptr, s->list_units = nullptr, s->exact = nullptr;
    s->wout = nullptr;
  }
  s->sim = sim;
  s->st = sim->st;
  return 0;
}

int racer_surrogate_set_fused(racer_surrogate* s, int fused) {
  if (!s) {
    racer_host::set_error("racer_surrogate_set_fused: null surrogate");
    return 1;
  }
  s->fused = fused != 0;
  for (auto& kv : s->sim->surrogate_graphs) cudaGraphExecDestroy(kv.second);
  s->sim->surrogate_graphs.clear();
  return 0;
}

int racer_surrogate_set_label_cache(racer_surrogate* s, int enable) {
  if (!s) {
    racer_host::set_error("racer_surrogate_set_label_cache: null surrogate");
    return 1;
  }
  s->use_cache = enable != 0;
  RACER_TRY(cudaStreamSynchronize(s->st));
  cudaFree(s->lcache);  // a later racer_surrogate_set_poses builds it again when enabled
  s->lcache = nullptr;
  s->lcached.assign(0, 0);
  return 0;
}

int racer_surrogate_set_spot_check(racer_surrogate* s, int stride, float tolerance_m) {
  if (!s || stride < 0 || !(tolerance_m > 0.0f)) {
    racer_host::set_error("racer_surrogate_set_spot_check: stride must be >= 0 and the tolerance positive");
    return 1;
  }
  s->spot_stride = stride;
  s->spot_tol = tolerance_m / RANGE;
  for (auto& kv : s->sim->surrogate_graphs) cudaGraphExecDestroy(kv.second);
  s->sim->surrogate_graphs.clear();
  return 0;
}

int racer_surrogate_set_loss(racer_surrogate* s, float huber_m) {
  if (!s || !(huber_m >= 0.0f)) {
    racer_host::set_error("racer_surrogate_set_loss: null surrogate or negative threshold");
    return 1;
  }
  s->huber = huber_m / RANGE;
  return 0;
}

// Poses (x, y, heading, layer) of the training set, for inspection.
int racer_surrogate_poses(racer_surrogate* s, void** poses, long* count) {
  if (!s) {
    racer_host::set_error("racer_surrogate_poses: null surrogate");
    return 1;
  }
  if (poses) *poses = s->poses;
  if (count) *count = s->npose;
  return 0;
}

// Gradient of the batch starting at pose `first` (no update); labels stay in the label buffer.
int racer_surrogate_gradient(racer_surrogate* s, long first, float* mse, float* label_dev_out) {
  if (!s || !s->poses || first < 0 || first + s->batch > s->npose) {
    racer_host::set_error("racer_surrogate_gradient: set poses first; the batch must lie inside the pose set");
    return 1;
  }
  if (int rc = gradient(s, first)) return rc;
  if (label_dev_out)
    RACER_TRY(cudaMemcpyAsync(label_dev_out, s->label + 4L * s->batch, (size_t)s->L.beams * s->batch * sizeof(float),
                              cudaMemcpyDeviceToDevice, s->st));
  double sums[2];
  RACER_TRY(cudaMemcpyAsync(sums, s->sums, sizeof sums, cudaMemcpyDeviceToHost, s->st));
  RACER_TRY(cudaStreamSynchronize(s->st));
  if (mse) *mse = (float)(sums[0] / ((double)s->batch * s->L.beams));
  return 0;
}

// `steps` Adam steps over consecutive batches of the pose set; lr decays by cosine to lr/100.
int racer_surrogate_train(racer_surrogate* s, int steps, float lr, float* last_mse, float* last_mae_m) {
  if (!s || !s->poses || steps < 1 || !(lr > 0)) {
    racer_host::set_error("racer_surrogate_train: set poses first; steps >= 1, lr > 0");
    return 1;
  }
  const int per_epoch = s->npose / s->batch;
  for (int k = 0; k < steps; ++k) {
    long first = (long)(s->step % per_epoch) * s->batch;
    if (int rc = gradient(s, first)) return rc;
    s->step += 1;
    const float frac = (float)k / (float)steps;
    const float rate = lr * (0.01f + 0.99f * 0.5f * (1.0f + cosf(3.14159265f * frac)));
    const float c1 = 1.0f - powf(0.9f, (float)s->step), c2 = 1.0f - powf(0.999f, (float)s->step);
    k_adam_s<<<592, 256, 0, s->st>>>(s->L.g, rate, 0.999f, 1e-8f, c1, c2, s->theta, s->grad, s->m1, s->m2);
    if (s->L.grid) {  // the feature grids: a higher rate, beta2 0.99, a tiny epsilon
      const long g = s->L.g;
      k_adam_s<<<592, 256, 0, s->st>>>(s->L.total - g, rate * GRID_LR_SCALE, 0.99f, 1e-15f, c1,
                                       1.0f - powf(0.99f, (float)s->step), s->theta + g, s->grad + g, s->m1 + g,
                                       s->m2 + g);
    }
    RACER_TRY(cudaGetLastError());
    if (int rc = refresh(s)) return rc;
  }
  double sums[2];
  RACER_TRY(cudaMemcpyAsync(sums, s->sums, sizeof sums, cudaMemcpyDeviceToHost, s->st));
  RACER_TRY(cudaStreamSynchronize(s->st));
  const double total = (double)s->batch * s->L.beams;
  if (last_mse) *last_mse = (float)(sums[0] / total);
  if (last_mae_m) *last_mae_m = (float)(sums[1] / total * RANGE);
  return 0;
}

// Held-out error: `batches` fresh batches of poses drawn with `seed`, surrogate vs exact tracer.
int racer_surrogate_evaluate(racer_surrogate* s, int batches, uint64_t seed, float* mae_m, float* rmse_m, float* max_m,
                             float* frac_over_5cm) {
  if (!s || batches < 1) {
    racer_host::set_error("racer_surrogate_evaluate: bad argument");
    return 1;
  }
  float4* keep = s->poses;
  int keep_n = s->npose;
  float* keep_cache = s->lcache;  // the held-out poses neither use nor replace the training set's labels
  std::vector<uint8_t> keep_cached;
  keep_cached.swap(s->lcached);
  const bool keep_use = s->use_cache;
  s->poses = nullptr;
  s->lcache = nullptr;
  s->use_cache = false;
  int rc = racer_surrogate_set_poses(s, (long)batches * s->batch, seed);
  s->use_cache = keep_use;
  if (rc) {
    s->poses = keep;
    s->npose = keep_n;
    s->lcache = keep_cache;
    s->lcached.swap(keep_cached);
    return rc;
  }
  RACER_TRY(cudaMemsetAsync(s->sums + 2, 0, 2 * sizeof(double), s->st));
  RACER_TRY(cudaMemsetAsync(s->maxbits, 0, sizeof(unsigned), s->st));
  RACER_TRY(cudaMemsetAsync(s->over, 0, sizeof(unsigned long long), s->st));
  SurrogateActs* a = &s->train;
  const int B = s->batch;
  for (int k = 0; k < batches && !rc; ++k) {
    if ((rc = prepare(s, a, (long)k * B))) break;
    if (s->L.world) {
      if ((rc = world_profiles(s, a, s->ray, s->wbatch, nullptr)) ||
          (rc = world_rotate(s, s->wbatch, s->ray, B, s->pred, B, s->st)))
        break;
    } else {
      EpiInfer inf{s->pred, B, s->theta + s->L.b4, B, s->L.beams, nullptr};
      if ((rc = forward(s, a, false, &inf))) break;
    }
    k_compare<<<296, 256, 0, s->st>>>(s->pred, s->label + 4L * B, (long)s->L.beams * B, s->sums + 2, s->maxbits,
                                      s->over);
  }
  cudaFree(s->poses);
  s->poses = keep;
  s->npose = keep_n;
  s->lcache = keep_cache;
  s->lcached.swap(keep_cached);
  if (rc) return rc;
  double sums[2];
  unsigned mx = 0;
  unsigned long long over = 0;
  RACER_TRY(cudaMemcpyAsync(sums, s->sums + 2, sizeof sums, cudaMemcpyDeviceToHost, s->st));
  RACER_TRY(cudaMemcpyAsync(&mx, s->maxbits, sizeof mx, cudaMemcpyDeviceToHost, s->st));
  RACER_TRY(cudaMemcpyAsync(&over, s->over, sizeof over, cudaMemcpyDeviceToHost, s->st));
  RACER_TRY(cudaStreamSynchronize(s->st));
  const double total = (double)batches * B * s->L.beams;
  if (mae_m) *mae_m = (float)(sums[0] / total);
  if (rmse_m) *rmse_m = (float)std::sqrt(sums[1] / total);
  if (max_m) {
    float f;
    memcpy(&f, &mx, sizeof f);
    *max_m = f;
  }
  if (frac_over_5cm) *frac_over_5cm = (float)((double)over / total);
  return 0;
}

// Rollout statistics since the last reset: audited error (metres) and the
// fraction of car-steps that fell back to the exact tracer.
int racer_surrogate_rollout_stats(racer_surrogate* s, float* mae_m, float* rmse_m, float* max_m,
                                  float* frac_over_5cm, float* fallback_frac, int reset) {
  if (!s) {
    racer_host::set_error("racer_surrogate_rollout_stats: null surrogate");
    return 1;
  }
  double sums[2] = {0, 0};
  unsigned mx = 0;
  unsigned long long counts[2] = {0, 0};
  if (s->rsums) {
    RACER_TRY(cudaMemcpyAsync(sums, s->rsums, sizeof sums, cudaMemcpyDeviceToHost, s->st));
    RACER_TRY(cudaMemcpyAsync(&mx, s->rmax, sizeof mx, cudaMemcpyDeviceToHost, s->st));
    RACER_TRY(cudaMemcpyAsync(counts, s->rcount, sizeof counts, cudaMemcpyDeviceToHost, s->st));
  }
  RACER_TRY(cudaStreamSynchronize(s->st));
  const double beams = s->audited_beams > 0 ? s->audited_beams : 1.0;
  if (mae_m) *mae_m = (float)(sums[0] / beams);
  if (rmse_m) *rmse_m = (float)std::sqrt(sums[1] / beams);
  if (max_m) {
    float f;
    memcpy(&f, &mx, sizeof f);
    *max_m = f;
  }
  if (frac_over_5cm) *frac_over_5cm = (float)((double)counts[0] / beams);
  if (fallback_frac) *fallback_frac = (float)(s->car_steps > 0 ? (double)counts[1] / s->car_steps : 0.0);
  if (reset && s->rsums) {
    RACER_TRY(cudaMemsetAsync(s->rsums, 0, 2 * sizeof(double), s->st));
    RACER_TRY(cudaMemsetAsync(s->rmax, 0, sizeof(unsigned), s->st));
    RACER_TRY(cudaMemsetAsync(s->rcount, 0, 2 * sizeof(unsigned long long), s->st));
    s->audited_beams = s->car_steps = 0;
  }
  return 0;
}

}  // extern "C"

// ---- rollout integration (used by racer_rollout_surrogate in api.cu) ----

int surrogate_prepare(racer_surrogate* s, racer_sim* sim) {
  if (s->sim != sim) {
    racer_host::set_error("surrogate: built for a different sim");
    return 1;
  }
  if (s->infer.M == sim->n) return 0;
  if (s->infer.M) {
    racer_host::set_error("surrogate: the sim's car count changed");
    return 1;
  }
  const int n = sim->n;
  int rc = 0;
  SURR_CHECK((gemm_configure<256, EpiTanhOut>()));
  SURR_CHECK((gemm_configure<256, EpiInfer>()));
  SURR_CHECK((gemm_configure<256, EpiWorldInfer>()));
  if (s->L.world) {
    SURR_CHECK(world_rotate_configure());  // before any capture
    if ((rc = salloc(&s->wout, (size_t)n * s->L.npad))) return rc;
  }
  if ((rc = make_acts(s, &s->infer, n, false)) || (rc = salloc(&s->minr, (size_t)n)) ||
      (rc = salloc(&s->list, (size_t)n)) || (rc = salloc(&s->list_count, 1)) || (rc = salloc(&s->list_units, 1)) ||
      (rc = salloc(&s->exact, (size_t)(4 + sim->beams) * n)))
    return rc;
  if (!s->rsums && ((rc = salloc(&s->rsums, 2)) || (rc = salloc(&s->rmax, 1)) || (rc = salloc(&s->rcount, 2))))
    return rc;
  return 0;
}

namespace racer {
namespace {
__global__ void k_count_fallback(const int* count, unsigned long long* total) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *total += (unsigned long long)*count;
}
}  // namespace
}  // namespace racer

// The lidar rows of obs for the sim's cars after their physics step: the
// surrogate's prediction, replaced by the exact tracer for every car on an
// audit step (with the error accumulated), else for the cars whose smallest
// predicted range is below `fallback` (obs units, range / RANGE).
int surrogate_lidar(racer_surrogate* s, racer_sim* sim, float* obs, bool audit, float fallback, cudaStream_t st,
                    const int64_t* step_base, int64_t step_add) {
  const int n = sim->n, beams = sim->beams;
  SurrogateActs* a = &s->infer;
  if (int rc = featurise(s, sim->ray, n, a->x, nullptr, st)) return rc;
  SURR_CHECK(cudaMemsetAsync(s->minr, 0x7f, (size_t)n * sizeof(unsigned), st));
  // on an audit step the prediction goes to the scratch rows and the exact tracer writes obs
  float* pred = audit ? s->exact + 4L * n : obs + 4L * n;
  const bool world = s->L.world != 0;
  if (s->fused && s->L.H == SF_H) {
    const float* th = s->theta;
    FusedArgs fa{th + s->L.b2, th + s->L.b3, th + s->L.b4, pred, s->minr, n, beams, (s->L.npad + 255) / 256, s->err,
                 world ? s->wout : nullptr, s->L.npad, s->L.nout, sim->ray};
    SURR_CHECK(surrogate_fused_launch(a->tx, s->tw1, s->tw2, s->tw3, s->tw4, fa, sim->sms, st));
  } else {
    cudaStream_t keep = s->st;
    s->st = st;
    int rc;
    if (world) {
      rc = world_profiles(s, a, sim->ray, s->wout, s->minr);
    } else {
      EpiInfer inf{pred, n, s->theta + s->L.b4, n, beams, s->minr};
      rc = forward(s, a, false, &inf);
    }
    s->st = keep;
    if (rc) return rc;
  }
  // The predicted rows first (the spot check reads them), then the exact
  // tracer for the audit or the fallback cars. (Tracing the fallback cars on a
  // second stream beside the world frame's gather measured slower than this
  // order: the two kernels contend for the SMs.)
  if (world)
    if (int rc = world_rotate(s, s->wout, sim->ray, n, pred, n, st)) return rc;
  if (audit) {
    launch_lidar(sim->t, sim->ray, obs, n, beams, sim->beam_dir, nullptr, st);
  } else if (fallback > 0.0f || s->spot_stride > 0) {
    if (s->spot_stride > 0)  // a checked beam off by more than the tolerance marks its car (minr = 0)
      launch_lidar_spot(sim->t, sim->ray, pred, n, beams, sim->beam_dir, s->spot_stride, step_base, step_add,
                        s->spot_tol, s->minr, st);
    SURR_CHECK(cudaMemsetAsync(s->list_count, 0, sizeof(int), st));
    // the threshold stays above 0 so that marked cars are always selected
    launch_select_cars(s->minr, n, fallback > 0.0f ? fallback : 1e-30f, s->list, s->list_count, st);
    launch_lidar_list(sim->t, sim->ray, obs, n, beams, sim->beam_dir, s->list, s->list_count, n, s->list_units,
                      sim->sms, st);
    k_count_fallback<<<1, 32, 0, st>>>(s->list_count, s->rcount + 1);
  }
  if (audit) k_compare<<<1216, 256, 0, st>>>(pred, obs + 4L * n, (long)beams * n, s->rsums, s->rmax, s->rcount);
  SURR_CHECK(cudaGetLastError());
  return 0;
}

void surrogate_account(racer_surrogate* s, racer_sim* sim, int steps, int audits) {
  s->audited_beams += (double)audits * sim->beams * sim->n;
  s->car_steps += (double)(steps - audits) * sim->n;
}
