// Fused inference of the lidar surrogate (hidden width 512): for each tile of
// 128 cars, encoded inputs -> 3 tanh layers -> ranges in one persistent kernel,
// the activations never leaving the SM.
//
// Per CTA (one per SM): warp 0 streams the weight k-blocks with TMA through a
// ring of 32 KB stages (256 weight rows x 64 k) and loads the tile's input
// block; warp 1 allocates all 512 TMEM columns (two 256-column slots) and
// issues the MMAs; warps 2-17 are the epilogue, four per TMEM lane quarter
// (enough warps to hide the accumulator loads and tanh latencies). The A operand of every layer
// lives in one 128 KB shared buffer (8 k-blocks of 128 rows x 64, K-major,
// 128B-swizzled): the input block in k-block 0 for layer 1, then each hidden
// epilogue writes its tanh output there in BF16 as the next layer's A. The
// output layer runs in 256-column chunks alternating between the two TMEM
// slots, so the epilogue of one chunk (clamp, then the obs rows in the car
// frame or the FP16 world-profile rows in the world frame, and the per-car
// minimum) overlaps the MMAs of the next; each CTA starts at a different chunk so the
// SMs do not all read the same weight lines at once. The MMAs, their k order
// and the BF16 rounding of
// the activations are those of the layer-by-layer GEMMs, so the two paths give
// the same bits.
//
// Barriers and their completions per tile (T tiles done before this one):
//   xfull      1   input block landed (TMA transaction count)
//   afree      1   every MMA reading the A buffer has completed (after the output layer)
//   edone      3   a hidden epilogue wrote A and drained TMEM (512 arrivals)
//   accfull[s] 3 + chunks in slot s: an accumulator slot is complete (MMA commit)
//   accempty[s] chunks in slot s: the epilogue drained an output chunk (512 arrivals)
// A wait for completion k of a barrier uses parity k & 1; every wait is bounded
// and a timeout sets *err.
#pragma once
#include <cuda_fp16.h>

#include "common.cuh"
#include "tc.cuh"

namespace racer {
namespace {

// World sample read by beam 0 of a car with heading (sin h, cos h), and the
// phase (fractional part) of its angle: u = (h - FOV / 2) K / (2 pi) mod K.
__device__ __forceinline__ int world_phase(float sh, float ch, int K, float* phase) {
  float u = (atan2f(sh, ch) - 0.5f * FOV) * ((float)K / TWO_PI_F);
  if (u < 0.0f) u += (float)K;        // u > -K before
  if (!(u < (float)K)) u = 0.0f;     // rounded up to K, or a NaN heading
  const int k = (int)u;
  *phase = u - (float)k;
  return k;
}

// World frame, inference: 16 world samples o0 .. o0 + 15 of one car (o0 a
// multiple of 16, K of 16), saturated to [0, 1], rounded to FP16 into row
// (16-byte aligned), and the smallest of those inside the car's field of view
// (beam (o - k0) mod K < beams), taken before the rounding and rounded once
// (rounding is monotonic, so that is the smallest rounded value). A group
// with no sample in the field of view is not stored (nothing reads it). The
// fused kernel and the layered epilogue both use it.
__device__ __forceinline__ float world_store16(const float* v, const float* bias, int o0, int K, int k0, int beams,
                                               __half* row, float lo) {
  if (o0 >= K) return lo;
  int b0 = o0 - k0;  // beam of sample o0 (mod K)
  if (b0 < 0) b0 += K;
  if (b0 >= beams && b0 + 15 < K) return lo;  // wholly outside the field of view
  float y[16];
#pragma unroll
  for (int j = 0; j < 16; ++j) y[j] = __saturatef(v[j] + bias[j]);
  uint32_t w[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const __half2 t = __floats2half2_rn(y[2 * j], y[2 * j + 1]);
    w[j] = *reinterpret_cast<const uint32_t*>(&t);
  }
  uint4* dst = reinterpret_cast<uint4*>(row + o0);
  dst[0] = make_uint4(w[0], w[1], w[2], w[3]);
  dst[1] = make_uint4(w[4], w[5], w[6], w[7]);
  float mn = 1.0f;
  if (b0 + 15 < beams) {  // wholly inside
#pragma unroll
    for (int j = 0; j < 16; ++j) mn = fminf(mn, y[j]);
  } else {
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      int b = b0 + j;
      if (b >= K) b -= K;
      if (b < beams) mn = fminf(mn, y[j]);
    }
  }
  return fminf(lo, __half2float(__float2half_rn(mn)));
}

constexpr int SF_H = 512;                      // hidden width
constexpr int SF_KB = SF_H / 64;               // k-blocks of a hidden activation
constexpr int SF_A_BYTES = SF_KB * 128 * 128;  // 128 rows x 512 BF16
constexpr int SF_STAGE = 256 * 128;            // 256 weight rows x 64 k (BF16)
constexpr int SF_STAGES = 3;
constexpr int SF_SMEM = SF_A_BYTES + SF_STAGES * SF_STAGE + 256 + 1024;  // + barriers, alignment slack
constexpr int SF_EPI = 512;  // epilogue threads: warps 2-17
constexpr int SF_THREADS = 64 + SF_EPI;

struct FusedArgs {
  const float* b2;
  const float* b3;
  const float* b4;
  float* out;  // obs + 4 n: out[o * n + car] (car frame)
  unsigned* minr;
  int n, beams, chunks;  // chunks = ceil(npad / 256)
  int* err;
  // world frame (wout not null): world profiles wout[car * ldw + o] (FP16), K world samples;
  // the ray frames [2, n] give each car's field of view
  __half* wout;
  int ldw, K;
  const float4* ray;
};

struct SfBars {
  uint64_t *full, *empty, *xfull, *afree, *edone, *accfull, *accempty, *mdone;
  volatile int* abort;  // set by the first wait that times out; every other wait then gives up at once
};

// Bounded wait for completion parity `parity`: false on timeout or once another role aborted.
__device__ __forceinline__ bool sf_wait(uint64_t* bar, uint32_t parity, volatile int* abort) {
  for (uint32_t i = 0; i < (1u << 22); ++i) {
    if (tc::mbar_try_wait(bar, parity)) return true;
    if ((i & 255u) == 255u && *abort) return false;
  }
  *abort = 1;
  return false;
}

// Producer (one thread). *issued counts the weight stages it issued.
__device__ bool sf_producer(const CUtensorMap* tx, const CUtensorMap* tw1, const CUtensorMap* tw2,
                            const CUtensorMap* tw3, const CUtensorMap* tw4, uint8_t* abuf, uint8_t* stages,
                            const SfBars& b, int tiles, int nc, uint32_t* issued, uint32_t* xloads) {
  uint32_t it = 0, local = 0;
  for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x, ++local) {
    for (int e = 0; e < 2 + 4 * SF_KB + nc * SF_KB; ++e) {
      if (e == 2) {  // the input block, once the previous tile's output layer no longer reads A
        if (local > 0 && !sf_wait(b.afree, (local - 1) & 1, b.abort)) return false;
        tc::mbar_arrive_expect_tx(b.xfull, 128 * 128);
        tc::tma_load_2d(abuf, tx, 0, tile * 128, b.xfull);
        *xloads = local + 1;
      }
      const CUtensorMap* map;
      int row, kb;
      if (e < 2) {
        map = tw1, row = 256 * e, kb = 0;
      } else if (e < 2 + 4 * SF_KB) {
        const int f = e - 2;  // layer (f / (2 KB)), then k-block, then half
        map = f < 2 * SF_KB ? tw2 : tw3;
        kb = (f % (2 * SF_KB)) / 2;
        row = 256 * (f & 1);
      } else {
        const int f = e - 2 - 4 * SF_KB;  // chunk position, then k-block
        map = tw4, row = 256 * ((f / SF_KB + blockIdx.x % nc) % nc), kb = f % SF_KB;
      }
      const uint32_t s = it % SF_STAGES;
      if (it >= (uint32_t)SF_STAGES && !sf_wait(&b.empty[s], ((it / SF_STAGES) - 1) & 1, b.abort)) return false;
      tc::mbar_arrive_expect_tx(&b.full[s], SF_STAGE);
      tc::tma_load_2d(stages + s * SF_STAGE, map, kb * 64, row, &b.full[s]);
      *issued = ++it;
    }
  }
  return true;
}

// MMA issuer (one thread).
__device__ bool sf_mma(uint32_t tmem, uint32_t a0, uint8_t* stages, const SfBars& b, int tiles, int nc, int c0,
                       int c1) {
  const uint32_t idesc = tc::idesc_bf16(128, 256);
  uint32_t it = 0, local = 0;
  for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x, ++local) {
    if (local > 0) {  // both slots drained by the previous tile's output epilogue
      if (c0 && !sf_wait(&b.accempty[0], (local * c0 - 1) & 1, b.abort)) return false;
      if (c1 && !sf_wait(&b.accempty[1], (local * c1 - 1) & 1, b.abort)) return false;
    }
    if (!sf_wait(b.xfull, local & 1, b.abort)) return false;
    tc::tc_fence_after();
    for (int e = 0; e < 2 + 4 * SF_KB + nc * SF_KB; ++e) {
      uint32_t d, a;
      bool first;
      if (e < 2) {
        d = tmem + 256 * e, a = a0, first = true;
      } else if (e < 2 + 4 * SF_KB) {
        const int f = e - 2;
        if (f % (2 * SF_KB) == 0) {  // a new hidden layer: its A written and TMEM drained
          if (!sf_wait(b.edone, (local * 3 + f / (2 * SF_KB)) & 1, b.abort)) return false;
          tc::tc_fence_after();
        }
        const int kb = (f % (2 * SF_KB)) / 2;
        d = tmem + 256 * (f & 1), a = a0 + kb * 16384, first = kb == 0;
      } else {
        const int f = e - 2 - 4 * SF_KB, c = f / SF_KB, kb = f % SF_KB, sl = c & 1;
        if (f == 0) {  // the last hidden layer's activations are in A
          if (!sf_wait(b.edone, (local * 3 + 2) & 1, b.abort)) return false;
          tc::tc_fence_after();
        }
        if (kb == 0 && c >= 2) {  // chunk c - 2 of this slot drained
          const uint32_t done = (sl ? local * c1 : local * c0) + (c - 2) / 2;
          if (!sf_wait(&b.accempty[sl], done & 1, b.abort)) return false;
          tc::tc_fence_after();
        }
        d = tmem + 256 * sl, a = a0 + kb * 16384, first = kb == 0;
      }
      const uint32_t s = it % SF_STAGES;
      if (!sf_wait(&b.full[s], (it / SF_STAGES) & 1, b.abort)) return false;
      tc::tc_fence_after();
      const uint32_t bs = tc::smem_u32(stages + s * SF_STAGE);
#pragma unroll
      for (int k = 0; k < 4; ++k)
        tc::mma_bf16(d, tc::sdesc_sw128(a + 32 * k), tc::sdesc_sw128(bs + 32 * k), idesc, (!first || k > 0) ? 1u : 0u);
      tc::mma_commit(&b.empty[s]);
      ++it;
      // accumulators complete: after layer 1, after each hidden layer, after each output chunk
      if (e == 1 || (e >= 2 && e < 2 + 4 * SF_KB && (e - 2) % (2 * SF_KB) == 2 * SF_KB - 1)) {
        tc::mma_commit(&b.accfull[0]);
        tc::mma_commit(&b.accfull[1]);
      } else if (e >= 2 + 4 * SF_KB && (e - 2 - 4 * SF_KB) % SF_KB == SF_KB - 1) {
        tc::mma_commit(&b.accfull[((e - 2 - 4 * SF_KB) / SF_KB) & 1]);
      }
    }
    tc::mma_commit(b.afree);
  }
  return true;
}

// Epilogue warp (q, h, g): TMEM lanes 32q .. 32q + 31, column half h of a slot, column quarter 2h + g.
__device__ bool sf_epilogue(uint32_t tmem, uint8_t* abuf, const SfBars& b, const FusedArgs& args, int tiles, int nc,
                            int c0, int c1, int q, int h, int g) {
  const int lane = threadIdx.x & 31;
  const uint32_t lane_addr = (uint32_t)(q * 32) << 16;
  const int r = q * 32 + lane;  // row of the tile
  const int rot = blockIdx.x % nc;  // output chunks start at a different chunk on each CTA
  uint32_t local = 0;
  float v[32];
  for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x, ++local) {
    const int m = tile * 128 + r;
    const uint32_t f0 = local * (3 + c0), f1 = local * (3 + c1);  // accfull completions before this tile
    for (int layer = 0; layer < 3; ++layer) {  // hidden: slot h holds units 256h .. 256h + 255
      if (!sf_wait(&b.accfull[h], ((h ? f1 : f0) + layer) & 1, b.abort)) return false;
      tc::tc_fence_after();
      const float* bias = layer == 0 ? nullptr : (layer == 1 ? args.b2 : args.b3);
#pragma unroll 1
      for (int i = 0; i < 4; ++i) {  // columns 128g + 32i .. + 31 of this slot
        const int col = 256 * h + 128 * g + 32 * i;  // first unit of these 32
        float bb[32];                      // their biases: 16-byte loads issued before the accumulator read
#pragma unroll
        for (int q4 = 0; q4 < 8; ++q4) {
          const float4 t4 = bias ? __ldg(reinterpret_cast<const float4*>(bias + col) + q4) : make_float4(0, 0, 0, 0);
          bb[4 * q4] = t4.x, bb[4 * q4 + 1] = t4.y, bb[4 * q4 + 2] = t4.z, bb[4 * q4 + 3] = t4.w;
        }
        tc::tmem_ld32_sync(tmem + lane_addr + col, v);
        uint8_t* kblock = abuf + (col >> 6) * 16384;
#pragma unroll
        for (int ch = 0; ch < 4; ++ch) {
          float t[8];
#pragma unroll
          for (int j = 0; j < 8; ++j) t[j] = tc::tanh_fast(v[8 * ch + j] + bb[8 * ch + j]);
          const uint4 packed = make_uint4(tc::pack_bf16(t[0], t[1]), tc::pack_bf16(t[2], t[3]),
                                          tc::pack_bf16(t[4], t[5]), tc::pack_bf16(t[6], t[7]));
          *reinterpret_cast<uint4*>(kblock + tc::sw128_offset(r, (col & 63) + 8 * ch)) = packed;
        }
      }
      tc::fence_proxy_async_smem();
      tc::tc_fence_before();
      tc::mbar_arrive(b.edone);
    }
    float lo = 1.0f;
    const int nout = args.wout ? args.K : args.beams;  // outputs: world samples or beams
    int k0 = 0;  // world frame: the world sample of the car's beam 0
    if (args.wout && m < args.n) {
      float ph;
      k0 = world_phase(args.ray[args.n + m].x, args.ray[m].w, args.K, &ph);
    }
    for (int p = 0; p < nc; ++p) {  // output: p-th chunk in slot p & 1, this warp's 64 of its 256 columns
      const int s = p & 1, c = (p + rot) % nc;
      if (!sf_wait(&b.accfull[s], ((s ? f1 : f0) + 3 + p / 2) & 1, b.abort)) return false;
      tc::tc_fence_after();
#pragma unroll 1
      for (int i = 0; i < 2; ++i) {
        const int o0 = 256 * c + 128 * h + 64 * g + 32 * i;
        float bb[32];
        if (o0 + 32 <= nout) {
#pragma unroll
          for (int q4 = 0; q4 < 8; ++q4) {
            const float4 t4 = __ldg(reinterpret_cast<const float4*>(args.b4 + o0) + q4);
            bb[4 * q4] = t4.x, bb[4 * q4 + 1] = t4.y, bb[4 * q4 + 2] = t4.z, bb[4 * q4 + 3] = t4.w;
          }
        } else {
#pragma unroll
          for (int j = 0; j < 32; ++j) bb[j] = o0 + j < nout ? __ldg(args.b4 + o0 + j) : 0.0f;
        }
        tc::tmem_ld32_sync(tmem + lane_addr + 256 * s + 128 * h + 64 * g + 32 * i, v);
        if (args.wout) {
          if (m < args.n && o0 < args.ldw) {  // o0 is a multiple of 32, ldw of 64
            __half* row = args.wout + (long)m * args.ldw;
            lo = world_store16(v, bb, o0, args.K, k0, args.beams, row, lo);
            lo = world_store16(v + 16, bb + 16, o0 + 16, args.K, k0, args.beams, row, lo);
          }
        } else if (m < args.n) {
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const int o = o0 + j;
            if (o < args.beams) {
              const float y = __saturatef(v[j] + bb[j]);  // as EpiInfer: [0, 1], NaN to 0
              args.out[(long)o * args.n + m] = y;
              lo = fminf(lo, y);
            }
          }
        }
      }
      tc::tc_fence_before();
      tc::mbar_arrive(&b.accempty[s]);
    }
    if (m < args.n && args.minr) atomicMin(args.minr + m, __float_as_uint(lo));
  }
  return true;
}

__global__ void __launch_bounds__(SF_THREADS, 1)
    k_surrogate_fused(const __grid_constant__ CUtensorMap tx, const __grid_constant__ CUtensorMap tw1,
                      const __grid_constant__ CUtensorMap tw2, const __grid_constant__ CUtensorMap tw3,
                      const __grid_constant__ CUtensorMap tw4, FusedArgs args) {
  extern __shared__ uint8_t sf_raw[];
  const uint32_t raw = tc::smem_u32(sf_raw);
  uint8_t* smem = sf_raw + (((raw + 1023u) & ~1023u) - raw);
  uint8_t* abuf = smem;
  uint8_t* stages = smem + SF_A_BYTES;
  SfBars b;
  b.full = reinterpret_cast<uint64_t*>(stages + SF_STAGES * SF_STAGE);
  b.empty = b.full + SF_STAGES;
  b.xfull = b.empty + SF_STAGES;
  b.afree = b.xfull + 1;
  b.edone = b.afree + 1;
  b.accfull = b.edone + 1;     // [2]
  b.accempty = b.accfull + 2;  // [2]
  b.mdone = b.accempty + 2;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(b.mdone + 1);
  b.abort = reinterpret_cast<volatile int*>(tslot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tiles = (args.n + 127) / 128;
  const int nc = args.chunks, c0 = (nc + 1) / 2, c1 = nc / 2;  // output chunks in slot 0 / slot 1
  bool ok = true;

  if (threadIdx.x == 0) {
    for (int s = 0; s < SF_STAGES; ++s) {
      tc::mbar_init(&b.full[s], 1);
      tc::mbar_init(&b.empty[s], 1);
    }
    tc::mbar_init(b.xfull, 1);
    tc::mbar_init(b.afree, 1);
    tc::mbar_init(b.edone, SF_EPI);
    for (int s = 0; s < 2; ++s) {
      tc::mbar_init(&b.accfull[s], 1);
      tc::mbar_init(&b.accempty[s], SF_EPI);
    }
    tc::mbar_init(b.mdone, 1);
    *b.abort = 0;
    tc::fence_barrier_init();
  }
  if (warp == 1) {
    tc::tmem_alloc(tslot, 512);
    tc::tmem_relinquish();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tslot;

  if (warp == 0 && lane == 0) {
    uint32_t issued = 0, xloads = 0;
    ok = sf_producer(&tx, &tw1, &tw2, &tw3, &tw4, abuf, stages, b, tiles, nc, &issued, &xloads);
    // no copy may still be landing in shared memory when the CTA exits
    for (uint32_t it = issued > (uint32_t)SF_STAGES ? issued - SF_STAGES : 0; it < issued; ++it)
      tc::mbar_wait(&b.full[it % SF_STAGES], (it / SF_STAGES) & 1, 1u << 20);
    if (xloads) tc::mbar_wait(b.xfull, (xloads - 1) & 1, 1u << 20);
  } else if (warp == 1 && lane == 0) {
    ok = sf_mma(tmem, tc::smem_u32(abuf), stages, b, tiles, nc, c0, c1);
    tc::mma_commit(b.mdone);  // every MMA issued has completed before TMEM is freed
    tc::mbar_wait(b.mdone, 0, 1u << 20);
  } else if (warp >= 2) {
    const int k = (warp - 2) >> 2;  // 0..3 within the lane quarter warp & 3
    ok = sf_epilogue(tmem, abuf, b, args, tiles, nc, c0, c1, warp & 3, k >> 1, k & 1);
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 1) tc::tmem_dealloc(tmem, 512);
  if (!ok) atomicExch(args.err, 1);
}

cudaError_t surrogate_fused_launch(const CUtensorMap& tx, const CUtensorMap& tw1, const CUtensorMap& tw2,
                                   const CUtensorMap& tw3, const CUtensorMap& tw4, const FusedArgs& args, int sms,
                                   cudaStream_t st) {
  static unsigned long long configured = 0;  // per device
  cudaError_t e = once_per_device(&configured, [] {
    return cudaFuncSetAttribute(k_surrogate_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, SF_SMEM);
  });
  if (e != cudaSuccess) return e;
  const int tiles = (args.n + 127) / 128;
  k_surrogate_fused<<<tiles < sms ? tiles : sms, SF_THREADS, SF_SMEM, st>>>(tx, tw1, tw2, tw3, tw4, args);
  return cudaGetLastError();
}

}  // namespace
}  // namespace racer
