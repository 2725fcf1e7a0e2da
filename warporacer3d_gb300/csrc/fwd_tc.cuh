// The policy forward's tcgen05 epilogue (racer/ppo.mojo:40-44,108-111 layers 2
// and 3, and the sampling of racer/sim.mojo:337-346), shared by the forward
// kernels (mlp_tc.cu) and the fused rollout kernel (sim.cu): both translation
// units are built with --fmad=false, so either gives the same bits.
#pragma once
#include <cuda_bf16.h>

#include "common.cuh"
#include "mlp_tc.h"
#include "sample.cuh"
#include "tc.cuh"

namespace racer {
namespace {

constexpr int TILE = 128;
constexpr int A_BYTES = TILE * 128;  // 128 rows x 64 bf16
constexpr int B_BYTES = 64 * 128;    // 64 rows x 64 bf16

// Epilogues of the forward (warps 0-3: TMEM lanes 0-127 = sample rows), once
// layer 1's accumulator is complete (`done`, completion p0): tanh, H = [h | 1 | 0]
// as the next layer's A in stages 0-1 (the layer-1 stages, free by then),
// layers 2 and 3 issued by thread 0, the outputs and the fused sampling.
// After a timed-out wait (*abort set) thread 0 issues no more MMAs, the
// waits return at once and no warp reads the accumulator (which no MMA may
// have written); the results are then undefined and the error word set.
// *issued records whether this thread issued an MMA (the drain commits only then).
__device__ bool fwd_epilogue(uint8_t* smem, int OFF_A, int OFF_W1, int OFF_W2, uint32_t tmem, uint64_t* done,
                             uint32_t p0, int r, bool live, int c, int cols, float* h1g, float* h2g, float* og,
                             int write_hidden, const SampleArgs& sa, volatile int* abort, uint32_t limit,
                             bool* issued) {
  const int tid = threadIdx.x, warp = tid >> 5;
  bool ok = true;
  const uint32_t id64 = tc::idesc_bf16(TILE, 64), id16 = tc::idesc_bf16(TILE, 16);
  {
    const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
    uint8_t* Hs = smem + OFF_A;
    if (!tc::mbar_wait_abort(done, p0 & 1, abort, limit)) ok = false;
    __syncwarp();  // the TMEM loads are warp-collective
    tc::tc_fence_after();
    float acc[64];
    for (int layer = 0; layer < 2; ++layer) {
      if (!__any_sync(0xffffffffu, *abort != 0)) {  // warp-uniform: the loads are warp-collective
#pragma unroll
        for (int q = 0; q < 4; ++q) tc::tmem_ld16(trow + 16 * q, acc + 16 * q);
        tc::tmem_wait_ld();
      } else {
#pragma unroll
        for (int q = 0; q < 64; ++q) acc[q] = 0.0f;
      }
#pragma unroll
      for (int q = 0; q < 64; ++q) acc[q] = tc::tanh_fast(acc[q]);
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        uint4 pk = make_uint4(tc::pack_bf16(acc[8 * q], acc[8 * q + 1]), tc::pack_bf16(acc[8 * q + 2], acc[8 * q + 3]),
                              tc::pack_bf16(acc[8 * q + 4], acc[8 * q + 5]),
                              tc::pack_bf16(acc[8 * q + 6], acc[8 * q + 7]));
        *reinterpret_cast<uint4*>(Hs + r * 128 + ((q ^ (r & 7)) << 4)) = pk;
        uint4 hi = q == 0 ? make_uint4(tc::pack_bf16(1.0f, 0.0f), 0u, 0u, 0u) : make_uint4(0u, 0u, 0u, 0u);
        *reinterpret_cast<uint4*>(Hs + A_BYTES + r * 128 + ((q ^ (r & 7)) << 4)) = hi;
      }
      if (write_hidden && live) {
        float* hg = layer == 0 ? h1g : h2g;
#pragma unroll
        for (int q = 0; q < 64; ++q) hg[(long)q * cols + c] = acc[q];
      }
      tc::fence_proxy_async_smem();
      tc::tc_fence_before();
      tc::named_sync(1, TILE);
      if (tid == 0 && !*abort) {
        *issued = true;
        tc::tc_fence_after();
        const uint32_t h = tc::smem_u32(Hs);
        const uint32_t w = tc::smem_u32(smem + (layer == 0 ? OFF_W1 : OFF_W2));
        const uint32_t wstride = layer == 0 ? B_BYTES : 16 * 128;
#pragma unroll
        for (int kb = 0; kb < 2; ++kb)
#pragma unroll
          for (int k = 0; k < 4; ++k)
            tc::mma_bf16(tmem, tc::sdesc_sw128(h + kb * A_BYTES + 32 * k),
                         tc::sdesc_sw128(w + kb * wstride + 32 * k), layer == 0 ? id64 : id16, (kb | k) ? 1u : 0u);
        tc::mma_commit(done);
      }
      if (!tc::mbar_wait_abort(done, (p0 + 1 + layer) & 1, abort, limit)) ok = false;
      __syncwarp();
      tc::tc_fence_after();
    }
    float o[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    if (!__any_sync(0xffffffffu, *abort != 0)) {
      tc::tmem_ld4(trow, o);
      tc::tmem_wait_ld();
    }
    if (live) {
      og[c] = o[0];
      og[(long)cols + c] = o[1];
      og[2L * cols + c] = o[2];
      if (sa.actions) {
        int64_t step = (sa.step_base ? *sa.step_base : 0) + sa.step_add;
        sample_car(cols, c, sa.seed, o[0], o[1], o[2], sa.log_std, sa.actions, sa.logp, sa.value, sa.deterministic,
                   step);
      }
    }
  }
  return ok;
}

}  // namespace
}  // namespace racer
