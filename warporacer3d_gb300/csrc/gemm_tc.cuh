// Generic tcgen05 GEMM: D[M, N] = A[M, K] . B[N, K]^T with BF16 operands
// (both K-major, loaded by TMA as 128B-swizzled 64-wide k-blocks) and FP32
// accumulation in TMEM, followed by a caller-supplied epilogue.
//
// Persistent: one CTA per SM walks the 128 x BN output tiles (and split-K
// ranges) blockIdx.x, blockIdx.x + gridDim.x, ... Warp 0 is the TMA producer
// (a ring of stages across tiles), warp 1 allocates two TMEM accumulators and
// issues the MMAs (one thread), warps 2-9 are the epilogue: two warps per
// 32-lane TMEM quadrant, each taking half of the columns. The accumulator of
// tile i + 1 fills while the epilogue drains tile i. Every mbarrier wait is
// bounded and a timeout sets *err.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>

#include "tc.cuh"

namespace racer {
// Internal linkage: every translation unit that includes this header gets its
// own kernel instantiations and its own one-time attribute flag, so setting the
// shared-memory limit always reaches the module that launches the kernel.
namespace {

template <int BN>
struct GemmCfg {
  static constexpr int BM = 128;
  static constexpr int A_BYTES = BM * 128;
  static constexpr int B_BYTES = BN * 128;
  static constexpr int STAGES = BN >= 256 ? 4 : 6;
  static constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
  static constexpr int ACC_COLS = BN < 16 ? 16 : BN;
  static constexpr int TMEM_COLS = 2 * ACC_COLS < 32 ? 32 : 2 * ACC_COLS;
  static constexpr int SMEM = STAGES * STAGE_BYTES + 256 + 1024;
  static constexpr int EPI_WARPS = 8;
  static constexpr int THREADS = (2 + EPI_WARPS) * 32;
};

// Epilogue contract: operator()(m, n, v, z) with v[0..15] = D[m][n .. n+15] of split z, called
// by all 32 lanes of an epilogue warp together (lane = row); callers mask
// m >= M and n + j >= N themselves.
template <int BN, typename Epi>
__global__ void __launch_bounds__(GemmCfg<BN>::THREADS, 1)
    k_gemm(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, int mtiles, int ntiles,
           int splits, int kblocks, int kb_per_split, Epi epi, int* err) {
  using C = GemmCfg<BN>;
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = tc::smem_u32(smem_raw);
  uint8_t* smem = smem_raw + (((raw + 1023u) & ~1023u) - raw);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + C::STAGES * C::STAGE_BYTES);
  uint64_t* empty = full + C::STAGES;
  uint64_t* afull = empty + C::STAGES;  // [2] accumulator ready
  uint64_t* aempty = afull + 2;         // [2] accumulator drained
  uint32_t* tslot = reinterpret_cast<uint32_t*>(aempty + 2);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tiles = mtiles * ntiles * splits;
  bool ok = true;

  if (threadIdx.x == 0) {
    for (int s = 0; s < C::STAGES; ++s) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      tc::mbar_init(&afull[b], 1);
      tc::mbar_init(&aempty[b], C::EPI_WARPS * 32);
    }
    tc::fence_barrier_init();
  }
  if (warp == 1) {
    tc::tmem_alloc(tslot, C::TMEM_COLS);
    tc::tmem_relinquish();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tslot;

  if (warp == 0 && lane == 0) {
    uint32_t it = 0;
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
      const int nt = tile % ntiles, mt = (tile / ntiles) % mtiles, z = tile / (ntiles * mtiles);
      const int kb0 = z * kb_per_split, kb1 = min(kblocks, kb0 + kb_per_split);
      for (int kb = kb0; kb < kb1; ++kb, ++it) {
        const uint32_t s = it % C::STAGES;
        if (it >= (uint32_t)C::STAGES && !tc::mbar_wait(&empty[s], ((it / C::STAGES) - 1) & 1)) ok = false;
        uint8_t* st = smem + s * C::STAGE_BYTES;
        tc::mbar_arrive_expect_tx(&full[s], C::STAGE_BYTES);
        tc::tma_load_2d(st, &ta, kb * 64, mt * C::BM, &full[s]);
        tc::tma_load_2d(st + C::A_BYTES, &tb, kb * 64, nt * BN, &full[s]);
      }
    }
  } else if (warp == 1 && lane == 0) {
    const uint32_t idesc = tc::idesc_bf16(C::BM, BN);
    uint32_t it = 0, local = 0;
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x, ++local) {
      const int z = tile / (ntiles * mtiles);
      const int kb0 = z * kb_per_split, kb1 = min(kblocks, kb0 + kb_per_split);
      const uint32_t buf = local & 1, use = local >> 1;
      if (use >= 1 && !tc::mbar_wait(&aempty[buf], (use - 1) & 1)) ok = false;
      tc::tc_fence_after();
      const uint32_t d = tmem + buf * C::ACC_COLS;
      for (int kb = kb0; kb < kb1; ++kb, ++it) {
        const uint32_t s = it % C::STAGES;
        if (!tc::mbar_wait(&full[s], (it / C::STAGES) & 1)) ok = false;
        tc::tc_fence_after();
        const uint32_t a = tc::smem_u32(smem + s * C::STAGE_BYTES), b = a + C::A_BYTES;
#pragma unroll
        for (int k = 0; k < 4; ++k)
          tc::mma_bf16(d, tc::sdesc_sw128(a + 32 * k), tc::sdesc_sw128(b + 32 * k), idesc,
                       (kb > kb0 || k > 0) ? 1u : 0u);
        tc::mma_commit(&empty[s]);
      }
      tc::mma_commit(&afull[buf]);
    }
  } else if (warp >= 2) {
    const int q = warp & 3;                // TMEM lane quadrant
    const int half = (warp - 2) >> 2;      // which half of the columns
    constexpr int HALF = C::ACC_COLS / 2;  // >= 8
    uint32_t local = 0;
    for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x, ++local) {
      const int nt = tile % ntiles, mt = (tile / ntiles) % mtiles, z = tile / (ntiles * mtiles);
      const int kb0 = z * kb_per_split, kb1 = min(kblocks, kb0 + kb_per_split);
      const uint32_t buf = local & 1, use = local >> 1;
      if (!tc::mbar_wait(&afull[buf], use & 1)) ok = false;
      tc::tc_fence_after();
      const int m = mt * C::BM + q * 32 + lane;
      const uint32_t trow = tmem + buf * C::ACC_COLS + ((uint32_t)(q * 32) << 16);
      float v[32];
      if (HALF >= 32) {
#pragma unroll 1
        for (int c = half * HALF; c < (half + 1) * HALF; c += 32) {
          tc::tmem_ld32_sync(trow + c, v);
          if (kb1 <= kb0) {
#pragma unroll
            for (int j = 0; j < 32; ++j) v[j] = 0.0f;
          }
          epi(m, nt * BN + c, v, z);
          epi(m, nt * BN + c + 16, v + 16, z);
        }
      } else if (half == 0) {  // narrow tiles: the first warp of each quadrant takes all columns
#pragma unroll 1
        for (int c = 0; c < BN; c += 16) {
          tc::tmem_ld16(trow + c, v);
          tc::tmem_wait_ld();
          if (kb1 <= kb0) {
#pragma unroll
            for (int j = 0; j < 16; ++j) v[j] = 0.0f;
          }
          epi(m, nt * BN + c, v, z);
        }
      }
      tc::tc_fence_before();
      tc::mbar_arrive(&aempty[buf]);
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 1) tc::tmem_dealloc(tmem, C::TMEM_COLS);
  if (!ok) atomicExch(err, 1);
}

// Sets the kernel's shared-memory limit once per device (call before capturing a launch into a graph).
template <int BN, typename Epi>
cudaError_t gemm_configure() {
  static unsigned long long configured = 0;
  return once_per_device(&configured, [] {
    return cudaFuncSetAttribute(k_gemm<BN, Epi>, cudaFuncAttributeMaxDynamicSharedMemorySize, GemmCfg<BN>::SMEM);
  });
}

// Launch over an M x N output with K = kblocks * 64 split into `splits` ranges.
template <int BN, typename Epi>
cudaError_t gemm_launch(const CUtensorMap& ta, const CUtensorMap& tb, int M, int N, int kblocks, int splits,
                        const Epi& epi, int* err, cudaStream_t st) {
  using C = GemmCfg<BN>;
  cudaError_t ce = gemm_configure<BN, Epi>();
  if (ce != cudaSuccess) return ce;
  const int sms = device_sms();
  if (splits < 1) splits = 1;
  const int per = (kblocks + splits - 1) / splits;
  splits = (kblocks + per - 1) / per;
  const int mtiles = (M + C::BM - 1) / C::BM, ntiles = (N + BN - 1) / BN;
  const int tiles = mtiles * ntiles * splits;
  k_gemm<BN, Epi><<<tiles < sms ? tiles : sms, C::THREADS, C::SMEM, st>>>(ta, tb, mtiles, ntiles, splits, kblocks,
                                                                          per, epi, err);
  return cudaGetLastError();
}

}  // namespace
}  // namespace racer
