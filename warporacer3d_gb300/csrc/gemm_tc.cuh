// Generic tcgen05 GEMM: D[M, N] = A[M, K] . B[N, K]^T with BF16 operands
// (both K-major, loaded by TMA as 128B-swizzled 64-wide k-blocks) and FP32
// accumulation in TMEM, followed by a caller-supplied epilogue.
//
// One CTA computes a 128 x BN tile over the k-blocks of its split
// (blockIdx.z): warp 0 is the TMA producer, warp 1 allocates TMEM and issues
// the MMAs (one thread), warps 2-5 read the accumulator (each its own 32-lane
// TMEM quadrant, so together all 128 rows) and call the epilogue on chunks of
// 16 consecutive columns of one row. Stages ping through full/empty mbarriers;
// every wait is bounded and a timeout sets *err.
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
  static constexpr int TMEM_COLS = BN < 32 ? 32 : BN;
  static constexpr int SMEM = STAGES * STAGE_BYTES + 256 + 1024;
  static constexpr int THREADS = 192;
};

// Epilogue contract: operator()(m, n, v) with v[0..15] = D[m][n .. n+15]
// (callers mask m >= M and n + j >= N themselves).
template <int BN, typename Epi>
__global__ void __launch_bounds__(192, 1)
    k_gemm(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, int kblocks,
           int kb_per_split, Epi epi, int* err) {
  using C = GemmCfg<BN>;
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = tc::smem_u32(smem_raw);
  uint8_t* smem = smem_raw + (((raw + 1023u) & ~1023u) - raw);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + C::STAGES * C::STAGE_BYTES);
  uint64_t* empty = full + C::STAGES;
  uint64_t* accum = empty + C::STAGES;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(accum + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * C::BM, n0 = blockIdx.y * BN;
  const int kb0 = blockIdx.z * kb_per_split;
  const int kb1 = min(kblocks, kb0 + kb_per_split);
  const int nk = kb1 - kb0;
  bool ok = true;

  if (threadIdx.x == 0) {
    for (int s = 0; s < C::STAGES; ++s) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    tc::mbar_init(accum, 1);
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
    for (int i = 0; i < nk; ++i) {
      const int s = i % C::STAGES;
      if (i >= C::STAGES && !tc::mbar_wait(&empty[s], ((i / C::STAGES) - 1) & 1)) ok = false;
      uint8_t* st = smem + s * C::STAGE_BYTES;
      tc::mbar_arrive_expect_tx(&full[s], C::STAGE_BYTES);
      tc::tma_load_2d(st, &ta, (kb0 + i) * 64, m0, &full[s]);
      tc::tma_load_2d(st + C::A_BYTES, &tb, (kb0 + i) * 64, n0, &full[s]);
    }
  } else if (warp == 1 && lane == 0) {
    const uint32_t idesc = tc::idesc_bf16(C::BM, BN);
    for (int i = 0; i < nk; ++i) {
      const int s = i % C::STAGES;
      if (!tc::mbar_wait(&full[s], (i / C::STAGES) & 1)) ok = false;
      tc::tc_fence_after();
      const uint32_t a = tc::smem_u32(smem + s * C::STAGE_BYTES), b = a + C::A_BYTES;
#pragma unroll
      for (int k = 0; k < 4; ++k)
        tc::mma_bf16(tmem, tc::sdesc_sw128(a + 32 * k), tc::sdesc_sw128(b + 32 * k), idesc, (i | k) ? 1u : 0u);
      tc::mma_commit(&empty[s]);
    }
    tc::mma_commit(accum);
  } else if (warp >= 2) {
    const int q = warp & 3;  // TMEM lane quadrant of this warp
    const int m = m0 + q * 32 + lane;
    if (!tc::mbar_wait(accum, 0)) ok = false;
    tc::tc_fence_after();
    const uint32_t trow = tmem + ((uint32_t)(q * 32) << 16);
    float v[16];
#pragma unroll 1
    for (int c = 0; c < BN; c += 16) {
      tc::tmem_ld16(trow + c, v);
      tc::tmem_wait_ld();
      if (nk <= 0) {
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] = 0.0f;
      }
      epi(m, n0 + c, v);
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 1) tc::tmem_dealloc(tmem, C::TMEM_COLS);
  if (!ok) atomicExch(err, 1);
}

// Sets the kernel's shared-memory limit once (call before capturing a launch into a graph).
template <int BN, typename Epi>
cudaError_t gemm_configure() {
  static bool configured = false;
  if (!configured) {
    cudaError_t e =
        cudaFuncSetAttribute(k_gemm<BN, Epi>, cudaFuncAttributeMaxDynamicSharedMemorySize, GemmCfg<BN>::SMEM);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  return cudaSuccess;
}

// Launch over an M x N output with K = kblocks * 64 split into `splits` ranges.
template <int BN, typename Epi>
cudaError_t gemm_launch(const CUtensorMap& ta, const CUtensorMap& tb, int M, int N, int kblocks, int splits,
                        const Epi& epi, int* err, cudaStream_t st) {
  using C = GemmCfg<BN>;
  cudaError_t ce = gemm_configure<BN, Epi>();
  if (ce != cudaSuccess) return ce;
  if (splits < 1) splits = 1;
  const int per = (kblocks + splits - 1) / splits;
  splits = (kblocks + per - 1) / per;
  dim3 grid((M + C::BM - 1) / C::BM, (N + BN - 1) / BN, splits);
  k_gemm<BN, Epi><<<grid, C::THREADS, C::SMEM, st>>>(ta, tb, kblocks, per, epi, err);
  return cudaGetLastError();
}

}  // namespace
}  // namespace racer
