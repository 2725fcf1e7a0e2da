// Policy forward on the tcgen05 tensor cores (racer/ppo.mojo:108-111), BF16
// operands with FP32 accumulation in TMEM, all three layers fused per tile of
// 128 samples:
//
//   layer 1  D[128, 64]  = X^T[128, IN] . W0^T   (K = IN padded to 64k)
//   layer 2  D[128, 64]  = [h1 | 1][128, 128] . W1^T (K = 65 padded to 128)
//   layer 3  D[128, 16]  = [h2 | 1][128, 128] . W2^T (N = 3 padded to 16)
//
// X arrives feature-major FP32 [IN, cols] (the reference's layout); the CTA's
// four warps load it coalesced along the samples, convert to BF16 and store
// the transposed K-major tile into 128B-swizzled shared memory (two stages,
// overlapped with the MMAs of the previous k-block). W0 k-blocks and the
// whole of W1/W2 come from pre-swizzled BF16 copies made by k_pack_weights
// whenever theta changes. One thread issues the MMAs; tcgen05.commit signals
// an mbarrier; every thread then reads its row of the accumulator with
// tcgen05.ld, applies tanh and writes the next layer's operand. The last
// epilogue can sample the Gaussian actions in place (racer/sim.mojo:337-346),
// saving a launch per environment step.
//
// Built with --fmad=false so the fused sampling matches the standalone kernel.
#include <cuda_bf16.h>

#include "common.cuh"
#include "fwd_tc.cuh"
#include "mlp_tc.h"
#include "sample.cuh"
#include "tc.cuh"
#include "tma.h"

namespace racer {
namespace {


// GROUPS producer groups of four warps, one k-block in flight each (four for
// wide inputs; two when the input has at most four k-blocks, which halves the
// shared memory so two CTAs share an SM), plus one MMA warp.
template <int GROUPS>
struct FwdCfg {
  static constexpr int THREADS = (GROUPS * 4 + 1) * 32;
  static constexpr int MMA_WARP = GROUPS * 4;
  static constexpr int OFF_A = 0;  // GROUPS x A; H = [h | 1 | 0] reuses A[0], A[1]
  static constexpr int OFF_B = OFF_A + GROUPS * A_BYTES;
  static constexpr int OFF_W1 = OFF_B + GROUPS * B_BYTES;
  static constexpr int OFF_W2 = OFF_W1 + 2 * B_BYTES;
  static constexpr int OFF_BAR = OFF_W2 + 2 * 16 * 128;
  // + barriers, + alignment slack, + 16 KB so every descriptor-addressed read stays inside the allocation
  static constexpr int SMEM_BYTES = OFF_BAR + 128 + 1024 + 16384;
  static constexpr int MIN_BLOCKS = GROUPS == 2 ? 2 : 1;
  static_assert((2 * GROUPS + 3) * 8 + 8 <= 128, "barriers, the TMEM slot and the abort word fit their 128 bytes");
};


// Grid: one CTA per 128 samples. Warps 0-15 form four producer groups; group
// g loads k-blocks g, g+4, g+8, ... of X (thread = sample row) and of W0 into
// stage g, then arrives on full[g]. Warp 16 waits on full[kb % 4], issues the
// four K=16 MMAs of the block and commits to empty[kb % 4]; after the last
// block it commits to `done`. Warps 0-3 (TMEM lanes 0-127) then run the
// epilogues and issue layers 2 and 3.
template <int GROUPS>
__global__ void __launch_bounds__(FwdCfg<GROUPS>::THREADS, FwdCfg<GROUPS>::MIN_BLOCKS)
    k_mlp_fwd(const float* __restrict__ x, int in, int cols, int c0, int c1,
                                                        const uint4* __restrict__ w0s, int kblocks,
                                                        const uint4* __restrict__ w1s,
                                                        const uint4* __restrict__ w2s, float* h1g, float* h2g,
                                                        float* og, int write_hidden, SampleArgs sa, int* err) {
  using C = FwdCfg<GROUPS>;
  constexpr int THREADS = C::THREADS, MMA_WARP = C::MMA_WARP, OFF_A = C::OFF_A, OFF_B = C::OFF_B,
                OFF_W1 = C::OFF_W1, OFF_W2 = C::OFF_W2, OFF_BAR = C::OFF_BAR;
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = tc::smem_u32(smem_raw);
  uint8_t* smem = smem_raw + (((raw + 1023u) & ~1023u) - raw);
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + OFF_BAR);
  uint64_t* empty = full + GROUPS;
  uint64_t* done = empty + GROUPS;
  uint64_t* drain = done + 1;  // [2]: thread 0's and the MMA lane's final commits after a timeout
  uint32_t* tslot = reinterpret_cast<uint32_t*>(drain + 2);
  volatile int* abort = reinterpret_cast<volatile int*>(tslot + 1);  // set by a timed-out wait
  constexpr uint32_t limit = tc::WAIT_LIMIT;

  const int tid = threadIdx.x, warp = tid >> 5;
  const int r = tid & (TILE - 1);  // sample row of a producer or epilogue thread
  const int c = c0 + (int)blockIdx.x * TILE + r;  // column (sample) of the [rows, cols] buffers
  const bool live = c < c1;

  if (tid == 0) {
    for (int g = 0; g < GROUPS; ++g) {
      tc::mbar_init(&full[g], TILE);
      tc::mbar_init(&empty[g], 1);
    }
    tc::mbar_init(done, 1);
    tc::mbar_init(&drain[0], 1);
    tc::mbar_init(&drain[1], 1);
    *abort = 0;
    tc::fence_barrier_init();
  }
  if (warp == MMA_WARP) {
    tc::tmem_alloc(tslot, 64);
    tc::tmem_relinquish();
  }
  {  // W1 (2 x 8 KB) and W2 (2 x 2 KB), resident for the whole tile
    uint4* w1 = reinterpret_cast<uint4*>(smem + OFF_W1);
    uint4* w2 = reinterpret_cast<uint4*>(smem + OFF_W2);
    for (int e = tid; e < 2 * B_BYTES / 16; e += THREADS) w1[e] = __ldg(w1s + e);
    for (int e = tid; e < 2 * 16 * 128 / 16; e += THREADS) w2[e] = __ldg(w2s + e);
  }
  tc::fence_proxy_async_smem();
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tslot;
  const uint32_t id64 = tc::idesc_bf16(TILE, 64);
  bool ok = true;
  bool issued = false;  // this thread issued an MMA

  if (warp < MMA_WARP) {
    // ---- producers: layer-1 operands, one k-block per group in flight ----
    const int g = warp >> 2;
    uint8_t* A = smem + OFF_A + g * A_BYTES;
    uint4* B = reinterpret_cast<uint4*>(smem + OFF_B + g * B_BYTES);
    for (int j = 0;; ++j) {
      const int kb = g + GROUPS * j;
      if (kb >= kblocks) break;
      float v[64];
#pragma unroll
      for (int q = 0; q < 64; ++q) {
        const int f = kb * 64 + q;
        v[q] = (live && f < in) ? __ldg(x + (long)f * cols + c) : 0.0f;
      }
      uint4 wb[4];
      const uint4* src = w0s + (long)kb * (B_BYTES / 16);
#pragma unroll
      for (int e = 0; e < 4; ++e) wb[e] = __ldg(src + r + e * TILE);
      if (j >= 1 && !tc::mbar_wait_abort(&empty[g], (j - 1) & 1, abort, limit)) ok = false;
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        uint4 pk = make_uint4(tc::pack_bf16(v[8 * q], v[8 * q + 1]), tc::pack_bf16(v[8 * q + 2], v[8 * q + 3]),
                              tc::pack_bf16(v[8 * q + 4], v[8 * q + 5]), tc::pack_bf16(v[8 * q + 6], v[8 * q + 7]));
        *reinterpret_cast<uint4*>(A + r * 128 + ((q ^ (r & 7)) << 4)) = pk;
      }
#pragma unroll
      for (int e = 0; e < 4; ++e) B[r + e * TILE] = wb[e];
      tc::fence_proxy_async_smem();
      tc::mbar_arrive(&full[g]);
    }
  } else if ((tid & 31) == 0) {
    // ---- MMA issuer: layer 1 ----
    for (int kb = 0; kb < kblocks; ++kb) {
      const int g = kb % GROUPS;
      if (!tc::mbar_wait_abort(&full[g], (kb / GROUPS) & 1, abort, limit)) ok = false;
      if (*abort) continue;  // issue nothing after a timeout
      issued = true;
      tc::tc_fence_after();
      const uint32_t a = tc::smem_u32(smem + OFF_A + g * A_BYTES), b = tc::smem_u32(smem + OFF_B + g * B_BYTES);
#pragma unroll
      for (int k = 0; k < 4; ++k)
        tc::mma_bf16(tmem, tc::sdesc_sw128(a + 32 * k), tc::sdesc_sw128(b + 32 * k), id64, (kb | k) ? 1u : 0u);
      tc::mma_commit(&empty[g]);
    }
    if (!*abort) tc::mma_commit(done);
  }

  if (warp < 4 && !fwd_epilogue(smem, OFF_A, OFF_W1, OFF_W2, tmem, done, 0, r, live, c, cols, h1g, h2g, og,
                                  write_hidden, sa, abort, limit, &issued))
    ok = false;
  tc::tc_fence_before();
  __syncthreads();
  if (*abort) {  // the MMAs issued before the timeout complete before the TMEM is freed
    if (issued) {  // thread 0 and the MMA warp's lane 0, if they issued any, each on its own barrier
      uint64_t* mine = &drain[tid == 0 ? 0 : 1];
      tc::mma_commit(mine);
      if (!tc::mbar_wait(mine, 0, tc::WAIT_LIMIT)) ok = false;
    }
    tc::tc_fence_before();
    __syncthreads();
  }
  __syncwarp();
  if (warp == MMA_WARP) tc::tmem_dealloc(tmem, 64);
  if (!ok) atomicExch(err, 1);
}

// Forward with the inputs staged by TMA (wide inputs whose sample columns are
// 16-byte aligned), so the bytes in flight no longer sit in registers: warp
// 4's first thread streams each k-block of X as an FP32 box [64 features][128
// samples] into a ring of XS stages; warps 0-3 (thread = sample row) read
// their column of the box, arrive on xempty, pack it to BF16 into the swizzled
// A stage once that stage's previous MMAs completed, with the W0 k-block
// brought by a bulk copy that thread 0 starts (the stage's extra arrival), and
// arrive on afull; warp 5's first thread issues the MMAs and commits aempty.
// Features past `in` and samples past `cols` read zero, as the register
// path's loads do; samples of a box outside [c0, c1) are never written back.
// The epilogues are the register path's, so both give the same bits.
// PERSIST: CTA b takes tiles b, b + gridDim.x, ...; the rings' stages and
// parities run on across tiles, so the TMA warp loads the next tile's first
// boxes while warps 0-3 run this tile's epilogue. Layer 1 of the next tile
// starts only after those warps packed its first k-block, which follows their
// last read of this tile's accumulator; `done` completes three times a tile.
constexpr int XS = 3, XA = 3;
constexpr int X_BYTES = 64 * TILE * 4;
struct TmaCfg {
  static constexpr int THREADS = 6 * 32;
  static constexpr int OFF_A = 0;  // XA x A; H = [h | 1 | 0] reuses A[0], A[1]
  static constexpr int OFF_B = OFF_A + XA * A_BYTES;
  static constexpr int OFF_X = OFF_B + XA * B_BYTES;
  static constexpr int OFF_W1 = OFF_X + XS * X_BYTES;
  static constexpr int OFF_W2 = OFF_W1 + 2 * B_BYTES;
  static constexpr int OFF_BAR = OFF_W2 + 2 * 16 * 128;
  // + barriers, + alignment slack, + 16 KB so every descriptor-addressed read stays inside the allocation
  static constexpr int SMEM_BYTES = OFF_BAR + 256 + 1024 + 16384;
};
static_assert(TmaCfg::SMEM_BYTES <= 227 * 1024, "one CTA per SM");
static_assert((2 * XS + 2 * XA + 3) * 8 + 8 <= 256, "barriers, the TMEM slot and the abort word fit their 256 bytes");

template <bool PERSIST>
__global__ void __launch_bounds__(TmaCfg::THREADS, 1)
    k_mlp_fwd_tma(const __grid_constant__ CUtensorMap xmap, int cols, int c0, int c1, const uint4* __restrict__ w0s,
                  int kblocks, const uint4* __restrict__ w1s, const uint4* __restrict__ w2s, float* h1g, float* h2g,
                  float* og, int write_hidden, SampleArgs sa, int* err) {
  using C = TmaCfg;
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = tc::smem_u32(smem_raw);
  uint8_t* smem = smem_raw + (((raw + 1023u) & ~1023u) - raw);
  uint64_t* xfull = reinterpret_cast<uint64_t*>(smem + C::OFF_BAR);
  uint64_t* xempty = xfull + XS;
  uint64_t* afull = xempty + XS;
  uint64_t* aempty = afull + XA;
  uint64_t* done = aempty + XA;
  uint64_t* drain = done + 1;  // [2]: thread 0's and the MMA lane's final commits after a timeout
  uint32_t* tslot = reinterpret_cast<uint32_t*>(drain + 2);
  volatile int* abort = reinterpret_cast<volatile int*>(tslot + 1);  // set by a timed-out wait
  constexpr uint32_t limit = tc::WAIT_LIMIT;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int r = tid & (TILE - 1);
  const int tiles = (c1 - c0 + TILE - 1) / TILE;
  const int stride = PERSIST ? (int)gridDim.x : tiles;  // one tile per CTA unless persistent

  if (tid == 0) {
    for (int s = 0; s < XS; ++s) {
      tc::mbar_init(&xfull[s], 1);
      tc::mbar_init(&xempty[s], TILE);
    }
    for (int s = 0; s < XA; ++s) {
      tc::mbar_init(&afull[s], TILE + 1);
      tc::mbar_init(&aempty[s], 1);
    }
    tc::mbar_init(done, 1);
    tc::mbar_init(&drain[0], 1);
    tc::mbar_init(&drain[1], 1);
    *abort = 0;
    tc::fence_barrier_init();
  }
  if (warp == 5) {
    tc::tmem_alloc(tslot, 64);
    tc::tmem_relinquish();
  }
  {  // W1 (2 x 8 KB) and W2 (2 x 2 KB), resident for the whole tile
    uint4* w1 = reinterpret_cast<uint4*>(smem + C::OFF_W1);
    uint4* w2 = reinterpret_cast<uint4*>(smem + C::OFF_W2);
    for (int e = tid; e < 2 * B_BYTES / 16; e += C::THREADS) w1[e] = __ldg(w1s + e);
    for (int e = tid; e < 2 * 16 * 128 / 16; e += C::THREADS) w2[e] = __ldg(w2s + e);
  }
  tc::fence_proxy_async_smem();
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tslot;
  bool ok = true;
  bool issued = false;   // this thread issued an MMA
  uint32_t w0_last = 0;  // thread 0: W0 copies issued (the stage of copy k is k % XA)

  if (warp == 4) {
    if (lane == 0) {  // ---- X boxes ----
      uint32_t it = 0;  // boxes issued
      for (int tile = blockIdx.x; tile < tiles; tile += stride) {
        for (int kb = 0; kb < kblocks; ++kb) {
          const uint32_t s = it % XS;
          if (it >= (uint32_t)XS && !tc::mbar_wait_abort(&xempty[s], ((it / XS) - 1) & 1, abort, limit)) ok = false;
          if (*abort) break;  // issue nothing after a timeout
          tc::mbar_arrive_expect_tx(&xfull[s], X_BYTES);
          tc::tma_load_2d(smem + C::OFF_X + s * X_BYTES, &xmap, c0 + tile * TILE, kb * 64, &xfull[s]);
          ++it;
        }
        if (*abort) break;
      }
      // no copy may still be landing in shared memory when the CTA exits: the
      // last box of each stage completes its phase with this thread's own
      // arrival and the bytes, whatever the other warps did
      for (uint32_t k = it > (uint32_t)XS ? it - XS : 0; k < it; ++k)
        if (!tc::mbar_wait(&xfull[k % XS], (k / XS) & 1, tc::WAIT_LIMIT)) ok = false;
    }
  } else if (warp == 5) {
    if (lane == 0) {  // ---- MMA issuer: layer 1 ----
      const uint32_t id64 = tc::idesc_bf16(TILE, 64);
      uint32_t it = 0;
      for (int tile = blockIdx.x; tile < tiles; tile += stride) {
        for (int kb = 0; kb < kblocks; ++kb, ++it) {
          const uint32_t a = it % XA;
          if (!tc::mbar_wait_abort(&afull[a], (it / XA) & 1, abort, limit)) ok = false;
          if (*abort) continue;  // issue nothing after a timeout
          issued = true;
          tc::tc_fence_after();
          const uint32_t sa_ = tc::smem_u32(smem + C::OFF_A + a * A_BYTES);
          const uint32_t sb = tc::smem_u32(smem + C::OFF_B + a * B_BYTES);
#pragma unroll
          for (int k = 0; k < 4; ++k)
            tc::mma_bf16(tmem, tc::sdesc_sw128(sa_ + 32 * k), tc::sdesc_sw128(sb + 32 * k), id64, (kb | k) ? 1u : 0u);
          tc::mma_commit(&aempty[a]);
        }
        if (!*abort) tc::mma_commit(done);
      }
    }
  } else {
    // ---- warps 0-3: BF16 operands of layer 1, then the epilogues ----
    const float* X = reinterpret_cast<const float*>(smem + C::OFF_X);
    uint32_t it = 0, t = 0;
    for (int tile = blockIdx.x; tile < tiles; tile += stride, ++t) {
      for (int kb = 0; kb < kblocks; ++kb, ++it) {
        const uint32_t s = it % XS, a = it % XA;
        if (!tc::mbar_wait_abort(&xfull[s], (it / XS) & 1, abort, limit)) ok = false;
        const float* box = X + s * (X_BYTES / 4);
        float v[64];
#pragma unroll
        for (int q = 0; q < 64; ++q) v[q] = box[q * TILE + r];
        tc::mbar_arrive(&xempty[s]);
        if (it >= (uint32_t)XA && !tc::mbar_wait_abort(&aempty[a], ((it / XA) - 1) & 1, abort, limit)) ok = false;
        uint8_t* A = smem + C::OFF_A + a * A_BYTES;
        if (r == 0 && !*abort) {  // the stage is free: announce and start the W0 copy
          tc::mbar_arrive_expect_tx(&afull[a], B_BYTES);
          tc::bulk_load(smem + C::OFF_B + a * B_BYTES, w0s + (long)kb * (B_BYTES / 16), B_BYTES, &afull[a]);
          w0_last = it + 1;
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          uint4 pk = make_uint4(tc::pack_bf16(v[8 * q], v[8 * q + 1]), tc::pack_bf16(v[8 * q + 2], v[8 * q + 3]),
                                tc::pack_bf16(v[8 * q + 4], v[8 * q + 5]), tc::pack_bf16(v[8 * q + 6], v[8 * q + 7]));
          *reinterpret_cast<uint4*>(A + r * 128 + ((q ^ (r & 7)) << 4)) = pk;
        }
        tc::fence_proxy_async_smem();
        if (kb == 0 && t > 0) tc::tc_fence_before();  // after the previous tile's accumulator reads
        tc::mbar_arrive(&afull[a]);
      }
      const int c = c0 + tile * TILE + r;
      if (!fwd_epilogue(smem, C::OFF_A, C::OFF_W1, C::OFF_W2, tmem, done, 3 * t, r, c < c1, c, cols, h1g, h2g, og,
                        write_hidden, sa, abort, limit, &issued))
        ok = false;
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (*abort) {
    // After a timeout every thread has made all its arrivals, so the phases
    // of thread 0's last W0 copies complete once their bytes land; and the
    // MMAs issued before the timeout complete before the TMEM is freed.
    if (tid == 0)
      for (uint32_t k = w0_last > (uint32_t)XA ? w0_last - XA : 0; k < w0_last; ++k)
        if (!tc::mbar_wait(&afull[k % XA], (k / XA) & 1, tc::WAIT_LIMIT)) ok = false;
    if (issued) {  // thread 0 and the MMA warp's lane 0, if they issued any, each on its own barrier
      uint64_t* mine = &drain[tid == 0 ? 0 : 1];
      tc::mma_commit(mine);
      if (!tc::mbar_wait(mine, 0, tc::WAIT_LIMIT)) ok = false;
    }
    tc::tc_fence_before();
    __syncthreads();
  }
  __syncwarp();
  if (warp == 5) tc::tmem_dealloc(tmem, 64);
  if (!ok) atomicExch(err, 1);
}

// theta -> pre-swizzled BF16 operand images: W0 [kblocks][64 x 64], W1 [2][64 x 64] (K = 65 padded),
// W2 [2][16 x 64] (rows 3..15 and K >= 65 zero).
__global__ void k_pack_weights(const float* __restrict__ theta, int in, int kblocks, __nv_bfloat16* w0s,
                               __nv_bfloat16* w1s, __nv_bfloat16* w2s) {
  const long n0 = (long)kblocks * 64 * 64, n1 = 2L * 64 * 64, n2 = 2L * 16 * 64;
  const int w1 = H * in, w2 = w1 + H * HA;
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < n0 + n1 + n2; e += (long)gridDim.x * blockDim.x) {
    if (e < n0) {
      int kb = (int)(e / 4096), r = (int)((e / 64) % 64), kk = (int)(e % 64), k = kb * 64 + kk;
      float v = k < in ? theta[(long)r * in + k] : 0.0f;
      w0s[((long)kb * 8192 + tc::sw128_offset(r, kk)) / 2] = __float2bfloat16_rn(v);
    } else if (e < n0 + n1) {
      long f = e - n0;
      int kb = (int)(f / 4096), r = (int)((f / 64) % 64), kk = (int)(f % 64), k = kb * 64 + kk;
      float v = k < HA ? theta[w1 + r * HA + k] : 0.0f;
      w1s[((long)kb * 8192 + tc::sw128_offset(r, kk)) / 2] = __float2bfloat16_rn(v);
    } else {
      long f = e - n0 - n1;
      int kb = (int)(f / 1024), r = (int)((f / 64) % 16), kk = (int)(f % 64), k = kb * 64 + kk;
      float v = (r < OUT && k < HA) ? theta[w2 + r * HA + k] : 0.0f;
      w2s[((long)kb * 2048 + tc::sw128_offset(r, kk)) / 2] = __float2bfloat16_rn(v);
    }
  }
}

// Timeout probe: a tensor-core kernel (it holds tensor memory) whose every
// thread waits on an mbarrier that nothing will ever arrive on, `polls` polls
// at most (or until another thread's wait ran out). It issues no copy, no MMA
// and no tensor-memory load; the timed-out wait sets *err, the tensor memory
// is freed and the kernel returns, as in the forward kernels' timeout path.
__global__ void __launch_bounds__(128, 1) k_wait_probe(int* err, uint32_t polls) {
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t slot;
  __shared__ int abort;
  const int tid = threadIdx.x;
  if (tid == 0) {
    tc::mbar_init(&bar, 1);
    abort = 0;
    tc::fence_barrier_init();
  }
  if (tid < 32) {
    tc::tmem_alloc(&slot, 32);
    tc::tmem_relinquish();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = slot;
  const bool ok = tc::mbar_wait_abort(&bar, 0, &abort, polls);
  tc::tc_fence_before();
  __syncthreads();
  if (tid < 32) tc::tmem_dealloc(tmem, 32);
  if (!ok) atomicExch(err, 2);
}

}  // namespace

cudaError_t launch_wait_probe(int* err, uint32_t polls, cudaStream_t st) {
  k_wait_probe<<<1, 128, 0, st>>>(err, polls);
  return cudaGetLastError();
}

size_t mlp_pack_bytes(int in) {
  int kb = (in + 63) / 64;
  return (size_t)kb * 8192 + 2 * 8192 + 2 * 2048;
}

void launch_pack_weights(const float* theta, int in, uint8_t* pack, cudaStream_t st) {
  int kb = (in + 63) / 64;
  auto* w0 = reinterpret_cast<__nv_bfloat16*>(pack);
  auto* w1 = reinterpret_cast<__nv_bfloat16*>(pack + (size_t)kb * 8192);
  auto* w2 = reinterpret_cast<__nv_bfloat16*>(pack + (size_t)kb * 8192 + 2 * 8192);
  k_pack_weights<<<device_sms(), 256, 0, st>>>(theta, in, kb, w0, w1, w2);
}

template <int GROUPS>
static cudaError_t fwd_launch(const float* x, int in, int cols, int c0, int c1, int kb, const uint4* w0,
                              const uint4* w1, const uint4* w2, float* h1, float* h2, float* o, int write_hidden,
                              const SampleArgs& sa, int* err, cudaStream_t st) {
  using C = FwdCfg<GROUPS>;
  static unsigned long long configured = 0;  // per device
  cudaError_t e = once_per_device(&configured, [] {
    return cudaFuncSetAttribute(k_mlp_fwd<GROUPS>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM_BYTES);
  });
  if (e != cudaSuccess) return e;
  if (c1 <= c0) return cudaSuccess;
  k_mlp_fwd<GROUPS><<<(c1 - c0 + TILE - 1) / TILE, C::THREADS, C::SMEM_BYTES, st>>>(x, in, cols, c0, c1, w0, kb, w1, w2,
                                                                                  h1, h2, o, write_hidden, sa, err);
  return cudaGetLastError();
}

cudaError_t launch_mlp_fwd(const float* x, int in, int cols, const uint8_t* pack, float* h1, float* h2, float* o,
                           int write_hidden, const SampleArgs& sa, int* err, cudaStream_t st, int c0, int c1) {
  if (c1 < 0) c1 = cols;
  int kb = (in + 63) / 64;
  const uint4* w0 = reinterpret_cast<const uint4*>(pack);
  const uint4* w1 = reinterpret_cast<const uint4*>(pack + (size_t)kb * 8192);
  const uint4* w2 = reinterpret_cast<const uint4*>(pack + (size_t)kb * 8192 + 2 * 8192);
  if (kb <= 4) return fwd_launch<2>(x, in, cols, c0, c1, kb, w0, w1, w2, h1, h2, o, write_hidden, sa, err, st);
  // wide inputs: X staged by TMA where its sample columns are 16-byte aligned
  CUtensorMap xmap;
  if (c1 > c0 && (cols & 3) == 0 && (c0 & 3) == 0 && (reinterpret_cast<uintptr_t>(x) & 15) == 0 &&
      make_tmap_f32(&xmap, x, (uint64_t)in, (uint64_t)cols, (uint64_t)cols, TILE, 64) == 0) {
    static unsigned long long configured = 0;  // per device
    cudaError_t e = once_per_device(&configured, [] {
      for (auto* k : {k_mlp_fwd_tma<false>, k_mlp_fwd_tma<true>}) {
        cudaError_t a = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, TmaCfg::SMEM_BYTES);
        if (a != cudaSuccess) return a;
      }
      return cudaSuccess;
    });
    if (e != cudaSuccess) return e;
    const int sms = device_sms();
    // more tiles than SMs: one persistent CTA per SM, each running ahead into its next tile
    const int tiles = (c1 - c0 + TILE - 1) / TILE;
    if (sms > 0 && tiles > sms)
      k_mlp_fwd_tma<true><<<sms, TmaCfg::THREADS, TmaCfg::SMEM_BYTES, st>>>(xmap, cols, c0, c1, w0, kb, w1, w2, h1, h2,
                                                                           o, write_hidden, sa, err);
    else
      k_mlp_fwd_tma<false><<<tiles, TmaCfg::THREADS, TmaCfg::SMEM_BYTES, st>>>(xmap, cols, c0, c1, w0, kb, w1, w2, h1,
                                                                             h2, o, write_hidden, sa, err);
    return cudaGetLastError();
  }
  return fwd_launch<4>(x, in, cols, c0, c1, kb, w0, w1, w2, h1, h2, o, write_hidden, sa, err, st);
}

}  // namespace racer
