// tcgen05 policy forward (mlp_tc.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace racer {

// Optional Gaussian sampling fused into the forward's epilogue
// (racer/sim.mojo:337-346); disabled when actions is null.
struct SampleArgs {
  uint64_t seed = 0;
  const float* log_std = nullptr;
  float* actions = nullptr;
  float* logp = nullptr;
  float* value = nullptr;
  int deterministic = 0;
  const int64_t* step_base = nullptr;
  int64_t step_add = 0;
};

size_t mlp_pack_bytes(int in);
void launch_pack_weights(const float* theta, int in, uint8_t* pack, cudaStream_t st);
// Columns [c0, c1) of the [rows, cols] buffers (c1 < 0: all of them). A bounded wait that runs
// out sets *err; the kernel then issues no further copy or MMA, drains those it issued and returns
// (its outputs are undefined).
cudaError_t launch_mlp_fwd(const float* x, int in, int cols, const uint8_t* pack, float* h1, float* h2, float* o,
                           int write_hidden, const SampleArgs& sa, int* err, cudaStream_t st, int c0 = 0,
                           int c1 = -1);
// The timeout probe (k_wait_probe, one CTA): waits on an mbarrier nothing arrives on, at most
// `polls` polls, sets *err = 2, frees its tensor memory and returns.
cudaError_t launch_wait_probe(int* err, uint32_t polls, cudaStream_t st);

}  // namespace racer
