// Gaussian action sampling for one car (racer/sim.mojo:337-346), shared by the
// standalone sample kernel and the fused policy epilogue. Both translation
// units are built with --fmad=false, so the two paths produce the same bits.
#pragma once
#include "common.cuh"
#include "philox.h"
#include "rmath.h"

namespace racer {

__device__ __forceinline__ void sample_car(int n, int i, uint64_t seed, float mu0, float mu1, float v,
                                           const float* log_std, float* actions, float* logp, float* value,
                                           int deterministic, int64_t step) {
  float noise[4];
  philox::normal4(seed + 1, (uint64_t)i, (uint64_t)step, noise);
  float probability = 0.0f;
  float mu[2] = {mu0, mu1};
  for (int a = 0; a < 2; ++a) {
    float z = deterministic ? 0.0f : noise[a];
    float ls = log_std[a];
    actions[(long)a * n + i] = mu[a] + rmath::expf_(ls) * z;
    probability -= ((0.5f * z) * z + ls) + HALF_LOG_2PI;
  }
  logp[i] = probability;
  value[i] = v;
}

}  // namespace racer
