// Counter-based random numbers shared by the CUDA kernels and the host code.
//
// Philox4x32-10 as published by Salmon, Moraes, Dror and Shaw, "Parallel
// random numbers: as easy as 1, 2, 3" (SC'11): ten rounds of two 32x32->64
// multiplications with the Weyl key schedule. The reference draws its streams
// from Mojo's std.random.philox (`Random(seed, subsequence, offset)`,
// racer/sim.mojo:172,338 and racer/ppo.mojo:86); that module is not part of
// the reference checkout and no reference test pins its values, so this file
// fixes its own documented mapping, used identically on the GPU and the CPU:
//
//   key     = (seed & 0xffffffff, seed >> 32)
//   counter = (offset & 0xffffffff, offset >> 32,
//              subsequence & 0xffffffff, subsequence >> 32)
//   uniform u_j = ((x_j >> 9) + 0.5) * 2^-23, exact in binary32, in (0, 1)
//   normal  (z0, z1) = sqrt(-2 log u0) * (cos 2 pi u1, sin 2 pi u1),
//           (z2, z3) likewise from (u2, u3)            (Box-Muller)
//
// Every step is exact integer or IEEE binary32 arithmetic through rmath.h,
// so both sides produce the same bits.
#pragma once
#include <stdint.h>
#include "rmath.h"

namespace philox {

RM_HD void block(uint64_t seed, uint64_t subsequence, uint64_t offset, uint32_t out[4]) {
  uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  uint32_t c0 = (uint32_t)offset, c1 = (uint32_t)(offset >> 32);
  uint32_t c2 = (uint32_t)subsequence, c3 = (uint32_t)(subsequence >> 32);
  for (int round = 0; round < 10; ++round) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
    uint32_t n1 = (uint32_t)p1;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    uint32_t n3 = (uint32_t)p0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

RM_HD float to_uniform(uint32_t x) { return ((float)(x >> 9) + 0.5f) * 1.19209290e-07f; }

RM_HD void uniform4(uint64_t seed, uint64_t subsequence, uint64_t offset, float u[4]) {
  uint32_t x[4];
  block(seed, subsequence, offset, x);
  for (int j = 0; j < 4; ++j) u[j] = to_uniform(x[j]);
}

RM_HD void normal4(uint64_t seed, uint64_t subsequence, uint64_t offset, float z[4]) {
  float u[4];
  uniform4(seed, subsequence, offset, u);
  for (int j = 0; j < 4; j += 2) {
    float rho = sqrtf(-2.0f * rmath::logf_(u[j]));
    float s, c;
    rmath::sincosf_(6.28318548f * u[j + 1], &s, &c);
    z[j] = rho * c;
    z[j + 1] = rho * s;
  }
}

}  // namespace philox
