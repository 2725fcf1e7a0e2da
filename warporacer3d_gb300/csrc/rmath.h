// Deterministic single-precision elementary functions shared by the CUDA
// kernels and the host code.
//
// Every function here is a fixed sequence of IEEE-754 binary32 additions,
// multiplications, divisions and square roots (no fused multiply-add, no
// hardware approximations), so a build with contraction disabled
// (nvcc --fmad=false, gcc -ffp-contract=off) returns bit-identical results on
// sm_103a, x86-64 and aarch64. That is what lets the simulator's integer
// outputs (layer, nearest waypoint, crash flags) and its lidar ranges match a
// CPU restatement exactly instead of within a tolerance.
//
// Methods (all from the open literature, coefficients derived here):
//  * sin/cos: Cody & Waite argument reduction by pi/2 (W. J. Cody, W. Waite,
//    "Software Manual for the Elementary Functions", 1980) with a three-part
//    split of pi/2, then the Taylor series of sin to x^9 and of cos to x^10 on
//    |r| <= pi/4 (truncation error below 2^-28).
//  * exp: reduction x = k ln2 + r (two-part split of ln2), Taylor series of
//    e^r to r^8 on |r| <= ln2/2, exact scaling by 2^k.
//  * log: x = m 2^e with m in [sqrt(1/2), sqrt(2)), log m = 2 atanh(s),
//    s = (m-1)/(m+1), odd series to s^11.
// Accuracy against a double-precision libm is checked by the host tests
// (a few ulp over the ranges the simulator uses).
#pragma once
#include <stdint.h>
#include <math.h>

#if defined(__CUDACC__)
#define RM_HD __host__ __device__ __forceinline__
#else
#define RM_HD static inline
#endif

namespace rmath {

RM_HD float from_bits(uint32_t u) {
  union { uint32_t u; float f; } v;
  v.u = u;
  return v.f;
}
RM_HD uint32_t to_bits(float f) {
  union { uint32_t u; float f; } v;
  v.f = f;
  return v.u;
}

// pi/2 = PIO2_A + PIO2_B + PIO2_C; A and B carry 12 significant bits each, so
// k * A and k * B are exact for |k| < 2^12.
#define RM_PIO2_A 1.570312500e+00f   // 0x3FC90000
#define RM_PIO2_B 4.837512970e-04f   // 0x39FDA000
#define RM_PIO2_C 7.549790126e-08f   // 0x33A22169, remainder rounded
#define RM_TWO_OVER_PI 0.636619772f

// Polynomial kernels on |r| <= pi/4 (r2 = r*r).
RM_HD float sin_kernel(float r, float r2) {
  const float s1 = -1.0f / 6.0f, s2 = 1.0f / 120.0f, s3 = -1.0f / 5040.0f, s4 = 1.0f / 362880.0f;
  float p = s3 + r2 * s4;
  p = s2 + r2 * p;
  p = s1 + r2 * p;
  return r + (r * r2) * p;
}
RM_HD float cos_kernel(float r2) {
  const float c1 = 1.0f / 24.0f, c2 = -1.0f / 720.0f, c3 = 1.0f / 40320.0f, c4 = -1.0f / 3628800.0f;
  float p = c3 + r2 * c4;
  p = c2 + r2 * p;
  p = c1 + r2 * p;
  return 1.0f - (0.5f * r2 - (r2 * r2) * p);
}

// sin and cos of x together for |x| <= RM_SINCOS_MAX; larger inputs (outside
// anything the simulator produces) and NaN return NaN. The bound keeps the
// quadrant |k| = rint(|x| 2/pi) <= 4092 < 2^12, where k * PIO2_A and
// k * PIO2_B are exact: beyond it the reduction would lose bits silently.
#define RM_SINCOS_MAX 6426.0f
RM_HD void sincosf_(float x, float* s, float* c) {
  if (!(fabsf(x) <= RM_SINCOS_MAX)) {
    *s = *c = x - x + from_bits(0x7fc00000u);
    return;
  }
  float kf = rintf(x * RM_TWO_OVER_PI);
  int k = (int)kf;
  float r = ((x - kf * RM_PIO2_A) - kf * RM_PIO2_B) - kf * RM_PIO2_C;
  float r2 = r * r;
  float sr = sin_kernel(r, r2), cr = cos_kernel(r2);
  switch (k & 3) {
    case 0: *s = sr; *c = cr; break;
    case 1: *s = cr; *c = -sr; break;
    case 2: *s = -sr; *c = -cr; break;
    default: *s = -cr; *c = sr; break;
  }
}
RM_HD float sinf_(float x) { float s, c; sincosf_(x, &s, &c); return s; }
RM_HD float cosf_(float x) { float s, c; sincosf_(x, &s, &c); return c; }

// ln2 = LN2_A + LN2_B; LN2_A has 16 significant bits, so k * LN2_A is exact
// for |k| < 2^8.
#define RM_LN2_A 6.931457520e-01f    // 0x3F317200
#define RM_LN2_B 1.428606765e-06f    // 0x35BFBE8E, remainder rounded
#define RM_LOG2E 1.44269504f

RM_HD float ldexp_small(float p, int k) {  // p * 2^k for -252 < k < 254, exact unless subnormal
  int k1 = k / 2, k2 = k - k1;
  return (p * from_bits((uint32_t)(k1 + 127) << 23)) * from_bits((uint32_t)(k2 + 127) << 23);
}

RM_HD float expf_(float x) {
  if (x != x) return x;
  if (x > 88.7228394f) return from_bits(0x7f800000u);
  if (x < -103.972084f) return 0.0f;
  float kf = rintf(x * RM_LOG2E);
  int k = (int)kf;
  float r = (x - kf * RM_LN2_A) - kf * RM_LN2_B;
  float p = 1.0f / 40320.0f;
  p = 1.0f / 5040.0f + r * p;
  p = 1.0f / 720.0f + r * p;
  p = 1.0f / 120.0f + r * p;
  p = 1.0f / 24.0f + r * p;
  p = 1.0f / 6.0f + r * p;
  p = 0.5f + r * p;
  p = 1.0f + r * p;
  p = 1.0f + r * p;
  return ldexp_small(p, k);
}

// Natural log for x > 0 (x == 0 gives -inf, x < 0 or NaN gives NaN).
RM_HD float logf_(float x) {
  if (x != x || x < 0.0f) return x - x + from_bits(0x7fc00000u);
  if (x == 0.0f) return -from_bits(0x7f800000u);
  if (x == from_bits(0x7f800000u)) return x;
  int e = 0;
  if (x < 1.17549435e-38f) {  // subnormal: scale into the normal range
    x = x * 8388608.0f;
    e = -23;
  }
  uint32_t b = to_bits(x);
  e += (int)((b >> 23) & 0xff) - 127;
  float m = from_bits((b & 0x007fffffu) | 0x3f800000u);
  if (m > 1.41421354f) {
    m = m * 0.5f;
    e += 1;
  }
  float s = (m - 1.0f) / (m + 1.0f);
  float s2 = s * s;
  float p = 2.0f / 11.0f;
  p = 2.0f / 9.0f + s2 * p;
  p = 2.0f / 7.0f + s2 * p;
  p = 2.0f / 5.0f + s2 * p;
  p = 2.0f / 3.0f + s2 * p;
  float lm = 2.0f * s + (s * s2) * p;
  float ef = (float)e;
  return ef * RM_LN2_A + (ef * RM_LN2_B + lm);
}

}  // namespace rmath
