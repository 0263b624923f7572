// FP32 math for the mixed-precision form, written from published methods:
//
//  * sincos of a phase given as a 32-bit fixed-point fraction of a turn:
//    the reduction to an octant is exact integer arithmetic, the remaining
//    |x| <= pi/4 uses the Taylor series of sin (to x^11) and cos (to x^12),
//    truncation error below 2e-9.
//  * sin of an FP32 radian argument: Cody-Waite reduction by pi/2 with a
//    two-term split of pi/2, then the same octant polynomials.
//  * erfc for x >= 0: the Chebyshev-fitted form erfc(x) = t exp(-x^2 + P(t)),
//    t = 1/(1 + x/2), of Press et al., Numerical Recipes (2nd ed., sec. 6.2,
//    "erfcc"), fractional error < 1.2e-7; x^2 is split into an exact
//    hi + lo pair so that exp sees the argument to full precision.
#pragma once

#include <stdint.h>

namespace gb {

// sin and cos of x, |x| <= pi/4 (Taylor coefficients (-1)^k / (2k+1)!, ...)
__device__ __forceinline__ void sincos_octant(float x, float *s, float *c) {
  float x2 = x * x;
  float ps = fmaf(x2, -2.5052108385e-8f, 2.7557319224e-6f);  // 1/11!, 1/9!
  ps = fmaf(x2, ps, -1.9841269841e-4f);                      // -1/7!
  ps = fmaf(x2, ps, 8.3333333333e-3f);                       // 1/5!
  ps = fmaf(x2, ps, -1.6666666667e-1f);                      // -1/3!
  *s = fmaf(x * x2, ps, x);
  float pc = fmaf(x2, 2.0876756988e-9f, -2.7557319224e-7f);  // 1/12!, -1/10!
  pc = fmaf(x2, pc, 2.4801587302e-5f);                       // 1/8!
  pc = fmaf(x2, pc, -1.3888888889e-3f);                      // -1/6!
  pc = fmaf(x2, pc, 4.1666666667e-2f);                       // 1/4!
  pc = fmaf(x2, pc, -0.5f);
  *c = fmaf(x2, pc, 1.0f);
}

// exp(2 pi i phase / 2^32) for a 32-bit phase; exact octant reduction.
__device__ __forceinline__ float2 cis_turns(uint32_t phase) {
  int32_t s = (int32_t)phase;                  // turns in [-1/2, 1/2)
  int32_t q = (s + (1 << 29)) >> 30;           // nearest quarter turn
  int32_t r = s - (int32_t)((uint32_t)q << 30);  // |r| <= 2^29
  float x = (float)r * 1.46291807926715968e-9f;  // 2 pi / 2^32
  float sn, cs;
  sincos_octant(x, &sn, &cs);
  switch (q & 3) {
    case 0: return make_float2(cs, sn);
    case 1: return make_float2(-sn, cs);
    case 2: return make_float2(-cs, -sn);
    default: return make_float2(sn, -cs);
  }
}

// sin(x) for a radian argument of moderate size (|x| < ~1e4).
__device__ __forceinline__ float sin_f32(float x) {
  float t = rintf(x * 0.636619772367581343f);  // x / (pi/2)
  float r = fmaf(-t, 1.57079601287841797f, x);  // pi/2 high part
  r = fmaf(-t, 3.13916473e-7f, r);              // pi/2 low part
  int q = (int)t;
  float sn, cs;
  sincos_octant(r, &sn, &cs);
  switch (q & 3) {
    case 0: return sn;
    case 1: return cs;
    case 2: return -sn;
    default: return -cs;
  }
}

// erfc(x), x >= 0 (Numerical Recipes erfcc Chebyshev fit).
__device__ __forceinline__ float erfc_f32(float x) {
  float t = 1.0f / fmaf(0.5f, x, 1.0f);
  float p = fmaf(t, 0.17087277f, -0.82215223f);
  p = fmaf(t, p, 1.48851587f);
  p = fmaf(t, p, -1.13520398f);
  p = fmaf(t, p, 0.27886807f);
  p = fmaf(t, p, -0.18628806f);
  p = fmaf(t, p, 0.09678418f);
  p = fmaf(t, p, 0.37409196f);
  p = fmaf(t, p, 1.00002368f);
  p = fmaf(t, p, -1.26551223f);
  float x2 = x * x;
  float x2lo = fmaf(x, x, -x2);  // x*x = x2 + x2lo exactly
  return t * expf(-x2) * expf(p - x2lo);
}

// Compensated (two-sum) accumulation: (hi, lo) += v.
__device__ __forceinline__ void two_sum_add(float &hi, float &lo, float v) {
  float s = hi + v;
  float bp = s - hi;
  float e = (hi - (s - bp)) + (v - bp);
  hi = s;
  lo += e;
}

}  // namespace gb
