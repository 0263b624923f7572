// FP32 math for the mixed-precision form, written from published methods:
//
//  * sincos of a phase given as a 32-bit fixed-point fraction of a turn:
//    the reduction to an octant is exact integer arithmetic, the remaining
//    |x| <= pi/4 uses the Taylor series of sin (to x^11) and cos (to x^12),
//    truncation error below 2e-9.
//  * sin of an FP32 radian argument: Cody-Waite reduction by pi/2 with a
//    two-term split of pi/2, then the same octant polynomials.
//  * erfc for x >= 0 in the form erfc(x) = t exp(-x^2 + P(s)), t = 1/(1 + x/2),
//    of Press et al., Numerical Recipes (2nd ed., sec. 6.2, "erfcc"), with P
//    this project's own degree-12 Chebyshev fit (fit_f32math.py; fit error
//    below 1e-10 over [0, 5]); x^2 is split into an exact hi + lo pair so
//    that exp sees the argument to full precision.
//  * erf(t)/t as a degree-16 polynomial in u = t^2 (fit_f32math.py), used
//    through its divided difference for close pairs.
//  * float-float arithmetic (hi + lo pairs, Dekker 1971; Knuth TAOCP 2,
//    sec. 4.2.2) for the 1/r difference of close pairs from exact integer
//    squared distances.
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
  float rf = (float)r;  // 2 pi / 2^32 as FP32 hi + lo
  float x = fmaf(rf, -4.07094027e-17f, rf * 1.46291812e-9f);
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
  // P of erfc_f32 in s = 2.8 t - 1.8 (FP32 values of both constants),
  // highest power first, with the low parts of the two lowest coefficients
  // (fit_f32math.py)
  constexpr float ERFC_P[13] = {
      5.615803502e-07f,  7.088095799e-07f,  -7.537935744e-06f,  2.896570777e-06f,
      5.682720439e-05f,  -1.166972652e-04f,  -2.909860341e-04f,  1.508955029e-03f,
      7.936029579e-04f,  -1.847265288e-02f,  2.271960257e-03f,  4.911400974e-01f,
      -4.768877327e-01f};
  constexpr float ERFC_P1_LO = -1.094552576e-08f, ERFC_P0_LO = 8.866951617e-09f;
  float t = 1.0f / fmaf(0.5f, x, 1.0f);
  float sv = fmaf(t, 2.79999995f, -1.79999995f);  // FP32-exact map
  float p = ERFC_P[0];
#pragma unroll
  for (int k = 1; k < 13; ++k)
    p = fmaf(sv, p, ERFC_P[k]);
  p += fmaf(sv, ERFC_P1_LO, ERFC_P0_LO);
  float x2 = x * x;
  float x2lo = fmaf(x, x, -x2);  // x*x = x2 + x2lo exactly
  return t * expf(-x2) * expf(p - x2lo);
}

// ---- float-float (value = hi + lo, |lo| <= ulp(hi) / 2) ----
// The error-free steps (the rounded sum or product whose error is recovered
// next) use the _rn intrinsics, which the compiler never contracts into an
// FMA with a neighbouring product.
struct ff2 {
  float hi, lo;
};
__device__ __forceinline__ ff2 ff_quick(float a, float b) {  // |a| >= |b|
  float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ ff2 ff_two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bp = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp))};
}
__device__ __forceinline__ ff2 ff_from_i64(long long v) {
  float hi = __ll2float_rn(v);
  return {hi, __ll2float_rn(v - (long long)hi)};
}
__device__ __forceinline__ ff2 ff_mul(ff2 a, ff2 b) {
  float p = __fmul_rn(a.hi, b.hi);
  float e = fmaf(a.hi, b.hi, -p);
  e += fmaf(a.hi, b.lo, a.lo * b.hi);
  return ff_quick(p, e);
}
__device__ __forceinline__ ff2 ff_add(ff2 a, ff2 b) {
  ff2 s = ff_two_sum(a.hi, b.hi);
  return ff_quick(s.hi, s.lo + (a.lo + b.lo));
}
__device__ __forceinline__ ff2 ff_sqrt(ff2 a) {
  float y = sqrtf(a.hi);
  float e = fmaf(-y, y, a.hi) + a.lo;
  return ff_quick(y, e / (2.0f * y));
}
__device__ __forceinline__ ff2 ff_div(ff2 a, ff2 b) {
  float q1 = a.hi / b.hi;
  ff2 p = ff_mul({q1, 0.0f}, b);
  ff2 r = ff_add(a, {-p.hi, -p.lo});
  return ff_quick(q1, r.hi / b.hi);
}

// Exact squared distances of a close pair in float-float: Do and Dn from the
// integer turn differences o (old) and n (new), dD = Dn - Do from the exact
// integer differences per axis; turn2[d] = (L_d 2^-32)^2 as hi + lo.
struct ClosePair {
  ff2 Do, Dn, dD;
};
__device__ __forceinline__ ClosePair close_pair(const int32_t o[3],
                                                const int32_t n[3],
                                                const float turn2_hi[3],
                                                const float turn2_lo[3]) {
  ClosePair c = {{0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    long long o2 = (long long)o[d] * o[d], n2 = (long long)n[d] * n[d];
    ff2 s2 = {turn2_hi[d], turn2_lo[d]};
    c.Do = ff_add(c.Do, ff_mul(ff_from_i64(o2), s2));
    c.Dn = ff_add(c.Dn, ff_mul(ff_from_i64(n2), s2));
    c.dD = ff_add(c.dD, ff_mul(ff_from_i64(n2 - o2), s2));
  }
  return c;
}

// 12-6 energy change eps_cn [(s'^6 - s'^3) - (s^6 - s^3)], s = sigma^2 / r^2,
// of a close pair in float-float (sigma^2 and eps_cn as hi + lo).
__device__ __forceinline__ ff2 close_lj(const ClosePair &c, ff2 sg2, ff2 ecn) {
  ff2 so = ff_div(sg2, c.Do), sn = ff_div(sg2, c.Dn);
  ff2 so3 = ff_mul(ff_mul(so, so), so), sn3 = ff_mul(ff_mul(sn, sn), sn);
  ff2 uo = ff_add(ff_mul(so3, so3), {-so3.hi, -so3.lo});
  ff2 un = ff_add(ff_mul(sn3, sn3), {-sn3.hi, -sn3.lo});
  return ff_mul(ecn, ff_add(un, {-uo.hi, -uo.lo}));
}

// Ewald bracket erfc(a r')/r' - erfc(a r)/r of a pair beyond the close range
// from the exact squared distances of close_pair (alpha as hi + lo):
//   erfc(t') (1/r' - 1/r) + (erfc(t') - erfc(t)) / r,
// with 1/r' - 1/r in float-float, t = a r and t' - t = a (r'^2 - r^2)/(r + r')
// accurate to FP32 relative to themselves, erfc(t') corrected for the low
// part of t', and erfc(t') - erfc(t) as 3-point Gauss-Legendre quadrature of
// (2/sqrt pi) exp(-s^2) over [t, t'] (the difference of two erfc values when
// the step is large).  The weights times 2/sqrt(pi) are FP32 hi + lo pairs.
__device__ __forceinline__ float far_coulomb(const ClosePair &c, ff2 alpha) {
  ff2 ro = ff_sqrt(c.Do), rn = ff_sqrt(c.Dn), sr = ff_add(ro, rn);
  ff2 dinv = ff_div({-c.dD.hi, -c.dD.lo}, ff_mul(ff_mul(ro, rn), sr));
  ff2 to = ff_mul(alpha, ro), tn = ff_mul(alpha, rn);
  float dt = ff_div(ff_mul(alpha, c.dD), sr).hi;  // t' - t
  float derfc;
  if (fabsf(dt) < 0.25f) {
    float hw = 0.5f * dt, tm = to.hi + (to.lo + hw);
    float t1 = fmaf(-0.774596669f, hw, tm), t3 = fmaf(0.774596669f, hw, tm);
    float em = expf(-tm * tm), e13 = expf(-t1 * t1) + expf(-t3 * t3);
    float g = fmaf(1.00300372f, em, 0.626877308f * e13) +
              fmaf(-1.23839108e-8f, em, 7.16121695e-9f * e13);
    derfc = -hw * g;
  } else {
    derfc = (erfc_f32(tn.hi) - erfc_f32(to.hi)) -
            1.12837917f * (expf(-tn.hi * tn.hi) * tn.lo -
                           expf(-to.hi * to.hi) * to.lo);
  }
  float en = fmaf(-1.12837917f * expf(-tn.hi * tn.hi), tn.lo, erfc_f32(tn.hi));
  return fmaf(en, dinv.hi, fmaf(en, dinv.lo, derfc / ro.hi));
}

// Coulomb bracket of a close pair, erfc(a r')/r' - erfc(a r)/r (Ewald) or
// 1/r' - 1/r, as hi + lo, from the exact squared distances of close_pair;
// alpha2 = alpha^2 in FP32 and alpha3 = alpha^3 as hi + lo.  1/r' - 1/r =
// -(r'^2 - r^2) / (r r' (r + r')) is taken in float-float, and the smooth
// part erf(a r)/r = a g(a^2 r^2), g(u) = erf(sqrt u)/sqrt u, enters through
// the divided difference of g, so neither part loses digits to cancellation.
// Valid while a^2 r^2 and a^2 r'^2 are at most 8.
__device__ __forceinline__ ff2 close_coulomb(const ClosePair &c, bool ewald,
                                            float alpha2, ff2 alpha3) {
  const ff2 &Do = c.Do, &Dn = c.Dn, &dD = c.dD;
  ff2 ro = ff_sqrt(Do), rn = ff_sqrt(Dn);
  ff2 den = ff_mul(ff_mul(ro, rn), ff_add(ro, rn));
  ff2 dinv = ff_div({-dD.hi, -dD.lo}, den);
  if (!ewald)
    return dinv;
  // erf(t)/t in v = t^2 / 4 - 1 over t^2 in [0, 8], highest power first
  constexpr float ERF_OVER_T[17] = {
      2.032793418e-07f,  -8.897155794e-07f,  2.865503120e-06f,  -1.098633129e-05f,
      4.077676203e-05f,  -1.371821127e-04f,  4.277413827e-04f,  -1.235923497e-03f,
      3.284808714e-03f,  -7.982767187e-03f,  1.764078625e-02f,  -3.527706116e-02f,
      6.369094551e-02f,  -1.042822003e-01f,  1.582058221e-01f,  -2.384970784e-01f,
      4.976611435e-01f};
  constexpr float ERF_OVER_T1_LO = 4.852327290e-09f;
  // [g(u_n) - g(u_o)] / (v_n - v_o) by synthetic division (one Horner pass)
  float vo = fmaf(alpha2 * Do.hi, 0.25f, -1.0f);
  float vn = fmaf(alpha2 * Dn.hi, 0.25f, -1.0f);
  float p = ERF_OVER_T[0], dd = p;
#pragma unroll
  for (int k = 1; k < 16; ++k) {
    p = fmaf(vn, p, ERF_OVER_T[k]);
    dd = fmaf(dd, vo, p);
  }
  dd += ERF_OVER_T1_LO;  // the power-1 coefficient enters dd once
  // a [g(u_n) - g(u_o)] = a^3 (r'^2 - r^2) dd / 4
  float w = 0.25f * dD.hi * dd;
  return ff_add(dinv, {-alpha3.hi * w, -alpha3.lo * w});
}

__device__ __forceinline__ void two_sum_add(float &hi, float &lo, float v) {
  ff2 s = ff_two_sum(hi, v);
  hi = s.hi;
  lo += s.lo;
}

// ---- complex float-float: float4 (re hi, re lo, im hi, im lo) ----
__device__ __forceinline__ float4 ffc_mul(float4 a, float4 b) {
  // re = a.re b.re - a.im b.im, im = a.re b.im + a.im b.re; the two leading
  // products and their sum are error-free, the low-order cross terms are
  // added in FP32.
  float p1 = __fmul_rn(a.x, b.x), p2 = __fmul_rn(a.z, b.z);
  float e1 = fmaf(a.x, b.x, -p1), e2 = fmaf(a.z, b.z, -p2);
  ff2 s = ff_two_sum(p1, -p2);
  float t = (e1 - e2) + s.lo;
  t += fmaf(a.x, b.y, a.y * b.x) - fmaf(a.z, b.w, a.w * b.z);
  ff2 re = ff_quick(s.hi, t);
  float p3 = __fmul_rn(a.x, b.z), p4 = __fmul_rn(a.z, b.x);
  float e3 = fmaf(a.x, b.z, -p3), e4 = fmaf(a.z, b.x, -p4);
  ff2 u = ff_two_sum(p3, p4);
  float v = (e3 + e4) + u.lo;
  v += fmaf(a.x, b.w, a.y * b.z) + fmaf(a.z, b.y, a.w * b.x);
  ff2 im = ff_quick(u.hi, v);
  return make_float4(re.hi, re.lo, im.hi, im.lo);
}
__device__ __forceinline__ float4 ffc_conj_if(float4 a, bool neg) {
  return neg ? make_float4(a.x, a.y, -a.z, -a.w) : a;
}
// (hi, lo) += v (float-float), renormalised
__device__ __forceinline__ void ff_acc(float &hi, float &lo, float vh, float vl) {
  ff2 s = ff_two_sum(hi, vh);
  ff2 r = ff_quick(s.hi, s.lo + (lo + vl));
  hi = r.hi;
  lo = r.lo;
}

// exp(2 pi i u / 2^64) in float-float for a phase u given as an exact 64-bit
// fraction of a turn.  u is rounded to the nearest 1/256 turn, whose cosine
// and sine come from `tab` (256 entries, double values split into hi + lo);
// the remainder |x| <= pi/256 takes the Taylor series
// sin x = x - x^3 (1/6 - x^2/120) and cos x = 1 - x^2/2 + x^4/24 - x^6/720
// (truncation below 1e-17): x, x^2, x^3 and 1/6 in float-float; x^2/120,
// x^4/24 and x^6/720 in FP32 (their size is at most 1.3e-6 relative to the
// term they correct, or 1e-9 absolute, so FP32 rounding stays below 1e-16).
__device__ __forceinline__ float4 cis_turns64_ff(uint64_t u, const float4 *tab) {
  uint64_t up = u + (1ULL << 55);
  uint32_t j = (uint32_t)(up >> 56);
  int64_t r = (int64_t)(u - ((uint64_t)j << 56));  // |r| <= 2^55
  constexpr double TP = 6.283185307179586476925286766559 / 18446744073709551616.0;
  constexpr float TP_HI = (float)TP;
  constexpr float TP_LO = (float)(TP - (double)TP_HI);
  constexpr float S6_HI = (float)(1.0 / 6.0);
  constexpr float S6_LO = (float)(1.0 / 6.0 - (double)S6_HI);
  ff2 x = ff_mul(ff_from_i64(r), {TP_HI, TP_LO});
  ff2 x2 = ff_mul(x, x);
  float h = x2.hi;
  ff2 s3 = ff_mul(ff_mul(x, x2), ff_quick(S6_HI, S6_LO - h * (1.0f / 120.0f)));
  ff2 sn = ff_add(x, {-s3.hi, -s3.lo});
  float c4 = h * h * fmaf(h, -1.0f / 720.0f, 1.0f / 24.0f);
  ff2 cs = ff_quick(1.0f, -0.5f * x2.hi);
  cs = ff_quick(cs.hi, cs.lo + (c4 - 0.5f * x2.lo));
  return ffc_mul(tab[j & 255], make_float4(cs.hi, cs.lo, sn.hi, sn.lo));
}

}  // namespace gb
