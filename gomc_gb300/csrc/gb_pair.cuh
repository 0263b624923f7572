// Pair terms and reductions shared by the real-space kernels.
#pragma once

#include "gb_internal.h"

namespace gb {

// FFParticle::CalcEn for lambda = 1 (src/FFParticle.cpp:295-325); the caller
// has checked r^2 < Rcut^2.  For n = 12 the (sigma^2/r^2)^6 term is the square
// of the attractive term instead of pow(), one rounding apart.
__device__ __forceinline__ double lj_energy(const FF &ff, double distSq,
                                            int idx) {
  double rRat2 = ff.sigmaSq[idx] / distSq;
  double rRat4 = rRat2 * rRat2;
  double attract = rRat4 * rRat2;
  double n = ff.nexp[idx];
  double repulse = (n == 12.0) ? attract * attract : pow(rRat2, n * 0.5);
  return ff.eps_cn[idx] * (repulse - attract);
}

// FFParticle::CalcVir for lambda = 1 (src/FFParticle.cpp:344-359)
__device__ __forceinline__ double lj_virial(const FF &ff, double distSq,
                                            int idx) {
  double rNeg2 = 1.0 / distSq;
  double rRat2 = rNeg2 * ff.sigmaSq[idx];
  double rRat4 = rRat2 * rRat2;
  double attract = rRat4 * rRat2;
  double n = ff.nexp[idx];
  double repulse = (n == 12.0) ? attract * attract : pow(rRat2, n * 0.5);
  return ff.eps_cn_6[idx] * (ff.nOver6[idx] * repulse - attract) * rNeg2;
}

// erfc(alpha r) / r from r^2 = s.  Inside the table's range: the segment
// from the bits of s (exponent and top 6 mantissa bits), u = 2 (s - a) / h
// - 1 in [-1, 1) exactly (a is s with the lower mantissa bits cleared, 2 / h
// a power of two), and a degree-8 polynomial in u (Chebyshev interpolant of
// the function on the segment, fitted on the host in extended precision;
// relative error near 1e-16 plus the FP64 rounding of the Horner steps).
// Outside it (r^2 < 0.5 A^2 or no table): the direct formula.  About a dozen
// FP64 operations against ~100 for sqrt, erfc and the division, which
// matters on GB300's two FP64 lanes per SM and clock.
// The segment polynomial of table `tab` at r^2 = s; false outside the range.
__device__ __forceinline__ bool seg_poly(const FF &ff, const double *tab,
                                         double s, double *out) {
  long long bits = __double_as_longlong(s);
  int seg = (int)(bits >> 46) - ff.etab_key0;
  if (tab == nullptr || (unsigned)seg >= (unsigned)ff.etab_nseg)
    return false;
  double a = __longlong_as_double(bits & ~((1LL << 46) - 1));
  double scale = __longlong_as_double((2053LL - (bits >> 52)) << 52);
  double u = fma(s - a, scale, -1.0);
  const double *c = tab + (size_t)seg * (ETAB_DEG + 1);
  double p = __ldg(c + ETAB_DEG);
#pragma unroll
  for (int m = ETAB_DEG - 1; m >= 0; --m)
    p = fma(p, u, __ldg(c + m));
  *out = p;
  return true;
}
__device__ __forceinline__ double erfc_over_r(const FF &ff, double s) {
  double p;
  if (seg_poly(ff, ff.erfc_tab, s, &p))
    return p;
  double r = sqrt(s);
  return erfc(ff.alpha * r) / r;
}

// FFParticle::CalcCoulomb, Ewald real-space term (src/FFParticle.cpp:361-399)
__device__ __forceinline__ double coulomb_energy(const FF &ff, double distSq,
                                                 double qq) {
  if (ff.rcutCoulSq < distSq)
    return 0.0;
  if (ff.ewald)
    return qq * erfc_over_r(ff, distSq);
  return qq / sqrt(distSq);
}

// FFParticle::CalcCoulombVir (src/FFParticle.cpp:401-446)
__device__ __forceinline__ double coulomb_virial(const FF &ff, double distSq,
                                                 double qq) {
  if (ff.rcutCoulSq < distSq)
    return 0.0;
  if (ff.ewald) {
    // the force factor from its table (same segments and accuracy as
    // erfc_over_r), else the direct formula
    double p;
    if (seg_poly(ff, ff.vir_tab, distSq, &p))
      return qq * p;
  }
  double dist = sqrt(distSq);
  if (ff.ewald) {
    double constValue = ff.alpha * M_2_SQRTPI;
    double expConstValue = exp(-1.0 * ff.alphaSq * distSq);
    double temp = 1.0 - erf(ff.alpha * dist);
    return qq * (temp / dist + constValue * expConstValue) / distSq;
  }
  return qq / (distSq * dist);
}

// Soft-core squared distance at coupling lambda (src/FFParticle.cpp:301-308):
// cbrt(sc_alpha (1 - lambda)^sc_power max(sigma^6, sc_sigma^6) + r^6).
__device__ __forceinline__ double soft_rsq(const FF &ff, double distSq,
                                           int idx, double lambda) {
  double sigma6 = ff.sigmaSq[idx] * ff.sigmaSq[idx] * ff.sigmaSq[idx];
  sigma6 = fmax(sigma6, ff.sc_sigma_6);
  double dist6 = __dmul_rn(__dmul_rn(distSq, distSq), distSq);
  double lambdaCoef = ff.sc_alpha * pow((1.0 - lambda), (double)ff.sc_power);
  double softDist6 = __dadd_rn(__dmul_rn(lambdaCoef, sigma6), dist6);
  return cbrt(softDist6);
}

// FFParticle::CalcEn at coupling lambda (src/FFParticle.cpp:295-316); the
// caller has checked r^2 < Rcut^2.
__device__ __forceinline__ double lj_energy_lambda(const FF &ff, double distSq,
                                                   int idx, double lambda) {
  if (lambda >= 0.999999)
    return lj_energy(ff, distSq, idx);
  return lambda * lj_energy(ff, soft_rsq(ff, distSq, idx, lambda), idx);
}

// FFParticle::CalcCoulomb at coupling lambda (src/FFParticle.cpp:361-387):
// the soft-core distance only with sc_coul.
__device__ __forceinline__ double coulomb_energy_lambda(const FF &ff,
                                                        double distSq, int idx,
                                                        double qq,
                                                        double lambda) {
  if (ff.rcutCoulSq < distSq)
    return 0.0;
  if (lambda >= 0.999999)
    return coulomb_energy(ff, distSq, qq);
  double r2 = ff.sc_coul ? soft_rsq(ff, distSq, idx, lambda) : distSq;
  double dist = sqrt(r2);
  double e = ff.ewald ? qq * erfc(ff.alpha * dist) / dist : qq / dist;
  return lambda * e;
}

// Block-wide sum of one double, deterministic order; result valid in thread 0.
template <int NT>
__device__ __forceinline__ double block_sum(double v, double *sh) {
  for (int o = 16; o > 0; o >>= 1)
    v += __shfl_down_sync(0xffffffffu, v, o);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0)
    sh[w] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0) {
    for (int i = 0; i < NT / 32; ++i)
      r += sh[i];
  }
  __syncthreads();
  return r;
}

}  // namespace gb
