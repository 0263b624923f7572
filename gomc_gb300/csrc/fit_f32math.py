"""Polynomial coefficients of the FP32 special functions of the mixed form
(gb_f32math.cuh).  Run: python gomc_gb300/csrc/fit_f32math.py

erfc_f32: erfc(x) = t exp(-x^2 + P(s)), t = 1 / (1 + x/2) -- the
  representation of Numerical Recipes' erfcc (Press et al., Numerical
  Recipes in C, 2nd ed., sec. 6.2) -- with P a degree-12 Chebyshev
  least-squares fit of log(erfcx(x) / t) in s = a t + b over x in [0, 5],
  a = fl32(2.8), b = fl32(-1.8) (t0 = 1 / (1 + 5/2) maps to s = -1),
  written in the monomial basis of s.
erf_over_t: g(u) = erf(sqrt(u)) / sqrt(u), a degree-16 Chebyshev fit over
  u in [0, 8] in v = u / 4 - 1, monomial basis of v.  It feeds the divided
  difference (g(u_n) - g(u_o)) / (u_n - u_o) of close pairs.
Both fits are far below FP32 resolution (printed); the two lowest
coefficients of each are kept as FP32 hi + lo pairs, so what remains is FP32
rounding, which changes from one argument to the next instead of biasing
every pair at one distance the same way.
"""
import numpy as np
from numpy.polynomial import chebyshev as cheb
from scipy.special import erf, erfcx

NODES = 4000
DEG = 12


def _nodes():
    return np.cos(np.pi * (np.arange(NODES) + 0.5) / NODES)


def fit_erfc(xmax=5.0):
    t0 = 1.0 / (1.0 + 0.5 * xmax)
    # the map t -> s with FP32-exact constants (the kernel evaluates exactly
    # this s), so no rounding of the map shifts every argument the same way
    a = float(np.float32(2.0 / (1.0 - t0)))
    b = float(np.float32(-(1.0 + t0) / (1.0 - t0)))
    t = 0.5 * (1.0 - t0) * _nodes() + 0.5 * (1.0 + t0)
    s = a * t + b
    x = 2.0 * (1.0 / t - 1.0)
    p = np.log(erfcx(x) / t)
    c = cheb.chebfit(s, p, DEG)
    err = np.abs(cheb.chebval(s, c) - p).max()
    return (a, b), cheb.cheb2poly(c), err


def fit_erf_over_t(umax=8.0, deg=16):
    v = _nodes()
    u = (v + 1.0) * umax / 2.0
    t = np.sqrt(u)
    g = erf(t) / t
    c = cheb.chebfit(v, g, deg)
    err = np.abs(cheb.chebval(v, c) - g).max()
    return cheb.cheb2poly(c), err


def _emit(name, mono):
    """C initialiser, highest power first; the two lowest coefficients, which
    set the value and slope of every result, as FP32 hi + lo pairs."""
    c = mono[::-1]
    hi = [float(np.float32(v)) for v in c]
    print("constexpr float %s[%d] = {" % (name, len(c)))
    print(",\n".join("    %.9ef" % v for v in hi) + "};")
    for k in (1, 0):
        v = c[len(c) - 1 - k]
        print("// %s low part of the power-%d coefficient: %.9ef"
              % (name, k, v - float(np.float32(v))))


if __name__ == "__main__":
    (a, b), mono, err = fit_erfc()
    print("// erfc: max |P - fit| = %.3e; s = t * %.9gf + %.9gf" % (err, a, b))
    _emit("ERFC_P", mono)
    mono, err = fit_erf_over_t()
    print("// erf(t)/t: max |g - fit| = %.3e" % err)
    _emit("ERF_OVER_T", mono)
