// ps_fastmath.cuh -- table-driven FP64 exp and log for the hot kernels.
//
// The stage kernels of the wind are bound by the FP64 pipe, and the line
// force takes one exponential and one logarithm per cell and sweep.  These
// two functions follow Tang's table-driven methods (P. T. P. Tang, ACM
// TOMS 15(2) 1989 for exp, 16(4) 1990 for log): an argument reduction
// against a 256-entry table (ps_fastmath_tables.cuh, generated by
// gen_fastmath_tables.py) leaves a reduced argument below 2^-8 in
// magnitude, on which a short Taylor polynomial is enough for double
// precision.  exp costs 11 FP64 instructions and log 13; the table reads go
// through the read-only data cache and the exponent handling through the
// integer units.
//
// Accuracy: within 1 ulp of the correctly rounded result over the ranges
// served here (tests/test_gpu_fastmath.py checks them against CUDA's exp and
// log and against mpmath-free identities on a million arguments).  Outside
// those ranges -- |x| > 700 for exp; zero, subnormal, negative, infinite or
// NaN arguments for log -- they return CUDA's exp / log.
#pragma once

#include "ps_fastmath_tables.cuh"

namespace ps {
namespace fm {

// exp(x) = 2^m 2^(j/256) e^r with k = 256 m + j = round(x 256/ln2) and
// r = x - k ln2/256 (|r| <= ln2/512):
// e^r - 1 ~ r + r^2 (1/2 + r/6 + r^2/24 + r^3/120) (remainder below
// r^6/720 < 1e-20).  k is rounded by the 1.5 * 2^52 shifter, whose low
// mantissa bits then hold k as an integer.
__device__ __forceinline__ double exp(double x)
{
  const unsigned long long ax = (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
  if (ax > 0x4085E00000000000ull) return ::exp(x);   // |x| > 700, inf, NaN
  constexpr double kShift = 0x1.8p52;
  const double t = fma(x, kExpInvL, kShift);
  const double kd = t - kShift;
  const long long k = __double_as_longlong(t) - __double_as_longlong(kShift);
  double r = fma(-kd, kExpL1, x);
  r = fma(-kd, kExpL2, r);
  double s = fma(r, 1.0 / 120.0, 1.0 / 24.0);
  s = fma(r, s, 1.0 / 6.0);
  s = fma(r, s, 0.5);
  const double p = fma(r * r, s, r);
  const int j = (int)(k & 255);
  const double th = __ldg(&kExpHi[j]), tl = __ldg(&kExpLo[j]);
  const double v = fma(th, p, tl) + th;   // 2^(j/256) e^r, in [1, 2.01)
  // times 2^m on the exponent field (|m| <= 1010: the result stays normal)
  return __longlong_as_double(__double_as_longlong(v) + ((k >> 8) << 52));
}

// log(x) = e ln2 + log(F) + log1p(r), x = 2^e m, F = 1 + j/256 the table
// point nearest to m, r = (m - F)/F (|r| <= 1/512):
// log1p(r) ~ r + r^2 (-1/2 + r (1/3 + r (-1/4 + r (1/5 - r/6)))) (remainder
// below r^7/7 < 2e-20, which also keeps results near 0 -- x near 1 -- within
// an ulp).  e ln2_hi + log(F)_hi is exact (both on the 2^-42 grid).
__device__ __forceinline__ double log(double x)
{
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  if (b - 0x0010000000000000ull >= 0x7FE0000000000000ull) return ::log(x);  // not positive normal
  const int e = (int)(b >> 52) - 1023;
  const unsigned long long mb = (b & 0x000FFFFFFFFFFFFFull) | 0x3FF0000000000000ull;
  const int j = (int)(((mb >> 43) & 0x1FF) + 1) >> 1;   // nearest j/256, 0..256
  const double m = __longlong_as_double((long long)mb);
  const double F = __longlong_as_double((long long)(0x3FF0000000000000ull +
                                                    ((unsigned long long)j << 44)));
  const double r = (m - F) * __ldg(&kLogInv[j]);   // m - F exact (Sterbenz)
  double s = fma(r, -1.0 / 6.0, 0.2);
  s = fma(r, s, -0.25);
  s = fma(r, s, 1.0 / 3.0);
  s = fma(r, s, -0.5);
  const double p = fma(r * r, s, r);
  // e as a double through the shifter (exact for |e| < 2^51)
  constexpr double kShift = 0x1.8p52;
  const double ed = __longlong_as_double(__double_as_longlong(kShift) + e) - kShift;
  const double hi = fma(ed, kLn2Hi, __ldg(&kLogHi[j]));
  const double lo = fma(ed, kLn2Lo, __ldg(&kLogLo[j])) + p;
  return hi + lo;
}

}  // namespace fm
}  // namespace ps
