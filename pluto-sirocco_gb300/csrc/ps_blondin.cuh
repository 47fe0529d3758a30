// ps_blondin.cuh -- BLONDIN heating/cooling on the device
// (Src/Cooling/BLONDIN/cooling.c:50-319): the per-cell
// implicit trapezoidal energy equation in T solved by bracket expansion and
// Brent's method, shared by the wind kernels, the batched kernels and the
// surrogate (which uses it as its fallback and to label training pairs).
#pragma once

#include "ps_hydro.cuh"

namespace ps {

// CONST_* of Src/pluto.h:299-321 (cgs)
constexpr double kAmu = 1.66053886e-24, kC = 2.99792458e10, kG = 6.6726e-8, kKB = 1.3806505e-16,
                 kMP = 1.67262171e-24, kPI = 3.14159265358979, kSigmaT = 6.6524e-25;
constexpr int kMaxCoolIter = 10000;  // the bracket search of the reference ends far earlier

struct BlCtx {
  double xi, sqxi, sqsqxi, nH, n, tx, E, hc_init, dt_share;
  // per-cell prefactors of the five rates (1 unless a SIROCCO prefactor
  // file was read): Compton heating, Compton cooling, X-ray heating, line
  // cooling, bremsstrahlung
  double ch = 1.0, cc = 1.0, xh = 1.0, lc = 1.0, bc = 1.0;
};

// ne_rat (cooling.c:210-222)
__device__ __forceinline__ double bl_ne_rat(double T)
{
  if (T < 1.5e4) return 1e-2 + pow(10.0, (-51.59417133 + 12.27740153 * log10(T)));
  if (T >= 1.5e4 && T < 3.3e4) return pow(10.0, (-3.80749689 + 0.86092628 * log10(T)));
  return 1.21;
}

// heatcool (cooling.c:173-202) with the cell's prefactors
__device__ __forceinline__ double bl_heatcool(const BlCtx &b, double T)
{
  const double sqT = sqrt(T);
  const double ne = b.nH * bl_ne_rat(T);
  const double comp_heat = b.ch * (8.9e-36 * b.xi * b.tx);
  const double comp_cool = b.cc * (8.9e-36 * b.xi * (4.0 * T));
  const double xray_heat = b.xh * (1.5e-21 * (b.sqsqxi / sqT));
  const double line_cool =
      b.lc * ((1e-16 * exp(-1.3e5 / T) / b.sqxi / T) + fmin(fmin(1e-24, 5e-27 * sqT), 1.5e-17 / T));
  const double brem_cool = b.bc * (3.3e-27 * sqT);
  return b.nH *
         (ne * comp_heat + b.nH * xray_heat - ne * comp_cool - ne * line_cool - ne * brem_cool);
}

// zfunc (cooling.c:233-237)
__device__ __forceinline__ double bl_zfunc(const BlCtx &b, double temp)
{
  return (temp * b.n * kKB / (2.0 / 3.0)) - b.E - b.dt_share * (b.hc_init + bl_heatcool(b, temp)) / 2.0;
}

__device__ __forceinline__ double bl_func(const BlCtx &b, int which, double x)
{
  return which == 0 ? bl_zfunc(b, x) : bl_heatcool(b, x);
}

// zbrent (cooling.c:250-319): ITMAX 100, EPS 3e-8
static __device__ __noinline__ double bl_zbrent(const BlCtx &bc, int which, double x1, double x2,
                                                double tol)
{
  const double EPS = 3.0e-8;
  double a = x1, b = x2, c = x2, d = 0.0, e = 0.0;
  double fa = bl_func(bc, which, a), fb = bl_func(bc, which, b), fc = fb;
  if (fb * fa > 0.0) return b;
  for (int iter = 1; iter <= 100; iter++) {
    if (fb * fc > 0.0) {
      c = a;
      fc = fa;
      e = d = b - a;
    }
    if (fabs(fc) < fabs(fb)) {
      a = b;
      b = c;
      c = a;
      fa = fb;
      fb = fc;
      fc = fa;
    }
    const double tol1 = 2.0 * EPS * fabs(b) + 0.5 * tol;
    const double xm = 0.5 * (c - b);
    if (fabs(xm) <= tol1 || fb == 0.0) return b;
    if (fabs(e) >= tol1 && fabs(fa) > fabs(fb)) {
      double p, q, r;
      const double s = fb / fa;
      if (a == c) {
        p = 2.0 * xm * s;
        q = 1.0 - s;
      } else {
        q = fa / fc;
        r = fb / fc;
        p = s * (2.0 * xm * q * (q - r) - (b - a) * (r - 1.0));
        q = (q - 1.0) * (r - 1.0) * (s - 1.0);
      }
      if (p > 0.0) q = -q;
      p = fabs(p);
      const double min1 = 3.0 * xm * q - fabs(tol1 * q);
      const double min2 = fabs(e * q);
      if (2.0 * p < (min1 < min2 ? min1 : min2)) {
        e = d;
        d = p / q;
      } else {
        d = xm;
        e = d;
      }
    } else {
      d = xm;
      e = d;
    }
    a = b;
    fa = fb;
    if (fabs(d) > tol1)
      b += d;
    else
      b += (xm > 0.0 ? fabs(tol1) : -fabs(tol1));
    fb = bl_func(bc, which, b);
  }
  return b;
}

// The per-cell set-up after E, nH, n, xi, tx and dt_share are known
// (cooling.c:108-113): the xi roots and the initial net rate.
__device__ __forceinline__ void bl_prepare(BlCtx &b, double T)
{
  b.sqxi = sqrt(b.xi);
  b.sqsqxi = pow(b.xi, 0.25);
  b.hc_init = bl_heatcool(b, T);
}

// Bracket expansion and Brent (cooling.c:115-157) from the prepared
// context at temperature T; returns T_f before the 1e4 K floor.  `overflow`
// is set when the bracket search hit kMaxCoolIter.
__device__ __forceinline__ double bl_solve(const BlCtx &b, double T, bool &overflow)
{
  double t_l = T * 0.9, t_u = T * 1.1;
  double test = bl_zfunc(b, t_l) * bl_zfunc(b, t_u);
  int it = 0;
  while (test > 0 && test == test && it < kMaxCoolIter) {
    t_l *= 0.9;
    t_u *= 1.1;
    test = bl_zfunc(b, t_l) * bl_zfunc(b, t_u);
    it++;
  }
  overflow = it >= kMaxCoolIter;
  double T_f;
  if (test != test) {
    T_f = T;
  } else {
    T_f = bl_zbrent(b, 0, t_l, t_u, 1.0);
    const double hc_final = bl_heatcool(b, T_f);
    if (hc_final * b.hc_init < 0.0) T_f = bl_zbrent(b, 1, fmin(T_f, T), fmax(T_f, T), 1.0);
  }
  return T_f;
}

}  // namespace ps
