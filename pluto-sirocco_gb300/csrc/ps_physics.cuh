// ps_physics.cuh -- per-cell / per-interface FP64 arithmetic of the HD path.
//
// Every expression keeps the operand order and rounding steps of the
// reference so that the device result is bit-identical to the reference's
// serial build (compiled without FMA contraction).  This file is built with
// -fmad=false; divisions and square roots are IEEE correctly rounded.
//
// Reference (paths inside the reference project):
//   PrimToCons / ConsToPrim   Src/HD/mappers.c:26-200
//   limiters                  Src/States/plm_coeffs.h:72-180
//   SoundSpeed2               Src/EOS/Ideal/eos.c:16-42
//   Flux                      Src/HD/fluxes.c:23-51
//   MaxSignalSpeed / Davis    Src/HD/eigenv.c:34-65, Src/HD/hll_speed.c:24-91
//   HLLC / HLL                Src/HD/hllc.c:28-180, Src/HD/hll.c:30-107
//   passive scalar flux       Src/adv_flux.c:47-80
#pragma once

#include <cstdint>

#include "ps_dmul.cuh"

namespace ps {

constexpr int RHO = 0, VX1 = 1, VX2 = 2, VX3 = 3, PRS = 4, NFLX = 5;
constexpr int LIM_MC = 0, LIM_VL = 1, LIM_MM = 2;
constexpr int HLLC = 0, HLL = 1;

constexpr double kSmallDensity = 1.e-12;   // g_smallDensity  (Src/globals.h:115)
constexpr double kSmallPressure = 1.e-12;  // g_smallPressure (Src/globals.h:116)

// device flag bits (mirrors PS_F_* of the C ABI)
constexpr unsigned F_NAN = 0x01, F_CONS2PRIM = 0x02, F_NEG_DENSITY = 0x04,
                   F_DT_SMALL = 0x08, F_TMA_TIMEOUT = 0x10, F_COOLING = 0x20;

__device__ __forceinline__ double abs_min(double a, double b)
{
  return fabs(a) < fabs(b) ? a : b;
}
__device__ __forceinline__ double dmax(double a, double b) { return a >= b ? a : b; }
__device__ __forceinline__ double dmin(double a, double b) { return a <= b ? a : b; }

__device__ __forceinline__ bool is_nan_bits(double x)
{
  unsigned long long b = dm_bits(x);
  return (b & 0x7FFFFFFFFFFFFFFFull) > 0x7FF0000000000000ull;
}

// Comparisons on the bit pattern, in the integer units: the FP64 pipe, at
// two lanes per cycle and multiprocessor, is what bounds the stage kernels.
// The pattern is read through dm_bits' opaque move, so that the compiler
// cannot fold a test back into a double-precision compare.
// Each equals its floating-point form for every value, NaN and signed zeros
// included: x > 0 (the patterns of +min_subnormal..+inf), x < 0 (those of
// -min_subnormal..-inf), x > c for a positive finite constant c, and
// a >= b ? a : b for a, b with the sign bit clear.
__device__ __forceinline__ bool gt0(double x)
{
  return dm_bits(x) - 1ull < 0x7FF0000000000000ull;
}
__device__ __forceinline__ bool lt0(double x)
{
  return dm_bits(x) - 0x8000000000000001ull < 0x7FF0000000000000ull;
}
template <unsigned long long CBITS>
__device__ __forceinline__ bool gt_pos(double x)
{
  static_assert(CBITS > 0 && CBITS < 0x7FF0000000000000ull, "positive finite constant");
  return dm_bits(x) - (CBITS + 1ull) < 0x7FF0000000000000ull - CBITS;
}
// x < c for a positive finite c known only at run time: the patterns of
// +0..c (exclusive) and those of -0..-inf
__device__ __forceinline__ bool lt_pos(double x, double c)
{
  const unsigned long long u = dm_bits(x);
  return u < dm_bits(c) || u - 0x8000000000000000ull <= 0x7FF0000000000000ull;
}
__device__ __forceinline__ double nn_max(double a, double b)
{
  const unsigned long long x = dm_bits(a), y = dm_bits(b);
  return (x >= y && x <= 0x7FF0000000000000ull) ? a : b;
}
// DBL_MIN <= x <= DBL_MAX
__device__ __forceinline__ bool normal_pos(double x)
{
  return dm_bits(x) - 0x0010000000000000ull < 0x7FE0000000000000ull;
}

// Limited slope on a uniform Cartesian grid (cp = cm = 2, d = 1/2).
template <int LIM>
__device__ __forceinline__ double limited_slope(double dvp, double dvm)
{
  if constexpr (LIM == LIM_MC) {
    double dv = 0.0;
    if (gt0(dvp * dvm)) {
      double qc = 0.5 * (dvm + dvp), scrh = 2.0 * abs_min(dvp, dvm);
      dv = abs_min(qc, scrh);
    }
    return dv;
  } else if constexpr (LIM == LIM_VL) {
    return gt0(dvp * dvm) ? 2.0 * dvp * dvm / (dvp + dvm) : 0.0;
  } else {
    return gt0(dvp * dvm) ? abs_min(dvp, dvm) : 0.0;
  }
}

// |a| < |b| ? a : b on the bit patterns, for a and b that are not NaN
__device__ __forceinline__ double abs_min_nn(double a, double b)
{
  return (dm_bits(a) << 1) < (dm_bits(b) << 1) ? a : b;
}

// limited_slope with INT: the sign test without the product (dposprod_int),
// the factors 1/2 and 2 as exponent shifts, the magnitude compares on the
// bit patterns (no NaN past the sign test), the van Leer product by
// dmul_int; the same value as limited_slope unless `bad` is set
template <int LIM, bool INT>
__device__ __forceinline__ double limited_slope_t(double dvp, double dvm, bool &bad)
{
  if constexpr (!INT) {
    return limited_slope<LIM>(dvp, dvm);
  } else {
    if (!dposprod_int(dvp, dvm, bad)) return 0.0;
    if constexpr (LIM == LIM_MC) {
      const double qc = dhalf_int(dvm + dvp, bad);
      const double scrh = dtwice_int(abs_min_nn(dvp, dvm), bad);
      return abs_min_nn(qc, scrh);
    } else if constexpr (LIM == LIM_VL) {
      return dmul_int(dtwice_int(dvp, bad), dvm, bad) / (dvp + dvm);
    } else {
      return abs_min_nn(dvp, dvm);
    }
  }
}

// The products no add absorbs by dmul_t<INT> (ps_dmul.cuh): on the integer
// pipes with INT, the same bits either way.
template <int NV, bool INT>
__device__ __forceinline__ void prim_to_cons_t(const double (&v)[NV], double (&u)[NV],
                                               double igmm1, bool &bad)
{
  // E = rho v^2 / 2 + p / (gamma - 1), the division as a product with
  // igmm1 = 1 / (gamma - 1)
  const double rho = v[RHO];
  u[RHO] = rho;
  u[VX1] = dmul_t<INT>(rho, v[VX1], bad);
  u[VX2] = dmul_t<INT>(rho, v[VX2], bad);
  u[VX3] = dmul_t<INT>(rho, v[VX3], bad);
  const double e = fma(v[VX3], v[VX3], fma(v[VX2], v[VX2], dmul_t<INT>(v[VX1], v[VX1], bad)));
  u[PRS] = fma(dhalf_t<INT>(rho, bad), e, dmul_t<INT>(v[PRS], igmm1, bad));
#pragma unroll
  for (int nv = NFLX; nv < NV; nv++) u[nv] = dmul_t<INT>(rho, v[nv], bad);
}
template <int NV>
__device__ __forceinline__ void prim_to_cons(const double (&v)[NV], double (&u)[NV],
                                             double igmm1)
{
  bool bad = false;
  prim_to_cons_t<NV, false>(v, u, igmm1, bad);
}

// Returns device flag bits; u may be repaired in place as in the reference.
// rho^e for the entropy switch as exp(e log rho): CUDA's exp and log cost
// about a third of its pow, and the result stays within |e log rho| ulps
// (a few 1e-15 relative) of the correctly rounded power.
__device__ __forceinline__ double rho_pow(double rho, double e) { return exp(e * log(rho)); }

template <int NV, bool INT>
__device__ __forceinline__ unsigned cons_to_prim_t(double (&u)[NV], double (&v)[NV], double gmm1,
                                                   int ent, bool &bad)
{
  // ent (ENTROPY_SWITCH, the entropy is variable NV-1): 0 switch off;
  // 1 pressure from the energy, then rho s redefined from it; 2 the zone is
  // tagged FLAG_ENTROPY, p = (rho s) rho^(gamma-1) and the energy redefined
  // (Src/HD/mappers.c:185-221).  The products no add absorbs by
  // dmul_t<INT> (ps_dmul.cuh), the same bits either way.
  unsigned flag = 0;
  const double m2 = fma(u[VX3], u[VX3], fma(u[VX2], u[VX2], dmul_t<INT>(u[VX1], u[VX1], bad)));
  if (lt0(u[RHO])) {
    u[RHO] = kSmallDensity;
    flag |= F_CONS2PRIM | F_NEG_DENSITY;
  }
  v[RHO] = u[RHO];
  const double tau = 1.0 / u[RHO];
  v[VX1] = dmul_t<INT>(u[VX1], tau, bad);
  v[VX2] = dmul_t<INT>(u[VX2], tau, bad);
  v[VX3] = dmul_t<INT>(u[VX3], tau, bad);
  const double kin = dmul_t<INT>(dhalf_t<INT>(m2, bad), tau, bad);
  if (lt0(u[PRS])) {
    u[PRS] = kSmallPressure / gmm1 + kin;
    flag |= F_CONS2PRIM;
  }
  if constexpr (NV > NFLX + 1) {
    if (ent == 2) {
      const double rhog1 = rho_pow(u[RHO], gmm1);
      v[PRS] = u[NV - 1] * rhog1;
      if (lt0(v[PRS])) {
        v[PRS] = kSmallPressure;
        flag |= F_CONS2PRIM;
      }
      u[PRS] = v[PRS] / gmm1 + kin;
    }
  }
  if (ent != 2) {
    v[PRS] = dmul_t<INT>(gmm1, u[PRS] - kin, bad);
    if (lt0(v[PRS])) {
      v[PRS] = kSmallPressure;
      u[PRS] = v[PRS] / gmm1 + kin;
      flag |= F_CONS2PRIM;
    }
    if constexpr (NV > NFLX + 1) {
      if (ent == 1) u[NV - 1] = v[PRS] * rho_pow(u[RHO], -gmm1);
    }
  }
#pragma unroll
  for (int nv = NFLX; nv < NV; nv++) v[nv] = dmul_t<INT>(u[nv], tau, bad);
  return flag;
}
template <int NV>
__device__ __forceinline__ unsigned cons_to_prim(double (&u)[NV], double (&v)[NV],
                                                 double gmm1, int ent = 0)
{
  bool bad = false;
  return cons_to_prim_t<NV, false>(u, v, gmm1, ent, bad);
}

// Riemann problem at one interface.  vL is the + state of the left cell,
// vR the - state of the right cell, VN the normal velocity index.
// Outputs the numerical flux (pressure kept apart, as with
// USE_PRS_GRADIENT), the interface pressure and cmax = max(|SL|, |SR|).
// `hll`: HLLC takes the HLL flux at this interface (FLAG_HLL on either
// side with SHOCK_FLATTENING MULTID, Src/HD/hllc.c:93-104).
// The products no add absorbs by dmul_t<INT> (on the integer pipes with
// INT, the same bits either way).
template <int NV, int SOLVER, int VN, bool INT>
__device__ __forceinline__ void riemann_t(const double (&vL)[NV], const double (&vR)[NV],
                                          double gam, double igmm1, double (&f)[NV],
                                          double &pr, double &cmax, bool hll, bool &bad)
{
  // the conserved states are formed in the branches that read them: a
  // supersonic face needs only its upwind side's
  double uL[NV], uR[NV];
  // sound speeds sqrt(gamma p / rho) as (gamma p) rsqrt(gamma p rho): one
  // reciprocal square root in place of a division and a square root
  const double gpL = dmul_t<INT>(gam, vL[PRS], bad), gpR = dmul_t<INT>(gam, vR[PRS], bad);
  const double aL = dmul_t<INT>(gpL, rsqrt(dmul_t<INT>(gpL, vL[RHO], bad)), bad);
  const double aR = dmul_t<INT>(gpR, rsqrt(dmul_t<INT>(gpR, vR[RHO], bad)), bad);
  const double SL = dmin(vL[VN] - aL, vR[VN] - aR);
  const double SR = dmax(vL[VN] + aL, vR[VN] + aR);
  cmax = nn_max(fabs(SL), fabs(SR));

  if (gt0(SL)) {
    prim_to_cons_t<NV, INT>(vL, uL, igmm1, bad);
    f[RHO] = uL[VN];
    f[VX1] = dmul_t<INT>(uL[VX1], vL[VN], bad);
    f[VX2] = dmul_t<INT>(uL[VX2], vL[VN], bad);
    f[VX3] = dmul_t<INT>(uL[VX3], vL[VN], bad);
    f[PRS] = dmul_t<INT>(uL[PRS] + vL[PRS], vL[VN], bad);
    pr = vL[PRS];
  } else if (lt0(SR)) {
    prim_to_cons_t<NV, INT>(vR, uR, igmm1, bad);
    f[RHO] = uR[VN];
    f[VX1] = dmul_t<INT>(uR[VX1], vR[VN], bad);
    f[VX2] = dmul_t<INT>(uR[VX2], vR[VN], bad);
    f[VX3] = dmul_t<INT>(uR[VX3], vR[VN], bad);
    f[PRS] = dmul_t<INT>(uR[PRS] + vR[PRS], vR[VN], bad);
    pr = vR[PRS];
  } else if (SOLVER == HLL || hll) {
    // (SL SR (uR - uL) + SR fL - SL fR) / (SR - SL) with the three weights
    // divided once; each component's conserved values and fluxes formed
    // where they are combined
    const double scrh = 1.0 / (SR - SL);
    const double a = dmul_t<INT>(dmul_t<INT>(SL, SR, bad), scrh, bad);
    const double bR = dmul_t<INT>(SR, scrh, bad), bL = dmul_t<INT>(SL, scrh, bad);
    const double mL = dmul_t<INT>(vL[RHO], vL[VN], bad), mR = dmul_t<INT>(vR[RHO], vR[VN], bad);
    f[RHO] = fma(-bL, mR, fma(bR, mL, dmul_t<INT>(a, vR[RHO] - vL[RHO], bad)));
#pragma unroll
    for (int nv = VX1; nv <= VX3; nv++) {
      const double qL = nv == VN ? mL : dmul_t<INT>(vL[RHO], vL[nv], bad);
      const double qR = nv == VN ? mR : dmul_t<INT>(vR[RHO], vR[nv], bad);
      f[nv] = fma(-bL, dmul_t<INT>(qR, vR[VN], bad),
                  fma(bR, dmul_t<INT>(qL, vL[VN], bad), dmul_t<INT>(a, qR - qL, bad)));
    }
    const double EL = fma(dhalf_t<INT>(vL[RHO], bad),
                          fma(vL[VX3], vL[VX3], fma(vL[VX2], vL[VX2], dmul_t<INT>(vL[VX1], vL[VX1], bad))),
                          dmul_t<INT>(vL[PRS], igmm1, bad));
    const double ER = fma(dhalf_t<INT>(vR[RHO], bad),
                          fma(vR[VX3], vR[VX3], fma(vR[VX2], vR[VX2], dmul_t<INT>(vR[VX1], vR[VX1], bad))),
                          dmul_t<INT>(vR[PRS], igmm1, bad));
    f[PRS] = fma(-bL, dmul_t<INT>(ER + vR[PRS], vR[VN], bad),
                 fma(bR, dmul_t<INT>(EL + vL[PRS], vL[VN], bad), dmul_t<INT>(a, ER - EL, bad)));
    pr = fma(-bL, vR[PRS], dmul_t<INT>(bR, vL[PRS], bad));
  } else {
    // HLLC: only the star state on the side selected by the contact speed
    // is formed; the reference forms both and discards one.
    prim_to_cons_t<NV, INT>(vL, uL, igmm1, bad);
    prim_to_cons_t<NV, INT>(vR, uR, igmm1, bad);
    const double qL = fma(uL[VN], vL[VN] - SL, vL[PRS]);
    const double qR = fma(uR[VN], vR[VN] - SR, vR[PRS]);
    const double wL = dmul_t<INT>(vL[RHO], vL[VN] - SL, bad);
    const double wR = dmul_t<INT>(vR[RHO], vR[VN] - SR, bad);
    const double vs = (qR - qL) / (wR - wL);
    const bool left = vs >= 0.0;
    const double S = left ? SL : SR;
    const double vx = left ? vL[VN] : vR[VN];
    double v[NFLX], u[NFLX];
#pragma unroll
    for (int nv = 0; nv < NFLX; nv++) {
      v[nv] = left ? vL[nv] : vR[nv];
      u[nv] = left ? uL[nv] : uR[nv];
    }
    double fs[NFLX];
    fs[RHO] = u[VN];
    fs[VX1] = dmul_t<INT>(u[VX1], v[VN], bad);
    fs[VX2] = dmul_t<INT>(u[VX2], v[VN], bad);
    fs[VX3] = dmul_t<INT>(u[VX3], v[VN], bad);
    fs[PRS] = dmul_t<INT>(u[PRS] + v[PRS], v[VN], bad);
    double us[NFLX];
    us[RHO] = dmul_t<INT>(u[RHO], S - vx, bad) / (S - vs);
#pragma unroll
    for (int nv = VX1; nv <= VX3; nv++)
      us[nv] = dmul_t<INT>(us[RHO], nv == VN ? vs : v[nv], bad);
    us[PRS] = fma(vs - vx, vs + v[PRS] / dmul_t<INT>(v[RHO], S - vx, bad), u[PRS] / v[RHO]);
    us[PRS] = dmul_t<INT>(us[PRS], us[RHO], bad);
#pragma unroll
    for (int nv = 0; nv < NFLX; nv++) f[nv] = fma(S, us[nv] - u[nv], fs[nv]);
    pr = v[PRS];
  }
  if constexpr (NV > NFLX) {
    const bool up = gt0(f[RHO]);
#pragma unroll
    for (int nv = NFLX; nv < NV; nv++) f[nv] = dmul_t<INT>(f[RHO], up ? vL[nv] : vR[nv], bad);
  }
}
template <int NV, int SOLVER, int VN>
__device__ __forceinline__ void riemann(const double (&vL)[NV], const double (&vR)[NV],
                                        double gam, double igmm1, double (&f)[NV],
                                        double &pr, double &cmax, bool hll = false)
{
  bool bad = false;
  riemann_t<NV, SOLVER, VN, false>(vL, vR, gam, igmm1, f, pr, cmax, hll, bad);
}

}  // namespace ps
