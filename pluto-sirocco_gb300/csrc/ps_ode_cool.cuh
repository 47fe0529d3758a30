// ps_ode_cool.cuh -- the ODE cooling path of the wind on the device:
// CoolingSource of the production problem (COOLING TABULATED,
// Test_Problems/LineDrivenWind/cv_idl/cooling_source.c:50-246) with its
// Radiat (BLONDIN rates with the SIROCCO prefactors as d(rho e)/dt,
// radiat.c:21-142), integrated per cell by the embedded RKF 1(2) step when
// the cell is not stiff and that step is accurate, else by adaptive Cash-Karp
// 4(5) substeps (Src/Cooling/cooling_ode_solver.c:26-218, 265-324).  The
// pressure change also lowers dt_cool (the step limit of NextTimeStep).
#pragma once

#include "ps_blondin.cuh"
#include "ps_physics.cuh"

namespace ps {

constexpr double kMaxCoolingRate = 0.1;  // g_maxCoolingRate (Src/globals.h:104)
constexpr double kMinCoolingTemp = 1.e4; // g_minCoolingTemp as Radiat sets it
constexpr int kOdeMaxSub = 1000;         // CK45's substep limit (QUIT_PLUTO beyond)
constexpr int kOdeMaxTries = 100000;     // bound on rejected tries (the reference has none)

// one cell's inputs of Radiat
struct OdeCell {
  double rho_cgs_nH;          // n_H = rho UNIT_DENSITY / (1.43 m_p)
  double rho;                 // code density
  double trc;                 // tracer: no heating or cooling below 0.01
  double xi, tx;              // ionisation parameter and X-ray temperature
  double sqxi, sqsqxi;
  double ch, cc, xh, lc, bc;  // prefactors
  double gm1, kmu, e_cost;    // gamma - 1, KELVIN mu, UNIT_LENGTH / UNIT_DENSITY / UNIT_VELOCITY^3
};

// Radiat for rho e = re (floored at the small pressure as the reference
// does); returns d(rho e)/dt in code units, NaN temperature -> bad
__device__ __forceinline__ double ode_radiat(const OdeCell &o, double &re, bool &bad)
{
  double prs = re * o.gm1;
  if (prs < 0.0) {
    prs = kSmallPressure;
    re = prs / o.gm1;
  }
  const double T = prs / o.rho * o.kmu;
  if (T != T) {
    bad = true;
    return 0.0;
  }
  if (T < kMinCoolingTemp) return 0.0;
  const double nH = o.rho_cgs_nH, ne = 1.21 * nH, sqT = sqrt(T);
  const double comp_heat = o.ch * (8.9e-36 * o.xi * o.tx);
  const double comp_cool = o.cc * (8.9e-36 * o.xi * (4.0 * T));
  const double xray_heat = o.xh * (1.5e-21 * (o.sqsqxi / sqT));
  const double line_cool = o.lc * ((1e-16 * exp(-1.3e5 / T) / o.sqxi / T) +
                                   fmin(fmin(1e-24, 5e-27 * sqT), 1.5e-17 / T));
  const double brem_cool = o.bc * (3.3e-27 * sqT);
  const double lambda =
      nH * (ne * comp_heat + nH * xray_heat - ne * comp_cool - ne * line_cool - ne * brem_cool);
  double rhs = o.trc > 0.01 ? lambda * o.e_cost : 0.0;
  rhs *= 1.0 - 1.0 / cosh(pow(T / kMinCoolingTemp, 12));
  return rhs;
}

// Cash-Karp 4(5) over dt in adaptive substeps from (re0, k1); returns the
// suggested next step, the result in re5.  An accepted substep grows the
// step by the cap 5, as the reference's (its growth error is reset to 1e-18
// before use).
static __device__ __noinline__ double ode_ck45(const OdeCell &o, double re0, double k1, double &re5,
                                        double dt, double tol, bool &bad)
{
  const double c1 = 37.0 / 378.0, c3 = 250.0 / 621.0, c4 = 125.0 / 594.0, c6 = 512.0 / 1771.0;
  const double cs1 = 2825.0 / 27648.0, cs3 = 18575.0 / 48384.0, cs4 = 13525.0 / 55296.0,
               cs5 = 277.0 / 14336.0, cs6 = 0.25;
  const double b21 = 0.2, b31 = 3.0 / 40.0, b32 = 9.0 / 40.0, b41 = 0.3, b42 = -0.9, b43 = 1.2;
  const double b51 = -11.0 / 54.0, b52 = 2.5, b53 = -70.0 / 27.0, b54 = 35.0 / 27.0;
  const double b61 = 1631.0 / 55296.0, b62 = 175.0 / 512.0, b63 = 575.0 / 13824.0,
               b64 = 44275.0 / 110592.0, b65 = 253.0 / 4096.0;
  double t = 0.0;
  const double tend = dt;
  int ksub = 0;
  for (int tries = 0; tries < kOdeMaxTries; tries++) {
    double v1 = re0 + dt * b21 * k1;
    const double k2 = ode_radiat(o, v1, bad);
    v1 = re0 + dt * (b31 * k1 + b32 * k2);
    const double k3 = ode_radiat(o, v1, bad);
    v1 = re0 + dt * (b41 * k1 + b42 * k2 + b43 * k3);
    const double k4 = ode_radiat(o, v1, bad);
    v1 = re0 + dt * (b51 * k1 + b52 * k2 + b53 * k3 + b54 * k4);
    const double k5 = ode_radiat(o, v1, bad);
    v1 = re0 + dt * (b61 * k1 + b62 * k2 + b63 * k3 + b64 * k4 + b65 * k5);
    const double k6 = ode_radiat(o, v1, bad);
    re5 = re0 + dt * (c1 * k1 + c3 * k3 + c4 * k4 + c6 * k6);
    const double v4 = re0 + dt * (cs1 * k1 + cs3 * k3 + cs4 * k4 + cs5 * k5 + cs6 * k6);
    const double vscal = fabs(re0) + dt * fabs(k1);
    const double err = fabs(re5 - v4) / fabs(vscal) / tol;
    if (err < 1.0) {
      ksub++;
      t += dt;
      dt = fmin(0.9 * dt * pow(1.e-18, -0.2), 5.0 * dt);
      if (fabs(t / tend - 1.0) < 1.e-9) return dt;
      if (dt > (tend - t)) dt = tend - t;
      re0 = re5;
      k1 = ode_radiat(o, re0, bad);
      if (ksub > kOdeMaxSub) break;
    } else {
      dt = fmax(0.9 * dt * pow(err, -0.25), 0.05 * dt);
    }
  }
  bad = true;
  return dt;
}

// The whole CoolingSource update of one cell: returns the new pressure and
// dt * g_maxCoolingRate / |p1/p0 - 1| for dt_cool.
__device__ __forceinline__ double ode_cool_cell(const OdeCell &o, double prs0, double dt,
                                                double mu0_kelvin, double &dt_cool, bool &bad)
{
  const double min_tol = 2.e-5;
  double re0 = prs0 / o.gm1, re1 = re0;
  const double T0 = prs0 / o.rho * mu0_kelvin;
  if (!(T0 > 0.0)) {
    bad = true;
    return prs0;
  }
  double k1 = ode_radiat(o, re0, bad);
  const bool stiff = fabs(k1) > 0.5 / dt;
  double err = 0.0;
  if (!stiff) {
    // SolveODE_RKF12: 2nd-order solution, error against the 1st-order one
    double v1 = re0 + 0.5 * dt * k1;
    const double k2 = ode_radiat(o, v1, bad);
    re1 = re0 + dt * k2;
    const double v1st = re0 + dt * k1;
    err = fabs(re1 - v1st) / fabs(fabs(re0) + dt * fabs(k1)) / min_tol;
  }
  if (stiff || err > 1.0) {
    double dt1 = 0.5 / (fabs(k1) + 1.0 / dt), t1 = 0.0;
    bool done = false;
    for (int it = 0; it < kOdeMaxTries; it++) {
      if ((t1 + dt1) >= dt) {
        dt1 = dt - t1;
        done = true;
      }
      const double dts = ode_ck45(o, re0, k1, re1, dt1, min_tol, bad);
      t1 += dt1;
      dt1 = dts;
      if (done || bad) break;
      re0 = re1;
      k1 = ode_radiat(o, re0, bad);
    }
    if (!done) bad = true;
  }
  double prs = re1 * o.gm1;
  const double T1 = prs / o.rho * mu0_kelvin;
  if (prs < 0.0) prs = kSmallPressure;
  if (T1 < kMinCoolingTemp && T0 > kMinCoolingTemp) prs = kMinCoolingTemp * o.rho / mu0_kelvin;
  dt_cool = dt * kMaxCoolingRate / fabs(prs / prs0 - 1.0);
  return prs;
}

}  // namespace ps
