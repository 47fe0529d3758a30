// ps_wind.cuh -- device data of the 2-D spherical line-driven disk wind:
// geometry factors, the sparse per-cell list of flux bins used by the line
// force, and the problem parameters (units, gravity, floors, cooling).
#pragma once

#include "ps_blondin.cuh"
#include "ps_hydro.cuh"

namespace ps {

// 1-D geometry arrays over the total box; every product the reference
// forms per cell (volumes, areas) is rebuilt from these with the same
// rounding: dV = dVr[i]*dmu[j], A1 = A1f[i]*dmu[j], A2 = rdr[i]*sxp[j].
struct SphGeom {
  // x1 direction (ntot[0] entries)
  const double *x1, *dx1, *inv_dx1;
  const double *rinv;    // 1/x1                    (r_1 of the x1 sources)
  const double *inv_absx1;  // 1/|x1|               (phi-momentum divisor, as a factor)
  const double *inv_dVr;    // 1/dVr                 (volume divisor, with inv_dmu)
  const double *absx1p;  // |x1p|                   (phi-momentum flux factor)
  const double *A1f;     // x1p*x1p
  const double *dVr;     // |x1p^3 - x1m^3| / 3
  const double *rdr;     // |x1|*dx1
  const double *rtinv;   // 1/rt                    (dx/dl in x2, r_1 of the x2 sources)
  const double *g0;      // -1*GM/(x1*x1)            (BodyForceVector)
  const double *fx;      // VGradCalc: bilinear weight of the cell centre in x1
  // x2 direction (ntot[1] entries)
  const double *x2, *dx2, *inv_dx2;
  const double *dmu;     // |cos(x2m) - cos(x2p)|
  const double *sxp;     // |sin(x2p)|
  const double *spabs;   // |sp|
  const double *inv_sn;  // 1/|sin(x2)|               (phi-momentum divisor, as a factor)
  const double *inv_dmu; // 1/dmu
  const double *ct;      // 1/tan(x2)
  const double *sin2, *cos2;
  const double *fy;      // VGradCalc: bilinear weight of the cell centre in x2
  // PLM weights per direction
  const double *cp[2], *cm[2], *wp[2], *wm[2], *dp[2], *dm[2];
};

// Flux bins with a nonzero (F_r, F_theta) per active cell, in increasing
// bin order (the order the reference sums them in), as a CSR list.
struct LineList {
  const int *off;        // [nx0*nx1 + 1], active cell (i, j) -> (j*nx0 + i)
  const double *Fr, *Ft; // the bin's flux
  const double *fr1, *fr2;  // bilinear weights of the bin's offset point (static)
  // projections of the interpolated (v_r, v_theta) on the bin direction,
  // times UNIT_VELOCITY: at the cell centre (c1a, c1b) and at the offset
  // point (c2a, c2b)
  const double *c1a, *c1b, *c2a, *c2b;
  const double *inv_ds;  // 1 / ds; 0 for a bin without direction (dv/ds = -999)
  double *lq;            // per entry and stage: (dv/ds)^-2 (power law, one bin;
                         // 0 if dv/ds <= 0), for cells with two or more
                         // bins exp(lf_a0 - alpharad log(dv/ds)) (0 if dv/ds <= 0),
                         // or -log10(dv/ds) (table, -inf if dv/ds <= 0)
  // tabulated force multiplier (KRAD = ALPHARAD = 999): log10 t at the
  // table's points and each cell's log10 M, [point][pitched cell]
  const double *t_fit, *m_fit;
};

struct WindParams {
  int body_force, line_force, floors, cooling;
  double unit_density, unit_length, unit_velocity;
  double mu, kelvin;     // KELVIN = UNIT_VELOCITY^2 * amu / kB
  double dfloor, tfloor, pfloor;
  double inv_dfloor, kmu;   // 1 / dfloor, KELVIN * mu
  double krad, alpharad, sigma_e, unit_acc;
  double lx, t_x;        // L_star*f_x, T_x
  double unit_pressure, unit_time;
  // force multiplier M = krad t^alpharad with t = C sqrt(rho p) / (dv/ds)
  // (code-unit rho and p): lf_a0 = log(krad) + alpharad log(C); the
  // acceleration per bin is (1 + M) F lf_cf
  double lf_a0, lf_cf;
  // KRAD = ALPHARAD = 999: M from each cell's table, log10 t = lt0 +
  // log10(rho p)/2 - log10(dv/ds) (lt0 = log10 C), nm points
  int mfit, nm;
  double lt0;
  // the ODE cooling path (cooling = 2): UNIT_LENGTH / UNIT_DENSITY /
  // UNIT_VELOCITY^3 and KELVIN times the tabulated-cooling mean molecular
  // weight (Src/mean_mol_weight.c:138-141)
  double ode_e_cost, ode_mu0_kelvin;
  // > 0: BLONDIN at this constant ionisation parameter with T_x (the
  // Cartesian cooling configuration); 0: xi from the state / sirocco_xi
  double xi_const;
  // the learned cooling step's unit factors, set by set_sg_units
  double sg_e_of_p, sg_nh_of_rho, sg_n_of_rho, sg_t_of_pr, sg_p_of_tn;
};

// The learned cooling step's unit conversions, the exact path's divisions by
// constants folded into factors (cooling.c:95-162): E = p sg_e_of_p,
// n_H = rho sg_nh_of_rho, n = rho sg_n_of_rho, T = (p / rho) sg_t_of_pr,
// p_new = T_new n sg_p_of_tn (p, rho in code units).  Formed once on the
// host with the units, the same products and quotients the device formed
// per cell before.
inline void set_sg_units(WindParams &W, double gamma)
{
  const double gm1 = gamma - 1.0;
  W.sg_e_of_p = W.unit_pressure / gm1;
  W.sg_nh_of_rho = W.unit_density / (1.43 * kMP);
  W.sg_n_of_rho = W.unit_density / (W.mu * kMP);
  W.sg_t_of_pr = W.sg_e_of_p / (1.5 * W.sg_n_of_rho * kKB);
  W.sg_p_of_tn = 1.5 * kKB * gm1 / W.unit_pressure;
}

struct WindStageArgs {
  StageArgs s;
  SphGeom g;
  LineList L;
  WindParams w;
  const unsigned char *shock;  // MULTID: 1 where FlagShock finds a shock (total box)
};

}  // namespace ps
