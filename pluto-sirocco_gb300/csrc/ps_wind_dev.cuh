// ps_wind_dev.cuh -- device code of the 2-D spherical line-driven disk
// wind, shared by the single-grid kernels (ps_wind.cu) and the batched
// kernels (ps_batch.cu): boundary and floor rules per cell, BLONDIN per
// cell, VGradCalc/LineForce and the spherical stage tile.
//
// Reference (paths inside the reference project):
//   Boundary, floors          Src/boundary.c:56-500, problem UserDefBoundary
//   PLM (general grid)        Src/States/plm_states.c:135-150, plm_coeffs.h:128-150
//   curvilinear RHS           Src/MHD/rhs.c:234-351, 423-630
//   sources                   Src/MHD/rhs_source.c:101-420
//   VGradCalc, bilinear       Src/LineDriven/line_connect.c:504-777
//   LineForce                 Src/LineDriven/line_connect.c:815-903
//   xi initialisation         Src/LineDriven/line_connect.c:287-306
//   BlondinCooling            Src/Cooling/BLONDIN/cooling.c:50-319
#pragma once

#include "ps_blondin.cuh"
#include "ps_fastmath.cuh"
#include "ps_ode_cool.cuh"
#include "ps_ctx.cuh"
#include "ps_physics.cuh"
#include "ps_stage.cuh"
#include "ps_tma.cuh"
#include "ps_userdef.cuh"
#include "ps_wind.cuh"

namespace ps {


struct WindDev {
  WindStageArgs a;       // geometry, line list, parameters (stage part filled per launch)
  double *geo = nullptr; // all 1-D geometry arrays in one allocation
  int *off = nullptr;
  double *ent = nullptr; // Fr, Ft, fr1, fr2, c1a, c1b, c2a, c2b, inv_ds (SoA, nent each)
  double *dvds = nullptr; // per-entry stage values (LineList::lq)
  double *xi = nullptr, *tr = nullptr;
  double *pre = nullptr;  // 5 prefactor arrays (ch, cc, xh, lc, bc), NULL: all 1
  unsigned char *shock = nullptr;  // SHOCK_FLATTENING MULTID: shocked zones, total box
  double *t_fit = nullptr, *m_fit = nullptr;  // tabulated force multiplier (log10)
  long nent = 0;
  const void *k1 = nullptr, *k2 = nullptr;
  size_t smem = 0;
};

// ------------------------------------------------------------------
// device helpers
// ------------------------------------------------------------------

// The stage kernels whose products no add absorbs run on the integer pipes
// (ps_dmul.cuh, the same bits as the FP64 unit's): the 6-variable
// primitive-PLM set of the batched wind.  The characteristic-limiting and
// entropy-switch sets keep the FP64 unit (and their build time).
template <int NV, bool CHAR>
constexpr bool kIntProducts = NV == NFLX + 1 && !CHAR;

template <int LIM>
__device__ __forceinline__ double limited_slope_general(double dvp, double dvm, double cp,
                                                        double cm)
{
  if constexpr (LIM == LIM_MC) {
    double dv = 0.0;
    if (gt0(dvp * dvm)) {
      double qc = 0.5 * (dvm + dvp), scrh = abs_min(dvp * cp, dvm * cm);
      dv = abs_min(qc, scrh);
    }
    return dv;
  } else if constexpr (LIM == LIM_VL) {
    return gt0(dvp * dvm) ? dvp * dvm * (cp * dvm + cm * dvp) /
                                 (dvp * dvp + dvm * dvm + (cp + cm - 2.0) * dvp * dvm)
                           : 0.0;
  } else {
    return gt0(dvp * dvm) ? abs_min(dvp, dvm) : 0.0;
  }
}

// PLM of one cell with the van Leer limiter on the general grid: the
// weighted one-sided differences, the slopes of the NV variables with one
// division per group of GS, the states at the cell's faces.  The
// denominators' reciprocals come from Montgomery's simultaneous inversion
// (prefix products, one reciprocal of the group's total, a backward pass;
// a dependent FP64 operation waits about 875 cycles on GB300, so shorter
// groups trade divisions for shorter chains); variables whose one-sided
// differences have opposite signs get slope 0 and denominator 1; when the
// product of the denominators leaves the normal range, each slope takes its
// own division.  The slopes stay within a few ulps of the direct quotients.
// The products that no add absorbs are formed by dmul_t<INT>: on the
// integer pipes with INT (ps_dmul.cuh); a cell whose operands leave the
// range of the integer product (`bad`) is done again with INT = false,
// which gives the same bits wherever the integer form applies.  Each
// variable's differences are formed where its numerator and denominator
// are, and the cell values are read again for the face states, so that
// few values stay live across the passes.
template <int NV, bool INT, class G, int GS = NV>
__device__ __forceinline__ void plm_vl_cell(const double *__restrict__ sv,
                                            double *__restrict__ svp,
                                            double *__restrict__ svm, int s0, int sst, int q,
                                            double wp, double wm, double cp, double cm,
                                            double dp, double dm, bool &bad)
{
  // GS variables share one inversion (NV / GS divisions per cell)
  static_assert(NV % GS == 0, "whole groups");
  const double c2 = cp + cm - 2.0;
#pragma unroll
  for (int g0 = 0; g0 < NV; g0 += GS) {
    double num[GS], den[GS], pre[GS];
    double prod = 1.0;
#pragma unroll
    for (int j = 0; j < GS; j++) {
      const int k = g0 + j;
      const double v0 = sv[k * G::VS + s0];
      const double dvp = dmul_t<INT>(sv[k * G::VS + s0 + sst] - v0, wp, bad);
      const double dvm = dmul_t<INT>(v0 - sv[k * G::VS + s0 - sst], wm, bad);
      const double pm = dmul_t<INT>(dvp, dvm, bad);
      const bool on = gt0(pm);
      num[j] = on ? dmul_t<INT>(pm, fma(cm, dvp, dmul_t<INT>(cp, dvm, bad)), bad) : 0.0;
      den[j] = on ? fma(c2, pm, fma(dvm, dvm, dmul_t<INT>(dvp, dvp, bad))) : 1.0;
      pre[j] = prod;
      prod = j == 0 ? den[0] : dmul_t<INT>(prod, den[j], bad);
    }
    const bool one = normal_pos(prod);
    double r = one ? 1.0 / prod : 0.0;
#pragma unroll
    for (int j = GS - 1; j >= 0; j--) {
      const int k = g0 + j;
      double dv;
      if (one) {
        dv = dmul_t<INT>(num[j], j == 0 ? r : dmul_t<INT>(r, pre[j], bad), bad);
        if (j > 0) r = dmul_t<INT>(r, den[j], bad);
      } else {
        dv = num[j] / den[j];
      }
      const double v0 = sv[k * G::VS + s0];
      svp[k * G::NPMAX + q] = fma(dv, dp, v0);
      svm[k * G::NPMAX + q] = fma(-dv, dm, v0);
    }
  }
}

// Limited slopes on characteristic variables (CHAR_LIMITING YES,
// Src/States/plm_states.c:481-746, HD with energy, general grid): the
// one-sided differences projected on the left primitive eigenvectors
// (HD/eigenv.c:92-240, PrimEigenvectors; eigenv.c:575-617, PrimToChar),
// each characteristic difference limited, projected back on the right
// eigenvectors, bounded by ABS_MIN(cp dvp, cm dvm) in primitive variables
// (minmod), passive scalars limited as primitives.  D selects the normal
// velocity (tangential ones: x1 sweep VX2, VX3; x2 sweep VX3, VX1).
template <int D, int NV, int LIM>
__device__ __forceinline__ void char_slopes(const double (&v)[NV], const double (&dvp)[NV],
                                            const double (&dvm)[NV], double cp, double cm,
                                            double gam, bool minmod, double (&dv)[NV])
{
  constexpr int vn = VX1 + D, vt = D == 0 ? VX2 : VX3, vb = D == 0 ? VX3 : VX1;
  // PrimEigenvectors' sound speed and the entries 1/(rho c), -1/c^2 and
  // rho/c of L and R from one division: with a = gamma p and
  // ir = 1/(rho a), c^2 = a^2 ir, 1/c^2 = rho^2 ir, 1/(rho c) = c rho ir
  const double a = gam * v[PRS], ir = 1.0 / (v[RHO] * a);
  const double cs2 = a * a * ir, icss = v[RHO] * v[RHO] * ir;
  const double cs = sqrt(cs2);
  const double rhocs = v[RHO] * cs, rho_cs = v[RHO] * cs * icss;
  const double l0p = cs * v[RHO] * ir, l2p = -icss;
  double wp[5], wm[5], wl[5];
  wm[0] = -1.0 * dvm[vn] + l0p * dvm[PRS];
  wm[1] = 1.0 * dvm[vn] + l0p * dvm[PRS];
  wm[2] = dvm[RHO] + l2p * dvm[PRS];
  wm[3] = dvm[vt];
  wm[4] = dvm[vb];
  wp[0] = -1.0 * dvp[vn] + l0p * dvp[PRS];
  wp[1] = 1.0 * dvp[vn] + l0p * dvp[PRS];
  wp[2] = dvp[RHO] + l2p * dvp[PRS];
  wp[3] = dvp[vt];
  wp[4] = dvp[vb];
  if (minmod) {   // FLAG_MINMOD
#pragma unroll
    for (int k = 0; k < 5; k++) wl[k] = gt0(wp[k] * wm[k]) ? abs_min(wp[k], wm[k]) : 0.0;
  } else {
#pragma unroll
    for (int k = 0; k < 5; k++) wl[k] = limited_slope_general<LIM>(wp[k], wm[k], cp, cm);
  }
  // dc = sum_k wl[k] R[nv][k] with the nonzero entries of the right
  // eigenvectors, in the order of k
  double dc[5];
  dc[RHO] = ((0.0 + wl[0] * (0.5 * rho_cs)) + wl[1] * (0.5 * rho_cs)) + wl[2] * 1.0;
  dc[vn] = (0.0 + wl[0] * -0.5) + wl[1] * 0.5;
  dc[PRS] = (0.0 + wl[0] * (0.5 * rhocs)) + wl[1] * (0.5 * rhocs);
  dc[vt] = 0.0 + wl[3] * 1.0;
  dc[vb] = 0.0 + wl[4] * 1.0;
#pragma unroll
  for (int nv = 0; nv < 5; nv++) {
    if (gt0(dvp[nv] * dvm[nv])) {
      const double d2v = abs_min(cp * dvp[nv], cm * dvm[nv]);
      dv[nv] = gt0(d2v * dc[nv]) ? (fabs(d2v) < fabs(dc[nv]) ? d2v : dc[nv]) : 0.0;
    } else {
      dv[nv] = 0.0;
    }
  }
#pragma unroll
  for (int nv = 5; nv < NV; nv++) dv[nv] = limited_slope_general<LIM>(dvp[nv], dvm[nv], cp, cm);
}

__device__ __forceinline__ long long vcell(const Params &p, int gj, int gi)
{
  return (long long)gj * p.px + gi + p.xoff;
}

// FlagShock's test for one zone of the 2-D spherical grid
// (Src/flag_shock.c:156-270): div v < 0 from the face areas and volume, and
// the pressure jump sum_d |p_{+1} - p_{-1}| against min(p, neighbours).
// Zones of the outer ring are never tested.
__device__ __forceinline__ unsigned char shock_zone(const double *V, const Params &p,
                                                    const SphGeom &g, int gi, int gj)
{
  if (gi < 1 || gi > p.ntot[0] - 2 || gj < 1 || gj > p.ntot[1] - 2) return 0;
  const long long c = vcell(p, gj, gi), sx = 1, sy = p.px;
  const double *vx1 = V + VX1 * p.vstride, *vx2 = V + VX2 * p.vstride, *pt = V + PRS * p.vstride;
  const double dvx1 = g.A1f[gi] * g.dmu[gj] * (vx1[c + sx] + vx1[c]) -
                      g.A1f[gi - 1] * g.dmu[gj] * (vx1[c - sx] + vx1[c]);
  const double dvx2 = g.rdr[gi] * g.sxp[gj] * (vx2[c + sy] + vx2[c]) -
                      g.rdr[gi] * g.sxp[gj - 1] * (vx2[c - sy] + vx2[c]);
  const double divv = (dvx1 + dvx2) / (g.dVr[gi] * g.dmu[gj]);
  if (!(divv < 0.0)) return 0;
  double pt_min = pt[c];
  const double pmin1 = dmin(pt[c + sx], pt[c - sx]), pmin2 = dmin(pt[c + sy], pt[c - sy]);
  pt_min = dmin(pt_min, pmin1);
  pt_min = dmin(pt_min, pmin2);
  const double gradp = fabs(pt[c + sx] - pt[c - sx]) + fabs(pt[c + sy] - pt[c - sy]);
  // bit 0: shocked for the flattening (EPS_PSHOCK_FLATTEN 5); bit 1: taken
  // off the entropy with ENTROPY_SWITCH SELECTIVE (EPS_PSHOCK_ENTROPY 0.05)
  return (gradp > 5.0 * pt_min ? 1 : 0) | (gradp > 0.05 * pt_min ? 2 : 0);
}

__device__ __forceinline__ long long vcell3(const Params &p, int gk, int gj, int gi)
{
  return ((long long)gk * p.ntot[1] + gj) * p.px + gi + p.xoff;
}

// Active cell q (x fastest) -> (gi, gj, gk) of the total box.
__device__ __forceinline__ void cell_of(const Params &p, long long q, int &gi, int &gj, int &gk)
{
  const long long r = q / p.nx[0];
  gi = (int)(q - r * p.nx[0]) + p.beg[0];
  gj = (int)(r % p.nx[1]) + p.beg[1];
  gk = (int)(r / p.nx[1]) + p.beg[2];
}

// Boundary() part 1: the problem's side-0 hook (floors) on the active cells,
// then the x1 ghost cells of the active rows, each written by the active
// cell it comes from (user sides through the X1 hooks of ps_userdef.cuh).
// One active cell q at state index c (column gi, row gj) whose density and
// pressure the caller loaded.
template <int NV>
__device__ __forceinline__ void bnd_x1_cell_rp(double *V, double *Us, const Params &p,
                                               const WindParams &w, int stage, int gi, int gj,
                                               long long c, double rho, double prs)
{
  {
    // density and pressure decide the floors; the other variables are
    // read only for a floored cell or a cell whose x1 ghosts it writes
    // (the first and last active columns, or every column within the ghost
    // width of either end for periodic and reflective boundaries)
    const int ng = p.beg[0];
    const bool edge = gi < p.beg[0] + ng || gi > p.beg[0] + p.nx[0] - 1 - ng;
    double v[NV];
    v[RHO] = rho;
    v[PRS] = prs;
    const bool floored = w.floors && (lt_pos(v[RHO], w.dfloor) || lt_pos(v[PRS], w.pfloor));
    if (floored || edge) {
      v[VX1] = V[VX1 * p.vstride + c];
      v[VX2] = V[VX2 * p.vstride + c];
      v[VX3] = V[VX3 * p.vstride + c];
#pragma unroll
      for (int nv = NFLX; nv < NV; nv++) v[nv] = V[nv * p.vstride + c];
    }
    if (floored && UserDefBoundary_Internal<NV>(v, w, p.gamma)) {
#pragma unroll
      for (int nv = 0; nv < NV; nv++) V[nv * p.vstride + c] = v[nv];
      if (stage == 2) {
        double u[NV];
        prim_to_cons<NV>(v, u, p.igmm1);
#pragma unroll
        for (int nv = 0; nv < NV; nv++) Us[nv * p.vstride + c] = u[nv];
      }
    }
    if constexpr (NV == NFLX + 2) {
      // ENTROPY_SWITCH: ComputeEntropy after Boundary (Src/entropy_switch.c:
      // 14-37), s = p / rho^gamma, once per zone; the ghost copies below and
      // in the x2 part carry it, and the stage kernels read it with the tile
      v[NV - 1] = v[PRS] * rho_pow(v[RHO], -p.gamma);
      V[(NV - 1) * p.vstride + c] = v[NV - 1];
    }
    if (!edge) return;
    // ghost layers: 2, or 3 with SHOCK_FLATTENING MULTID (GetNghost)
    const int b = p.beg[0], e = p.beg[0] + p.nx[0] - 1, nn = p.nx[0];
#pragma unroll
    for (int side = 0; side < 2; side++) {
      const int type = p.bc[side];
      int tg[3] = {-1, -1, -1};
      bool flip = false;
      const bool user = type == PS_BC_USERDEF;
      if (type == BC_OUTFLOW || user) {
        for (int k = 0; k < ng; k++) {
          if (side == 0 && gi == b) tg[k] = b - 1 - k;
          if (side == 1 && gi == e) tg[k] = e + 1 + k;
        }
      } else if (type == BC_PERIODIC) {
        if (side == 0 && gi >= e - (ng - 1)) tg[0] = gi - nn;
        if (side == 1 && gi <= b + (ng - 1)) tg[0] = gi + nn;
      } else if (type == BC_REFLECTIVE || type == BC_AXISYM || type == BC_EQTSYM) {
        flip = true;
        if (side == 0 && gi <= b + (ng - 1)) tg[0] = 2 * b - 1 - gi;
        if (side == 1 && gi >= e - (ng - 1)) tg[0] = 2 * e + 1 - gi;
      }
#pragma unroll
      for (int wi = 0; wi < 3; wi++) {
        const int t = tg[wi];
        if (t < 0) continue;
        const long long g = vcell(p, gj, t);
#pragma unroll
        for (int nv = 0; nv < NV; nv++) {
          double val = v[nv];
          if (flip && (nv == VX1 || (type == BC_AXISYM && nv == VX3))) val = -1 * val;
          if (user) val = side == 0 ? UserDefBoundary_X1Beg(nv, val) : UserDefBoundary_X1End(nv, val);
          V[nv * p.vstride + g] = val;
        }
      }
    }
  }
}

// K active cells per thread, q0 + k stride (k < K, below n): the densities
// and pressures of all K are loaded before any is processed, so that a
// pass in which few cells are floored is not bound by one load latency per
// cell.
template <int NV, int K>
__device__ __forceinline__ void bnd_x1_cells(double *V, double *Us, const Params &p,
                                             const WindParams &w, int stage, int q0, int stride,
                                             int n)
{
  double rho[K], prs[K];
  long long c[K];
  int gi[K], gj[K];
#pragma unroll
  for (int k = 0; k < K; k++) {
    const int q = q0 + k * stride;
    if (q < n) {
      const int j = q / p.nx[0];
      gi[k] = q - j * p.nx[0] + p.beg[0];
      gj[k] = j + p.beg[1];
      c[k] = vcell(p, gj[k], gi[k]);
      rho[k] = V[RHO * p.vstride + c[k]];
      prs[k] = V[PRS * p.vstride + c[k]];
    }
  }
#pragma unroll
  for (int k = 0; k < K; k++)
    if (q0 + k * stride < n) bnd_x1_cell_rp<NV>(V, Us, p, w, stage, gi[k], gj[k], c[k], rho[k], prs[k]);
}

// Boundary() part 2: the x2 ghost rows over every column (x1 ghosts
// included), after part 1 -- the side order of Boundary().
template <int NV>
__device__ __forceinline__ void bnd_x2_item(double *V, const Params &p, int q)
{
  {
    const int gi = q % p.ntot[0], r = q / p.ntot[0];
    const int ng = p.beg[1], side = r / ng, layer = r % ng;
    const int b = p.beg[1], e = p.beg[1] + p.nx[1] - 1, nn = p.nx[1];
    const int gj = side == 0 ? b - 1 - layer : e + 1 + layer;
    const int type = p.bc[2 + side];
    int src;
    bool flip = false;
    if (type == PS_BC_USERDEF) {
      // X2_BEG of the production problem (X2_END user sides are refused by
      // ps_set_wind): velocities mirrored, density and pressure copied
      const int mirror = 2 * b - 1 - gj;
#pragma unroll
      for (int nv = 0; nv < NV; nv++)
        V[nv * p.vstride + vcell(p, gj, gi)] = UserDefBoundary_X2Beg<NV>(
            nv, V[nv * p.vstride + vcell(p, mirror, gi)], V[nv * p.vstride + vcell(p, b, gi)]);
      return;
    }
    if (type == BC_OUTFLOW)
      src = side == 0 ? b : e;
    else if (type == BC_PERIODIC)
      src = side == 0 ? gj + nn : gj - nn;
    else {
      flip = true;
      src = side == 0 ? 2 * b - 1 - gj : 2 * e + 1 - gj;
    }
#pragma unroll
    for (int nv = 0; nv < NV; nv++) {
      double val = V[nv * p.vstride + vcell(p, src, gi)];
      if (flip && (nv == VX2 || (type == BC_AXISYM && nv == VX3))) val = -1 * val;
      V[nv * p.vstride + vcell(p, gj, gi)] = val;
    }
  }
}

// read_sirocco_heatcool(flag = 0): xi = L_x / n_H / r^2 from the state.
__device__ __forceinline__ void init_xi_cell(const double *V, double *xi, double *tr,
                                             const Params &p, const WindParams &w,
                                             const double *x1, int q)
{
  {
    const int gi = q % p.nx[0] + p.beg[0], gj = q / p.nx[0] + p.beg[1];
    const long long c = vcell(p, gj, gi);
    const double rho = V[RHO * p.vstride + c] * w.unit_density;
    const double r = x1[gi] * w.unit_length;
    const double nH = rho / (1.43 * kMP);
    xi[c] = w.lx / nH / (r * r);
    tr[c] = w.t_x;
  }
}

// ---------------------------------------------------------------
// BLONDIN heating/cooling, one thread per active cell
// (Src/Cooling/BLONDIN/cooling.c:50-165)
// ---------------------------------------------------------------

// The cell's BLONDIN context from the state; false when the cell is below
// the minimum cooling temperature and is left alone.  q is the active cell
// (x fastest, 2-D or 3-D); x1 is only read for the wind's xi.
__device__ __forceinline__ bool blondin_ctx(const double *V, const double *xi_s, const double *tr_s,
                                            const Params &p, const WindParams &w,
                                            const double *x1, double dt, double t, long long q,
                                            BlCtx &b, double &T, long long &c,
                                            const double *pre = nullptr)
{
  int gi, gj, gk;
  cell_of(p, q, gi, gj, gk);
  c = vcell3(p, gk, gj, gi);
  if (pre) {
    b.ch = pre[c];
    b.cc = pre[p.vstride + c];
    b.xh = pre[2 * p.vstride + c];
    b.lc = pre[3 * p.vstride + c];
    b.bc = pre[4 * p.vstride + c];
  }
  b.dt_share = dt * w.unit_time;
  const double rho = V[RHO * p.vstride + c] * w.unit_density;
  const double pr = V[PRS * p.vstride + c];
  b.E = (pr * w.unit_pressure) / (p.gamma - 1);
  b.nH = rho / (1.43 * kMP);
  if (w.xi_const > 0.0) {
    b.xi = w.xi_const;
    b.tx = w.t_x;
  } else if (t <= 3.0) {
    const double r = x1[gi] * w.unit_length;
    b.xi = w.lx / b.nH / r / r;
    b.tx = w.t_x;
  } else {
    b.xi = xi_s[c];
    b.tx = tr_s[c];
  }
  b.n = rho / (w.mu * kMP);
  T = b.E * (2.0 / 3.0) / (b.n * kKB);
  return T >= 1.e4;
}

// The new pressure of a cell from its final temperature (cooling.c:158-162).
__device__ __forceinline__ void blondin_store(double *V, const Params &p, const WindParams &w,
                                              const BlCtx &b, long long c, double T_f)
{
  T_f = dmax(T_f, 1.e4);
  const double E_f = T_f / (2.0 / 3.0) * (b.n * kKB);
  V[PRS * p.vstride + c] = E_f * (p.gamma - 1) / w.unit_pressure;
}

__device__ __forceinline__ void blondin_cell(double *V, const double *xi_s, const double *tr_s,
                                             const Params &p, const WindParams &w,
                                             const double *x1, Scalars *sc, double dt, double t,
                                             long long q, const double *pre = nullptr)
{
  BlCtx b;
  double T;
  long long c;
  if (!blondin_ctx(V, xi_s, tr_s, p, w, x1, dt, t, q, b, T, c, pre)) return;
  bl_prepare(b, T);
  bool overflow;
  const double T_f = bl_solve(b, T, overflow);
  if (overflow) atomicOr(&sc->flags, F_NAN);
  blondin_store(V, p, w, b, c, T_f);
}

// CoolingSource with the production Radiat on one cell (the ODE path,
// cooling = 2): the new pressure and this cell's bound on dt_cool, kept as
// the minimum over cells (positive doubles order as their bit patterns).
__device__ __forceinline__ void ode_wind_cell(double *V, const double *xi_s, const double *tr_s,
                                              const Params &p, const WindParams &w,
                                              const double *x1, Scalars *sc, double dt, double t,
                                              long long q, const double *pre)
{
  int gi, gj, gk;
  cell_of(p, q, gi, gj, gk);
  const long long c = vcell3(p, gk, gj, gi);
  OdeCell o;
  o.ch = o.cc = o.xh = o.lc = o.bc = 1.0;
  if (pre) {
    o.ch = pre[c];
    o.cc = pre[p.vstride + c];
    o.xh = pre[2 * p.vstride + c];
    o.lc = pre[3 * p.vstride + c];
    o.bc = pre[4 * p.vstride + c];
  }
  o.rho = V[RHO * p.vstride + c];
  o.trc = V[NFLX * p.vstride + c];
  o.rho_cgs_nH = o.rho * w.unit_density / (1.43 * kMP);
  if (t < 3.0) {
    const double r = x1[gi] * w.unit_length;
    o.xi = w.lx / o.rho_cgs_nH / r / r;
    o.tx = w.t_x;
  } else {
    o.xi = xi_s[c];
    o.tx = tr_s[c];
  }
  o.sqxi = sqrt(o.xi);
  o.sqsqxi = pow(o.xi, 0.25);
  o.gm1 = p.gmm1;
  o.kmu = w.kelvin * w.mu;
  o.e_cost = w.ode_e_cost;
  bool bad = false;
  double dtc = 1.e38;
  const double prs = ode_cool_cell(o, V[PRS * p.vstride + c], dt, w.ode_mu0_kelvin, dtc, bad);
  if (bad) {
    atomicOr(&sc->flags, F_COOLING);
    return;
  }
  V[PRS * p.vstride + c] = prs;
  if (dtc >= 0.0 && dtc < 1.e38)
    atomicMin(reinterpret_cast<unsigned long long *>(&sc->dt_cool),
              static_cast<unsigned long long>(__double_as_longlong(dtc)));
}

// ---------------------------------------------------------------
// spherical stage kernel
// ---------------------------------------------------------------

// bilinear() of line_connect.c:746-777 with the weights of the target
// point given: ans = (1-fy)((1-fx) v11 + fx v21) + fy((1-fx) v12 + fx v22)
// (products by dmul_t<INT>, ps_dmul.cuh: the same bits either way)
template <bool INT>
__device__ __forceinline__ void bilinear_w(double fx, double fy, const double (&v11)[2],
                                           const double (&v12)[2], const double (&v21)[2],
                                           const double (&v22)[2], double (&ans)[2], bool &bad)
{
  const double gx = 1.0 - fx, gy = 1.0 - fy;
#pragma unroll
  for (int k = 0; k < 2; k++) {
    const double t1 = fma(fx, v21[k], dmul_t<INT>(gx, v11[k], bad));
    const double t2 = fma(fx, v22[k], dmul_t<INT>(gx, v12[k], bad));
    ans[k] = fma(fy, t2, dmul_t<INT>(gy, t1, bad));
  }
}

// LineForce component `comp` (0: r, 1: theta) for the state vg of one cell
// (line_connect.c:815-903): sum over the cell's bins of
// (1 + M) sigma_e F / c, M = min(krad t^alpharad, 4400), t = sigma_e rho
// v_th / (dv/ds), M = 0 where dv/ds <= 0.  Evaluated for a cell with one
// bin as M = exp(lf_a0 + alpharad/2 log(rho p lq)) with lq = (dv/ds)^-2 from
// VGradCalc (one log and one exp per call); for cells with two or more bins
// as M = (rho p)^(alpharad/2) B, B = exp(lf_a0 - alpharad log(dv/ds)) formed
// once per stage in VGradCalc (one log and one exp per call).  The
// exponentials and logarithms are the table-driven ones of ps_fastmath.cuh
// (11 and 13 FP64 instructions against 15 and 29 for CUDA's).  With KRAD = ALPHARAD
// = 999, M is interpolated in the cell's table at log10 t = lt0 +
// log10(rho p)/2 + lq, lq = -log10(dv/ds).
constexpr unsigned long long kM4400 = 0x40B1300000000000ull;   // 4400.0

template <int NV>
__device__ __forceinline__ double line_force(const double (&vg)[NV], const LineList &L,
                                             const WindParams &w, int e0, int e1, int comp,
                                             long long cell, long long vstride)
{
  double g = 0.0;
  if (w.mfit) {
    // linterp (line_connect.c:778-808) of the cell's log10 M over log10 t:
    // the first point not below x by a linear scan, ends clamped
    const double base = w.lt0 + 0.5 * log10(vg[RHO] * vg[PRS]);
    const double *m = L.m_fit + cell;
    for (int e = e0; e < e1; e++) {
      double M = 0.0;
      if (L.lq[e] != -INFINITY) {
        const double x = base + L.lq[e];
        int idx = 0;
        while (idx < w.nm && L.t_fit[idx] < x) idx++;
        double y;
        if (idx == 0) {
          y = m[0];
        } else if (idx >= w.nm) {
          y = m[(w.nm - 1) * vstride];
        } else {
          const double x_low = L.t_fit[idx - 1], y_low = m[(idx - 1) * vstride];
          const double slope = (m[idx * vstride] - y_low) / (L.t_fit[idx] - x_low);
          y = y_low + slope * (x - x_low);
        }
        M = exp10(y);
        if (is_nan_bits(M)) M = 0.0;
        if (gt_pos<kM4400>(M)) M = 4400.;
      }
      const double F = comp == 0 ? L.Fr[e] : L.Ft[e];
      g += (1.0 + M) * F;
    }
    return g * w.lf_cf;
  }
  if (e1 - e0 >= 2) {
    // M = (rho p)^(alpharad/2) times the bin's factor from VGradCalc (0 where
    // dv/ds <= 0)
    const double Q = fm::exp(0.5 * w.alpharad * fm::log(vg[RHO] * vg[PRS]));
    for (int e = e0; e < e1; e++) {
      const double B = L.lq[e];
      double M = 0.0;
      if (gt0(B)) {
        M = Q * B;
        if (gt_pos<kM4400>(M)) M = 4400.;
      }
      const double F = comp == 0 ? L.Fr[e] : L.Ft[e];
      g += (1.0 + M) * F;
    }
    return g * w.lf_cf;
  }
  // one bin: M = exp(lf_a0 + alpharad/2 log(rho p) - alpharad log(dv/ds))
  // with the two logarithms as one, of rho p (dv/ds)^-2
  const double rp = vg[RHO] * vg[PRS];
  for (int e = e0; e < e1; e++) {
    const double q = L.lq[e];
    double M = 0.0;
    if (gt0(q)) {
      M = fm::exp(w.lf_a0 + 0.5 * w.alpharad * fm::log(rp * q));
      if (gt_pos<kM4400>(M)) M = 4400.;
    }
    const double F = comp == 0 ? L.Fr[e] : L.Ft[e];
    g += (1.0 + M) * F;
  }
  return g * w.lf_cf;
}

// CHAR: CHAR_LIMITING YES (a kernel of its own, so that the primitive
// path keeps its register budget)
// The right-hand side of one own cell in direction D (Src/MHD/rhs.c:234-351,
// 423-630; Src/MHD/rhs_source.c:101-420): -dt/dV (F_r A_r - F_l A_l) with
// the area and dt/dV folded into one weight per face (the phi momentum's
// face factors as well), the pressure gradient, the curvilinear source of
// the momentum along D, gravity and the line force `glf` (both along x1
// only in this problem; the reference's x2 and x3 components of gravity
// and the x3 component of the line force are exact zeros and are left
// out); with stage1 the cell's CFL sum `cdt` gains its term.  vc is the
// face-averaged state for D = 0 and the cell value for D = 1.  Products by
// dmul_t<INT> (on the integer pipes with INT, the same bits either way).
template <int D, int NV, bool INT, class G>
__device__ __forceinline__ void sph_rhs(const double *__restrict__ sf,
                                        const double *__restrict__ spr,
                                        const double *__restrict__ scm, const double (&vc)[NV],
                                        double glf, const WindStageArgs &A, int gi, int gj,
                                        int ql, int qr, double dt, double dtdV, bool stage1,
                                        double (&rhs)[NV], double &cdt, bool &bad)
{
  constexpr int VN = VX1 + D;
  const SphGeom &g = A.g;
  double Al, Ar, fl_phi, fr_phi, dtdl;
  if (D == 0) {
    Al = dmul_t<INT>(g.A1f[gi - 1], g.dmu[gj], bad);
    Ar = dmul_t<INT>(g.A1f[gi], g.dmu[gj], bad);
    fl_phi = g.absx1p[gi - 1];
    fr_phi = g.absx1p[gi];
    dtdl = A.s.dtdx[0][gi];
  } else {
    Al = dmul_t<INT>(g.rdr[gi], g.sxp[gj - 1], bad);
    Ar = dmul_t<INT>(g.rdr[gi], g.sxp[gj], bad);
    fl_phi = g.spabs[gj - 1];
    fr_phi = g.spabs[gj];
    dtdl = dmul_t<INT>(A.s.dtdx[1][gj], g.rtinv[gi], bad);
  }
  const double cl = dmul_t<INT>(dtdV, Al, bad), cr = -dmul_t<INT>(dtdV, Ar, bad);
#pragma unroll
  for (int nv = 0; nv < NV; nv++) {
    const double wl = nv == VX3 ? dmul_t<INT>(cl, fl_phi, bad) : cl;
    const double wr = nv == VX3 ? dmul_t<INT>(cr, fr_phi, bad) : cr;
    rhs[nv] = fma(sf[nv * G::NFMAX + ql], wl, dmul_t<INT>(sf[nv * G::NFMAX + qr], wr, bad));
  }
  rhs[VN] = fma(-dtdl, spr[qr] - spr[ql], rhs[VN]);
  rhs[VX3] = dmul_t<INT>(rhs[VX3], D == 0 ? g.inv_absx1[gi] : g.inv_sn[gj], bad);
  const double mflux = sf[RHO * G::NFMAX + qr] + sf[RHO * G::NFMAX + ql];
  const double dtr = dmul_t<INT>(dt, vc[RHO], bad);
  const double dtm = dmul_t<INT>(dhalf_t<INT>(dt, bad), mflux, bad);
  const double vphi = vc[VX3];
  if (D == 0) {
    const double Sm =
        dmul_t<INT>(vc[RHO], fma(vphi, vphi, dmul_t<INT>(vc[VX2], vc[VX2], bad)), bad);
    rhs[VX1] = fma(dmul_t<INT>(dt, Sm, bad), g.rinv[gi], rhs[VX1]);
    if (A.w.body_force) {
      const double g0 = g.g0[gi];
      rhs[VX1] = fma(dtr, g0, rhs[VX1]);
      rhs[PRS] = fma(dtm, g0, rhs[PRS]);
    }
  } else {
    const double Sm = dmul_t<INT>(
        vc[RHO],
        fma(dmul_t<INT>(g.ct[gj], vphi, bad), vphi, -dmul_t<INT>(vc[VX2], vc[VX1], bad)), bad);
    rhs[VX2] = fma(dmul_t<INT>(dt, Sm, bad), g.rtinv[gi], rhs[VX2]);
  }
  if (A.w.line_force) {
    rhs[VN] = fma(dtr, glf, rhs[VN]);
    rhs[PRS] = fma(dtm, glf, rhs[PRS]);
  }
  if (stage1) {
    const double inv_dl = D == 0 ? g.inv_dx1[gi] : dmul_t<INT>(g.inv_dx2[gj], g.rinv[gi], bad);
    cdt = fma(dhalf_t<INT>(scm[ql] + scm[qr], bad), inv_dl, cdt);
  }
}

template <int D, int NV, int LIM, int SOLVER, class TL, bool CHAR>
__device__ __forceinline__ void sweep_sph(const double *__restrict__ sv, double *__restrict__ svp,
                                          double *__restrict__ svm, double *__restrict__ sf,
                                          double *__restrict__ spr, double *__restrict__ scm,
                                          double (&U)[NV], double &cdt, bool own, int cx, int cy,
                                          int gi, int gj, double dt, double dtdV, int e0, int e1,
                                          const WindStageArgs &A, bool stage1, int ox, int oy)
{
  using G = TileGeom<TL>;
  constexpr bool IP = kIntProducts<NV, CHAR>;
  constexpr int PX = G::ext(0, D, 2), PY = G::ext(1, D, 2);
  constexpr int FX = G::ext(0, D, 1), FY = G::ext(1, D, 1);
  constexpr int NP = PX * PY, NF = FX * FY;
  constexpr int SST = D == 0 ? 1 : G::SX;
  constexpr int VN = VX1 + D;
  const Params &p = A.s.p;
  const SphGeom &g = A.g;
  const double gam = p.gamma;

  // (1) PLM with the general-grid weights of the cell, on the primitive or
  // (CHAR_LIMITING) the characteristic variables
  for (int q = threadIdx.x; q < NP; q += G::NT) {
    const int ix = q % PX, iy = q / PX;
    const int sx = ix + TL::HX - (D == 0), sy = iy + TL::HY - (D == 1);
    const int s0 = sy * G::SX + sx;
    // cells past the end of the grid (partial last tile) read the last
    // weights; their states are never used
    const int gc = min(D == 0 ? p.beg[0] + ox + ix - 1 : p.beg[1] + oy + iy - 1, p.ntot[D] - 1);
    const double cp = g.cp[D][gc], cm = g.cm[D][gc], wp = g.wp[D][gc], wm = g.wm[D][gc];
    const double dp = g.dp[D][gc], dm = g.dm[D][gc];
    bool minmod = false;
    if (p.shock) {
      // FLAG_MINMOD: this zone or a neighbour in either direction is shocked
      const int ci = p.beg[0] + ox + sx - TL::HX, cj = p.beg[1] + oy + sy - TL::HY;
      if (ci >= 1 && cj >= 1 && ci <= p.ntot[0] - 2 && cj <= p.ntot[1] - 2) {
        const unsigned char *S = A.shock;
        const long long c = vcell(p, cj, ci);
        minmod = ((S[c] | S[c - 1] | S[c + 1] | S[c - p.px] | S[c + p.px]) & 1) != 0;
      }
    }
    if constexpr (CHAR) {
      double v0[NV], dvp[NV], dvm[NV], dv[NV];
#pragma unroll
      for (int nv = 0; nv < NV; nv++) {
        v0[nv] = sv[nv * G::VS + s0];
        dvp[nv] = (sv[nv * G::VS + s0 + SST] - v0[nv]) * wp;
        dvm[nv] = (v0[nv] - sv[nv * G::VS + s0 - SST]) * wm;
      }
      char_slopes<D, NV, LIM>(v0, dvp, dvm, cp, cm, gam, minmod, dv);
#pragma unroll
      for (int nv = 0; nv < NV; nv++) {
        svp[nv * G::NPMAX + q] = v0[nv] + dv[nv] * dp;
        svm[nv * G::NPMAX + q] = v0[nv] - dv[nv] * dm;
      }
      continue;
    }
    if (minmod) {   // FLAG_MINMOD
#pragma unroll
      for (int nv = 0; nv < NV; nv++) {
        const double vm1 = sv[nv * G::VS + s0 - SST], v0 = sv[nv * G::VS + s0],
                     vp1 = sv[nv * G::VS + s0 + SST];
        const double dvp = (vp1 - v0) * wp, dvm = (v0 - vm1) * wm;
        const double dv = gt0(dvp * dvm) ? abs_min(dvp, dvm) : 0.0;
        svp[nv * G::NPMAX + q] = v0 + dv * dp;
        svm[nv * G::NPMAX + q] = v0 - dv * dm;
      }
      continue;
    }
    if constexpr (LIM == LIM_VL) {
      // on the FP64 unit: the integer form's live values cost the 16x16
      // tiles at three CTAs per multiprocessor more in spills than it saves.
      // Three variables per inversion (two divisions for six): shorter
      // dependent chains, 1.5% faster than one inversion for all six.
      bool bad = false;
      plm_vl_cell<NV, false, G, NV % 3 == 0 ? 3 : NV>(sv, svp, svm, s0, SST, q, wp, wm, cp, cm,
                                                       dp, dm, bad);
      continue;
    }
#pragma unroll
    for (int nv = 0; nv < NV; nv++) {
      const double vm1 = sv[nv * G::VS + s0 - SST], v0 = sv[nv * G::VS + s0],
                   vp1 = sv[nv * G::VS + s0 + SST];
      const double dvp = (vp1 - v0) * wp, dvm = (v0 - vm1) * wm;
      const double dv = limited_slope_general<LIM>(dvp, dvm, cp, cm);
      svp[nv * G::NPMAX + q] = v0 + dv * dp;
      svm[nv * G::NPMAX + q] = v0 - dv * dm;
    }
  }
  __syncthreads();

  // (2) Riemann problem at every face of the tile line
  for (int q = threadIdx.x; q < NF; q += G::NT) {
    const int fx = q % FX, fy = q / FX;
    const int pl = fy * PX + fx;
    constexpr int PST = D == 0 ? 1 : PX;
    double vL[NV], vR[NV], f[NV], pr, cmx;
#pragma unroll
    for (int nv = 0; nv < NV; nv++) {
      vL[nv] = svp[nv * G::NPMAX + pl];
      vR[nv] = svm[nv * G::NPMAX + pl + PST];
    }
    bool hll = false;
    if constexpr (SOLVER == HLLC) {
      if (p.shock) {
        // FLAG_HLL: the zone on either side of the face is shocked
        const int ci = p.beg[0] + ox + fx - (D == 0), cj = p.beg[1] + oy + fy - (D == 1);
        if (ci + (D == 0) <= p.ntot[0] - 1 && cj + (D == 1) <= p.ntot[1] - 1) {
          const long long c = vcell(p, cj, ci);
          hll = ((A.shock[c] | A.shock[c + (D == 0 ? 1 : p.px)]) & 1) != 0;
        }
      }
    }
    bool bad = false;
    riemann_t<NV, SOLVER, VN, IP>(vL, vR, gam, p.igmm1, f, pr, cmx, hll, bad);
    if constexpr (IP) {
      if (bad) riemann_t<NV, SOLVER, VN, false>(vL, vR, gam, p.igmm1, f, pr, cmx, hll, bad);
    }
#pragma unroll
    for (int nv = 0; nv < NV; nv++) sf[nv * G::NFMAX + q] = f[nv];
    spr[q] = pr;
    scm[q] = cmx;
  }
  __syncthreads();

  // (3) curvilinear flux difference, sources, update
  if (own) {
    const int ql = cy * FX + cx;
    constexpr int FST = D == 0 ? 1 : FX;
    const int qr = ql + FST;
    double vc[NV];
    if (D == 0) {
      // face-averaged state of the cell: mean of its own + and - states
      const int pc = cy * PX + cx + 1;
      bool bad = !IP;
      if constexpr (IP) {
#pragma unroll
        for (int nv = 0; nv < NV; nv++)
          vc[nv] = dhalf_int(svp[nv * G::NPMAX + pc] + svm[nv * G::NPMAX + pc], bad);
      }
      if (bad) {
#pragma unroll
        for (int nv = 0; nv < NV; nv++)
          vc[nv] = 0.5 * (svp[nv * G::NPMAX + pc] + svm[nv * G::NPMAX + pc]);
      }
    } else {
      const int s0 = (cy + TL::HY) * G::SX + cx + TL::HX;
#pragma unroll
      for (int nv = 0; nv < NV; nv++) vc[nv] = sv[nv * G::VS + s0];
    }
    const double glf =
        A.w.line_force ? line_force<NV>(vc, A.L, A.w, e0, e1, D, vcell(p, gj, gi), p.vstride) : 0.0;
    double rhs[NV], cdt1 = cdt;
    bool bad = false;
    sph_rhs<D, NV, IP, G>(sf, spr, scm, vc, glf, A, gi, gj, ql, qr, dt, dtdV, stage1, rhs, cdt1,
                          bad);
    if (IP && bad) {
      cdt1 = cdt;
      sph_rhs<D, NV, false, G>(sf, spr, scm, vc, glf, A, gi, gj, ql, qr, dt, dtdV, stage1, rhs,
                               cdt1, bad);
    }
#pragma unroll
    for (int nv = 0; nv < NV; nv++) U[nv] += rhs[nv];
    cdt = cdt1;
  }
  __syncthreads();
}

// dv/ds of one bin of VGradCalc (line_connect.c:690-717): the velocity at
// the bin's far point (bilinear in the cell's four corner velocities) and at
// the cell, projected on the bin's direction, differenced over the path.
template <bool INT>
__device__ __forceinline__ void vgrad_bin(const LineList &L, int e, double ids,
                                          const double (&v11)[2], const double (&v12)[2],
                                          const double (&v21)[2], const double (&v22)[2],
                                          const double (&ans1)[2], double &dvds, bool &bad)
{
  double ans2[2];
  bilinear_w<INT>(L.fr1[e], L.fr2[e], v11, v12, v21, v22, ans2, bad);
  const double v1 = fma(ans1[1], L.c1b[e], dmul_t<INT>(ans1[0], L.c1a[e], bad));
  const double v2 = fma(ans2[1], L.c2b[e], dmul_t<INT>(ans2[0], L.c2a[e], bad));
  dvds = dmul_t<INT>(fabs(v2 - v1), ids, bad);
}

// One tile (bx, by) of one stage of one wind grid.
template <int NV, int LIM, int SOLVER, int STAGE, class TL, bool CHAR>
__device__ __forceinline__ void stage_sph_tile(const CUtensorMap *tm, const WindStageArgs &A,
                                               int bx, int by, unsigned char *smem_raw)
{
  using G = TileGeom<TL>;
  constexpr bool IP = kIntProducts<NV, CHAR>;
  double *sv = reinterpret_cast<double *>(smem_raw);
  double *svp = sv + NV * G::VS;
  double *svm = svp + NV * G::NPMAX;
  double *sf = svm + NV * G::NPMAX;
  double *spr = sf + NV * G::NFMAX;
  double *scm = spr + G::NFMAX;
  uint64_t *bar = reinterpret_cast<uint64_t *>(scm + G::NFMAX);
  unsigned &s_flags = *reinterpret_cast<unsigned *>(bar + 1);
  unsigned long long *s_red = reinterpret_cast<unsigned long long *>(bar + 2);

  const StageArgs &a = A.s;
  if (a.sc->done) return;
  const Params &p = a.p;
  const int tid = threadIdx.x;
  const int ox = bx * TL::X, oy = by * TL::Y;
  if (tid == 0) {
    s_flags = 0;
    mbar_init(bar, 1);
  }
  __syncthreads();
  if (tid == 0) {
    mbar_expect_tx(bar, (uint32_t)(NV * G::VS * sizeof(double)));
    // x counts memory columns: an even x (16-byte start) for every tile
    tma_load_4d(sv, tm, ox + p.beg[0] - TL::HX + p.xoff, oy + p.beg[1] - TL::HY, 0, 0, bar);
  }
  const bool landed = mbar_wait_bounded(bar, 0, 1u << 22);
  if (!__syncthreads_and(landed)) {
    if (tid == 0) {
      atomicOr(&a.sc->flags, F_TMA_TIMEOUT);
      mbar_wait_bounded(bar, 0, 1u << 22);
    }
    return;
  }
  // (ENTROPY_SWITCH: the entropy plane of the tile holds s = p / rho^gamma of
  // every zone, as the boundary kernel's ComputeEntropy left it)

  // VGradCalc's corner velocities (line_connect.c:637-660: the mean of the
  // four zones that meet at a zone corner), formed once per corner of the
  // tile for the four zones that share it; kept in the flux buffer, which
  // the sweeps write only after their PLM pass
  constexpr int CX = TL::X + 1, CY = TL::Y + 1;
  static_assert(2 * CX * CY <= NV * G::NFMAX, "corner velocities fit the flux buffer");
  const double *cv1 = sf, *cv2 = sf + CX * CY;
  if (A.w.line_force) {
    const double *V1 = sv + VX1 * G::VS, *V2 = sv + VX2 * G::VS;
    for (int k = tid; k < CX * CY; k += G::NT) {
      const int kx = k % CX, ky = k / CX;
      const int s = (ky + TL::HY) * G::SX + kx + TL::HX, sm = s - G::SX;
      // the quotients by 4 as exact quarterings on the integer pipes
      const double s1 = V1[sm - 1] + V1[sm] + V1[s - 1] + V1[s];
      const double s2 = V2[sm - 1] + V2[sm] + V2[s - 1] + V2[s];
      bool bad = !IP;
      double c1 = 0.0, c2 = 0.0;
      if constexpr (IP) {
        c1 = dpow2m_int<2>(s1, bad);
        c2 = dpow2m_int<2>(s2, bad);
      }
      if (bad) {
        c1 = s1 / 4.0;
        c2 = s2 / 4.0;
      }
      sf[k] = c1;
      sf[CX * CY + k] = c2;
    }
    __syncthreads();
  }

  const int cx = tid % TL::X, cy = tid / TL::X;
  const bool own = tid < G::NC && (ox + cx < p.nx[0]) && (oy + cy < p.nx[1]);
  const int gi = p.beg[0] + ox + cx, gj = p.beg[1] + oy + cy;
  const long long cell = vcell(p, gj, gi);
  const double dt = a.sc->dt;
  const SphGeom &g = A.g;

  double U[NV];
  double cdt = 0.0, dtdV = 0.0;
  int e0 = 0, e1 = 0;
  unsigned flags = 0;
  if (own) {
    bool bad = false;
    if constexpr (STAGE == 1) {
      double v[NV];
      const int s0 = (cy + TL::HY) * G::SX + cx + TL::HX;
#pragma unroll
      for (int nv = 0; nv < NV; nv++) v[nv] = sv[nv * G::VS + s0];
      prim_to_cons_t<NV, IP>(v, U, p.igmm1, bad);
      if (IP && bad) prim_to_cons_t<NV, false>(v, U, p.igmm1, bad);
    } else {
#pragma unroll
      for (int nv = 0; nv < NV; nv++) U[nv] = a.Us[nv * p.vstride + cell];
    }
    bad = bad || !IP;
    if constexpr (IP) dtdV = dmul_int(dmul_int(dt, g.inv_dVr[gi], bad), g.inv_dmu[gj], bad);
    if (bad) dtdV = dt * g.inv_dVr[gi] * g.inv_dmu[gj];
    if (A.w.line_force) {
      // VGradCalc for the bins of this cell (line_connect.c:628-738)
      const int dc = (oy + cy) * p.nx[0] + (ox + cx);
      e0 = A.L.off[dc];
      e1 = A.L.off[dc + 1];
      // the corners (i-1/2, j-1/2), (i-1/2, j+1/2), (i+1/2, j+1/2), (i+1/2, j-1/2)
      const int k0 = cy * CX + cx;
      double v11[2], v12[2], v21[2], v22[2], ans1[2];
      v11[0] = cv1[k0];
      v11[1] = cv2[k0];
      v12[0] = cv1[k0 + CX];
      v12[1] = cv2[k0 + CX];
      v22[0] = cv1[k0 + CX + 1];
      v22[1] = cv2[k0 + CX + 1];
      v21[0] = cv1[k0 + 1];
      v21[1] = cv2[k0 + 1];
      bool bad = false;
      bilinear_w<IP>(g.fx[gi], g.fy[gj], v11, v12, v21, v22, ans1, bad);
      if (IP && bad) bilinear_w<false>(g.fx[gi], g.fy[gj], v11, v12, v21, v22, ans1, bad);
      const double alpha = A.w.alpharad;
      // two or more bins: the bin's factor k C^alpha (dv/ds)^-alpha is kept
      // instead of its log, so that each sweep needs one power of rho p and
      // a product per bin (line_force)
      const bool fact = e1 - e0 >= 2;
      for (int e = e0; e < e1; e++) {
        const double ids = A.L.inv_ds[e];
        double lq = A.w.mfit ? -INFINITY : 0.0;
        if (ids != 0.0) {
          double dvds;
          bool badb = false;
          vgrad_bin<IP>(A.L, e, ids, v11, v12, v21, v22, ans1, dvds, badb);
          if (IP && badb) vgrad_bin<false>(A.L, e, ids, v11, v12, v21, v22, ans1, dvds, badb);
          if (is_nan_bits(dvds)) flags |= F_NAN;
          if (gt0(dvds))
            lq = A.w.mfit ? -log10(dvds)
                 : fact   ? fm::exp(A.w.lf_a0 - alpha * fm::log(dvds))
                          : 1.0 / (dvds * dvds);
        }
        A.L.lq[e] = lq;
      }
    }
  }

  sweep_sph<0, NV, LIM, SOLVER, TL, CHAR>(sv, svp, svm, sf, spr, scm, U, cdt, own, cx, cy, gi, gj, dt,
                                    dtdV, e0, e1, A, STAGE == 1, ox, oy);
  sweep_sph<1, NV, LIM, SOLVER, TL, CHAR>(sv, svp, svm, sf, spr, scm, U, cdt, own, cx, cy, gi, gj, dt,
                                    dtdV, e0, e1, A, STAGE == 1, ox, oy);

  if (own) {
    double v[NV];
    int ent = 0;
    if constexpr (NV == NFLX + 2) {
      // FLAG_ENTROPY: every zone with ALWAYS; with SELECTIVE not in or next
      // to a compressive zone with a pressure jump above 0.05 min(p)
      ent = 2;
      if (p.entropy == 1) {
        const unsigned char *S = A.shock;
        const unsigned char e = S[cell] | S[cell - 1] | S[cell + 1] | S[cell - p.px] |
                                S[cell + p.px];
        if (e & 2) ent = 1;
      }
    }
    // stage 2: U = (U0 + U*) / 2 with U0 from V^n; then the primitive state
    // (the integer form first, again on the FP64 unit if it hands back)
    double Uw[NV];
    bool bad = false;
#pragma unroll
    for (int nv = 0; nv < NV; nv++) Uw[nv] = U[nv];
    unsigned f = stage_out<NV, STAGE, IP>(Uw, v, a, p, cell, ent, bad);
    if (IP && bad) {
#pragma unroll
      for (int nv = 0; nv < NV; nv++) Uw[nv] = U[nv];
      f = stage_out<NV, STAGE, false>(Uw, v, a, p, cell, ent, bad);
    }
#pragma unroll
    for (int nv = 0; nv < NV; nv++) U[nv] = Uw[nv];
    flags |= f;
#pragma unroll
    for (int nv = 0; nv < NV; nv++)
      if (is_nan_bits(v[nv])) flags |= F_NAN;
#pragma unroll
    for (int nv = 0; nv < NV; nv++) {
      if constexpr (STAGE == 1) a.Us[nv * p.vstride + cell] = U[nv];
      a.Vout[nv * p.vstride + cell] = v[nv];
    }
  }
  if (flags) atomicOr(&s_flags, flags);
  if constexpr (STAGE == 1) {
    unsigned long long b = (unsigned long long)__double_as_longlong(cdt);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      unsigned long long ob = __shfl_xor_sync(0xffffffffu, b, o);
      b = ob > b ? ob : b;
    }
    if ((tid & 31) == 0) s_red[tid >> 5] = b;
  }
  __syncthreads();
  if (tid == 0) {
    if constexpr (STAGE == 1) {
      unsigned long long b = 0;
#pragma unroll
      for (int w = 0; w < G::NT / 32; w++) b = s_red[w] > b ? s_red[w] : b;
      atomicMax(&a.sc->cdt_bits, b);
    }
    if (s_flags) {
      atomicOr(&a.sc->flags, s_flags);
      if (s_flags & F_NAN) a.sc->done = 1;
    }
  }
}


}  // namespace ps
