/* ps_oracle.c -- CPU oracle for the PLUTO-sirocco hydro step.
 *
 * TEST INFRASTRUCTURE ONLY (see ps_oracle.h).  A plain-C restatement of the
 * reference algorithm, organised like the reference (1-D row sweeps over a
 * gathered copy of each row) so that every floating-point operation happens
 * in the same order and the result is bit-identical to the reference's own
 * serial build compiled with gcc -O3 -ffp-contract=off.
 *
 * Reference files followed (paths inside the reference project):
 *   grid            Src/set_grid.c:100-140 (ghosts), 405-450 (patches)
 *   geometry        Src/set_geometry.c:243-250 (inv_dx)
 *   PLM             Src/States/plm_states.c:83-338, Src/States/plm_coeffs.h:72-180
 *   prim<->cons     Src/HD/mappers.c:26-200
 *   sound speed     Src/EOS/Ideal/eos.c:16-42
 *   flux            Src/HD/fluxes.c:23-51
 *   wave speeds     Src/HD/hll_speed.c:24-91, Src/HD/eigenv.c:34-65
 *   Riemann         Src/HD/hllc.c:28-180, Src/HD/hll.c:30-107, Src/adv_flux.c:47
 *   RHS             Src/MHD/rhs.c:84-420
 *   stage           Src/Time_Stepping/update_stage.c:35-410
 *   RK2             Src/Time_Stepping/rk_step.c:18-20, 29-384
 *   boundaries      Src/boundary.c:56-760
 *   main loop / dt  Src/main.c:215-337, 383-497, 521-697
 */
#include "ps_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define RHO 0
#define VX1 1
#define VX2 2
#define VX3 3
#define PRS 4
#define NFLX 5
#define NVMAX 16

#define MAXD(a, b) ((a) >= (b) ? (a) : (b))
#define MIND(a, b) ((a) <= (b) ? (a) : (b))
#define ABS_MIN(a, b) (fabs(a) < fabs(b) ? (a) : (b))

static const double small_density = 1.e-12;
static const double small_pressure = 1.e-12;

struct or_sim {
  or_config c;
  int ngh[3], ntot[3], beg[3], end[3];
  double *x[3], *xl[3], *xr[3], *dx[3], *inv_dx[3];
  double *V;     /* [nv][k][j][i] */
  double *U;     /* [k][j][i][nv] */
  double *U0;    /* [k][j][i][nv] */
  double *Cdt;   /* [k][j][i]     */
  /* row workspace, [i][nv] */
  double *rv, *rvp, *rvm, *rup, *rum, *rdv, *rflux, *rrhs, *rfL, *rfR;
  double *rpress, *rpL, *rpR, *ra2L, *ra2R, *rcmax, *rSL, *rSR;
  double g_time, g_dt;
  long step;
  double invDt_hyp, dt_cool;
  int fail;
  int nhist;
  double *hist_dt, *hist_inv;
  int hist_cap;
};

/* ------------------------------------------------------------------ */
/* grid                                                                */
/* ------------------------------------------------------------------ */

/* Active-cell patch (Src/set_grid.c:405-450).  xl/xr/dx are indexed from
 * the first active cell. */
static void make_patch(int type, int n, double xL, double xR, double ratio,
                       double *xl, double *xr, double *dx)
{
  int i;
  if (type == OR_GRID_UNIFORM) {
    for (i = 0; i < n; i++) {
      dx[i] = (xR - xL) / (double)(n);
      xl[i] = xL + (double)(i)*dx[i];
      xr[i] = xl[i] + dx[i];
    }
  } else if (type == OR_GRID_LOG_INC) {
    double dy = log10((xR + fabs(xL) - xL) / fabs(xL));
    dy /= (double)(n);
    xl[0] = xL;
    for (i = 0; i < n; i++) {
      dx[i] = (xl[i] + fabs(xL) - xL) * (pow(10.0, dy) - 1.0);
      xr[i] = xl[i] + dx[i];
      if (i + 1 < n) xl[i + 1] = xr[i];
    }
  } else { /* OR_GRID_RATIO */
    xl[0] = xL;
    dx[0] = (xR - xL) * (ratio - 1.0) / (pow(ratio, n) - 1.0);
    xr[0] = xl[0] + dx[0];
    for (i = 1; i < n; i++) {
      dx[i] = dx[i - 1] * ratio;
      xl[i] = xl[i - 1] + dx[i - 1];
      xr[i] = xl[i] + dx[i];
    }
  }
}

static void build_grid(or_sim *s, int d)
{
  int ngh = s->ngh[d], n = s->c.nx[d], nt = s->ntot[d];
  int ib = ngh, ie = ngh + n - 1, i;
  double *x, *xl, *xr, *dx;
  x  = s->x[d]  = calloc(nt, sizeof(double));
  xl = s->xl[d] = calloc(nt, sizeof(double));
  xr = s->xr[d] = calloc(nt, sizeof(double));
  dx = s->dx[d] = calloc(nt, sizeof(double));
  s->inv_dx[d] = calloc(nt, sizeof(double));
  make_patch(s->c.gridtype[d], n, s->c.xbeg[d], s->c.xend[d], s->c.ratio[d],
             xl + ib, xr + ib, dx + ib);
  for (i = 0; i < ngh; i++) {
    dx[i] = dx[ib];
    xl[i] = xl[ib] - (ngh - i) * dx[ib];
    xr[i] = xl[i] + dx[ib];
    dx[ie + i + 1] = dx[ie];
    xl[ie + i + 1] = xl[ie] + (i + 1) * dx[ie];
    xr[ie + i + 1] = xl[ie] + (i + 2) * dx[ie];
  }
  for (i = 0; i < nt; i++) x[i] = 0.5 * (xl[i] + xr[i]);
  for (i = 0; i < nt; i++) s->inv_dx[d][i] = 1.0 / (dx[i]);
}

/* ------------------------------------------------------------------ */
/* lifecycle                                                           */
/* ------------------------------------------------------------------ */

or_sim *or_create(const or_config *cfg)
{
  or_sim *s = calloc(1, sizeof(or_sim));
  int d, nmax = 0, nv = cfg->nvar;
  size_t ncell;
  s->c = *cfg;
  for (d = 0; d < 3; d++) {
    s->ngh[d] = (d < cfg->dims) ? 2 : 0;
    s->ntot[d] = cfg->nx[d] + 2 * s->ngh[d];
    s->beg[d] = s->ngh[d];
    s->end[d] = s->ngh[d] + cfg->nx[d] - 1;
    if (s->ntot[d] > nmax) nmax = s->ntot[d];
    build_grid(s, d);
  }
  ncell = (size_t)s->ntot[0] * s->ntot[1] * s->ntot[2];
  s->V = calloc(ncell * nv, sizeof(double));
  s->U = calloc(ncell * nv, sizeof(double));
  s->U0 = calloc(ncell * nv, sizeof(double));
  s->Cdt = calloc(ncell, sizeof(double));
#define ROWBUF(p) p = calloc((size_t)(nmax + 2) * NVMAX, sizeof(double))
  ROWBUF(s->rv); ROWBUF(s->rvp); ROWBUF(s->rvm); ROWBUF(s->rup);
  ROWBUF(s->rum); ROWBUF(s->rdv); ROWBUF(s->rflux); ROWBUF(s->rrhs);
  ROWBUF(s->rfL); ROWBUF(s->rfR);
#undef ROWBUF
#define ROW1(p) p = calloc((size_t)(nmax + 2), sizeof(double))
  ROW1(s->rpress); ROW1(s->rpL); ROW1(s->rpR); ROW1(s->ra2L); ROW1(s->ra2R);
  ROW1(s->rcmax); ROW1(s->rSL); ROW1(s->rSR);
#undef ROW1
  s->g_time = 0.0;
  s->g_dt = cfg->first_dt;
  s->step = 0;
  s->invDt_hyp = 0.0;
  s->dt_cool = 1.e38;
  return s;
}

void or_destroy(or_sim *s)
{
  int d;
  if (!s) return;
  for (d = 0; d < 3; d++) {
    free(s->x[d]); free(s->xl[d]); free(s->xr[d]); free(s->dx[d]);
    free(s->inv_dx[d]);
  }
  free(s->V); free(s->U); free(s->U0); free(s->Cdt);
  free(s->rv); free(s->rvp); free(s->rvm); free(s->rup); free(s->rum);
  free(s->rdv); free(s->rflux); free(s->rrhs); free(s->rfL); free(s->rfR);
  free(s->rpress); free(s->rpL); free(s->rpR); free(s->ra2L); free(s->ra2R);
  free(s->rcmax); free(s->rSL); free(s->rSR);
  free(s->hist_dt); free(s->hist_inv);
  free(s);
}

int or_ntot(const or_sim *s, int dir) { return s->ntot[dir]; }
int or_nghost(const or_sim *s, int dir) { return s->ngh[dir]; }
double *or_state(or_sim *s) { return s->V; }

const double *or_grid(const or_sim *s, int dir, int which)
{
  switch (which) {
    case 0: return s->x[dir];
    case 1: return s->xl[dir];
    case 2: return s->xr[dir];
    default: return s->dx[dir];
  }
}

void or_time(const or_sim *s, double *t, double *dt, long *step)
{
  if (t) *t = s->g_time;
  if (dt) *dt = s->g_dt;
  if (step) *step = s->step;
}

void or_set_time(or_sim *s, double t, double dt, long step)
{
  s->g_time = t;
  s->g_dt = dt;
  s->step = step;
}

int or_history(const or_sim *s, double *dt_used, double *inv_dt, int max)
{
  int n = s->nhist < max ? s->nhist : max, i;
  for (i = 0; i < n; i++) {
    if (dt_used) dt_used[i] = s->hist_dt[i];
    if (inv_dt) inv_dt[i] = s->hist_inv[i];
  }
  return n;
}

/* ------------------------------------------------------------------ */
/* indexing helpers                                                    */
/* ------------------------------------------------------------------ */

static inline size_t cidx(const or_sim *s, int k, int j, int i)
{
  return ((size_t)k * s->ntot[1] + j) * s->ntot[0] + i;
}

static inline size_t vidx(const or_sim *s, int nv, int k, int j, int i)
{
  return (size_t)nv * s->ntot[0] * s->ntot[1] * s->ntot[2] + cidx(s, k, j, i);
}

/* ------------------------------------------------------------------ */
/* initial condition                                                   */
/* ------------------------------------------------------------------ */

/* 64-bit Mersenne Twister MT19937-64 (Matsumoto & Nishimura 2004, the
 * published algorithm), as selected by PRNG_MT in
 * Src/Math_Tools/math_random.c:36-105; real numbers on [0, 1] are
 * (x >> 11) / (2^53 - 1). */
#define MT_NN 312
#define MT_MM 156
typedef struct { uint64_t mt[MT_NN]; int mti; } or_mt64;

static void mt64_seed(or_mt64 *g, uint64_t seed)
{
  int i;
  g->mt[0] = seed;
  for (i = 1; i < MT_NN; i++)
    g->mt[i] = 6364136223846793005ull * (g->mt[i - 1] ^ (g->mt[i - 1] >> 62)) + (uint64_t)i;
  g->mti = MT_NN;
}

static uint64_t mt64_next(or_mt64 *g)
{
  const uint64_t upper = 0xFFFFFFFF80000000ull, lower = 0x7FFFFFFFull;
  const uint64_t mag = 0xB5026F5AA96619E9ull;
  uint64_t x;
  int i;
  if (g->mti >= MT_NN) {
    for (i = 0; i < MT_NN; i++) {
      x = (g->mt[i] & upper) | (g->mt[(i + 1) % MT_NN] & lower);
      g->mt[i] = g->mt[(i + MT_MM) % MT_NN] ^ (x >> 1) ^ ((x & 1ull) ? mag : 0ull);
    }
    g->mti = 0;
  }
  x = g->mt[g->mti++];
  x ^= (x >> 29) & 0x5555555555555555ull;
  x ^= (x << 17) & 0x71D67FFFEDA60000ull;
  x ^= (x << 37) & 0xFFF7EEE000000000ull;
  x ^= (x >> 43);
  return x;
}

static double mt64_real1(or_mt64 *g)
{
  return (double)(mt64_next(g) >> 11) * (1.0 / 9007199254740991.0);
}

void or_init_blast(or_sim *s, double p_amb, double p_in, double r_in,
                   double noise, long seed)
{
  int i, j, k, nv;
  or_mt64 g;
  size_t ncell = (size_t)s->ntot[0] * s->ntot[1] * s->ntot[2];
  /* whole box (ghosts included) starts at the ambient state */
  for (nv = 0; nv < s->c.nvar; nv++) {
    double val = (nv == RHO) ? 1.0 : (nv == PRS ? p_amb : 0.0);
    for (size_t q = 0; q < ncell; q++) s->V[(size_t)nv * ncell + q] = val;
  }
  mt64_seed(&g, (uint64_t)seed);
  for (k = s->beg[2]; k <= s->end[2]; k++)
  for (j = s->beg[1]; j <= s->end[1]; j++)
  for (i = s->beg[0]; i <= s->end[0]; i++) {
    double rnd = mt64_real1(&g);
    double ax, ay, az, r2, r;
    s->V[vidx(s, RHO, k, j, i)] = 1.0 * (1.0 + (-noise + rnd * (noise - (-noise))));
    s->V[vidx(s, VX1, k, j, i)] = 0.0;
    s->V[vidx(s, VX2, k, j, i)] = 0.0;
    s->V[vidx(s, VX3, k, j, i)] = 0.0;
    ax = s->x[0][i] - 0.5;
    ay = s->x[1][j] - 0.5;
    r2 = ax * ax + ay * ay;
    if (s->c.dims == 3) {
      az = s->x[2][k] - 0.5;
      r2 = r2 + az * az;
    }
    r = sqrt(r2);
    s->V[vidx(s, PRS, k, j, i)] = (r < r_in) ? p_in : p_amb;
  }
}

/* ------------------------------------------------------------------ */
/* boundary conditions (Src/boundary.c:56-760)                          */
/* ------------------------------------------------------------------ */

static void boundary(or_sim *s)
{
  int side, nv, i, j, k;
  int nvar = s->c.nvar;
  for (side = 0; side < 6; side++) {
    int d = side / 2, isend = side % 2;
    int type = s->c.bc[side];
    int lo[3], hi[3];
    int vsign[NVMAX];
    if (d >= s->c.dims) continue;
    lo[0] = 0; hi[0] = s->ntot[0] - 1;
    lo[1] = 0; hi[1] = s->ntot[1] - 1;
    lo[2] = 0; hi[2] = s->ntot[2] - 1;
    if (!isend) { lo[d] = 0; hi[d] = s->beg[d] - 1; }
    else        { lo[d] = s->end[d] + 1; hi[d] = s->ntot[d] - 1; }
    for (nv = 0; nv < nvar; nv++) vsign[nv] = 1;
    if (type == OR_BC_REFLECTIVE || type == OR_BC_AXISYMMETRIC ||
        type == OR_BC_EQTSYMMETRIC) {
      vsign[VX1 + d] = -1;
      if (type == OR_BC_AXISYMMETRIC && s->c.geometry != OR_CARTESIAN)
        vsign[VX3] = -1;
    }
    for (nv = 0; nv < nvar; nv++)
    for (k = lo[2]; k <= hi[2]; k++)
    for (j = lo[1]; j <= hi[1]; j++)
    for (i = lo[0]; i <= hi[0]; i++) {
      int src[3] = {i, j, k};
      int n = s->c.nx[d];
      int idx = src[d];
      double val;
      if (type == OR_BC_OUTFLOW) {
        src[d] = isend ? s->end[d] : s->beg[d];
      } else if (type == OR_BC_PERIODIC) {
        src[d] = isend ? idx - n : idx + n;
      } else if (type == OR_BC_REFLECTIVE || type == OR_BC_AXISYMMETRIC ||
                 type == OR_BC_EQTSYMMETRIC) {
        int i0 = isend ? 2 * s->end[d] + 1 : 2 * s->beg[d] - 1;
        src[d] = i0 - idx;
      } else {
        continue; /* user-defined sides are filled by the caller */
      }
      val = s->V[vidx(s, nv, src[2], src[1], src[0])];
      if (type == OR_BC_OUTFLOW || type == OR_BC_PERIODIC)
        s->V[vidx(s, nv, k, j, i)] = val;
      else
        s->V[vidx(s, nv, k, j, i)] = vsign[nv] * val;
    }
  }
}

/* ------------------------------------------------------------------ */
/* prim <-> cons (Src/HD/mappers.c:26-200)                             */
/* ------------------------------------------------------------------ */

static inline void prim_to_cons(const double *v, double *u, int nvar, double gmm1)
{
  double rho = v[RHO];
  int nv;
  u[RHO] = rho;
  u[VX1] = rho * v[VX1];
  u[VX2] = rho * v[VX2];
  u[VX3] = rho * v[VX3];
  u[PRS] = v[VX1] * v[VX1] + v[VX2] * v[VX2] + v[VX3] * v[VX3];
  u[PRS] = 0.5 * rho * u[PRS] + v[PRS] / gmm1;
  for (nv = NFLX; nv < nvar; nv++) u[nv] = rho * v[nv];
}

/* returns nonzero flag bits on failure (64 = cons2prim fail) */
static inline int cons_to_prim(double *u, double *v, int nvar, double gmm1)
{
  int flag = 0, nv;
  double m2 = u[VX1] * u[VX1] + u[VX2] * u[VX2] + u[VX3] * u[VX3];
  double tau, kin, rho;
  if (u[RHO] < 0.0) {
    u[RHO] = small_density;
    flag |= 64 | 512;
  }
  v[RHO] = rho = u[RHO];
  tau = 1.0 / u[RHO];
  v[VX1] = u[VX1] * tau;
  v[VX2] = u[VX2] * tau;
  v[VX3] = u[VX3] * tau;
  kin = 0.5 * m2 / u[RHO];
  if (u[PRS] < 0.0) {
    u[PRS] = small_pressure / gmm1 + kin;
    flag |= 64;
  }
  v[PRS] = gmm1 * (u[PRS] - kin);
  if (v[PRS] < 0.0) {
    v[PRS] = small_pressure;
    u[PRS] = v[PRS] / gmm1 + kin;
    flag |= 64;
  }
  (void)rho;
  for (nv = NFLX; nv < nvar; nv++) v[nv] = u[nv] * tau;
  return flag;
}

/* ------------------------------------------------------------------ */
/* one row sweep                                                       */
/* ------------------------------------------------------------------ */

#define R(p, i, nv) (p)[(size_t)(i) * NVMAX + (nv)]

static inline double limit(int lim, double dvp, double dvm)
{
  double dv;
  if (lim == OR_LIM_MC) {
    if (dvp * dvm > 0.0) {
      double qc = 0.5 * (dvm + dvp), scrh = 2.0 * ABS_MIN(dvp, dvm);
      dv = ABS_MIN(qc, scrh);
    } else dv = 0.0;
  } else if (lim == OR_LIM_VL) {
    dv = (dvp * dvm > 0.0 ? 2.0 * dvp * dvm / (dvp + dvm) : 0.0);
  } else {
    dv = (dvp * dvm > 0.0 ? ABS_MIN(dvp, dvm) : 0.0);
  }
  return dv;
}

static void row_sweep(or_sim *s, int d, int k0, int j0, int i0, int stage,
                      double dt)
{
  int nvar = s->c.nvar, nt = s->ntot[d];
  int nbeg = s->beg[d], nend = s->end[d];
  int i, nv;
  int vn = VX1 + d;
  double gmm1 = s->c.gamma - 1.0, gam = s->c.gamma;
  size_t stride = (d == 0) ? 1 : (d == 1 ? (size_t)s->ntot[0]
                                         : (size_t)s->ntot[0] * s->ntot[1]);
  size_t base = cidx(s, k0, j0, i0);
  size_t nc = (size_t)s->ntot[0] * s->ntot[1] * s->ntot[2];
  double *v = s->rv, *vp = s->rvp, *vm = s->rvm, *up = s->rup, *um = s->rum;
  double *dvv = s->rdv, *fl = s->rflux, *rhs = s->rrhs;
  double *fL = s->rfL, *fR = s->rfR;
  double *pr = s->rpress, *pL = s->rpL, *pR = s->rpR;
  double *a2L = s->ra2L, *a2R = s->ra2R, *cmax = s->rcmax;
  double *SL = s->rSL, *SR = s->rSR;
  int beg, end;

  /* gather the row (update_stage.c:186-195) */
  for (i = 0; i < nt; i++)
    for (nv = 0; nv < nvar; nv++) R(v, i, nv) = s->V[nv * nc + base + i * stride];

  /* PLM states on [nbeg-1, nend+1] (plm_states.c:83-338) */
  beg = nbeg - 1; end = nend + 1;
  for (i = beg - 1; i <= end; i++)
    for (nv = 0; nv < nvar; nv++) R(dvv, i, nv) = R(v, i + 1, nv) - R(v, i, nv);
  for (i = beg; i <= end; i++) {
    for (nv = 0; nv < nvar; nv++) {
      double dvp = R(dvv, i, nv), dvm = R(dvv, i - 1, nv);
      double dvl = limit(s->c.limiter, dvp, dvm);
      R(vp, i, nv) = R(v, i, nv) + dvl * 0.5;
      R(vm, i, nv) = R(v, i, nv) - dvl * 0.5;
    }
    prim_to_cons(&R(vp, i, 0), &R(up, i, 0), nvar, gmm1);
    prim_to_cons(&R(vm, i, 0), &R(um, i, 0), nvar, gmm1);
  }

  /* Riemann problem at interfaces i+1/2, i in [nbeg-1, nend];
   * left state = vp[i], right state = vm[i+1] (hllc.c / hll.c) */
  for (i = nbeg - 1; i <= nend; i++) {
    const double *vL = &R(vp, i, 0), *vR = &R(vm, i + 1, 0);
    const double *uL = &R(up, i, 0), *uR = &R(um, i + 1, 0);
    double *f = &R(fl, i, 0), *FL = &R(fL, i, 0), *FR = &R(fR, i, 0);
    double aL, aR;
    a2L[i] = gam * vL[PRS] / vL[RHO];
    a2R[i] = gam * vR[PRS] / vR[RHO];
    /* Flux() */
    FL[RHO] = uL[vn];
    FL[VX1] = uL[VX1] * vL[vn];
    FL[VX2] = uL[VX2] * vL[vn];
    FL[VX3] = uL[VX3] * vL[vn];
    pL[i] = vL[PRS];
    FL[PRS] = (uL[PRS] + vL[PRS]) * vL[vn];
    FR[RHO] = uR[vn];
    FR[VX1] = uR[VX1] * vR[vn];
    FR[VX2] = uR[VX2] * vR[vn];
    FR[VX3] = uR[VX3] * vR[vn];
    pR[i] = vR[PRS];
    FR[PRS] = (uR[PRS] + vR[PRS]) * vR[vn];
    /* Davis estimate */
    aL = sqrt(a2L[i]);
    aR = sqrt(a2R[i]);
    SL[i] = MIND(vL[vn] - aL, vR[vn] - aR);
    SR[i] = MAXD(vL[vn] + aL, vR[vn] + aR);
    cmax[i] = MAXD(fabs(SL[i]), fabs(SR[i]));

    if (SL[i] > 0.0) {
      for (nv = 0; nv < NFLX; nv++) f[nv] = FL[nv];
      pr[i] = pL[i];
    } else if (SR[i] < 0.0) {
      for (nv = 0; nv < NFLX; nv++) f[nv] = FR[nv];
      pr[i] = pR[i];
    } else if (s->c.solver == OR_HLL) {
      double scrh = 1.0 / (SR[i] - SL[i]);
      for (nv = 0; nv < NFLX; nv++) {
        f[nv] = SL[i] * SR[i] * (uR[nv] - uL[nv]) + SR[i] * FL[nv] - SL[i] * FR[nv];
        f[nv] *= scrh;
      }
      pr[i] = (SR[i] * pL[i] - SL[i] * pR[i]) * scrh;
    } else {
      double vxl = vL[vn], vxr = vR[vn];
      double qL = vL[PRS] + uL[vn] * (vL[vn] - SL[i]);
      double qR = vR[PRS] + uR[vn] * (vR[vn] - SR[i]);
      double wL = vL[RHO] * (vL[vn] - SL[i]);
      double wR = vR[RHO] * (vR[vn] - SR[i]);
      double vs = (qR - qL) / (wR - wL);
      double us[NFLX];
      if (vs >= 0.0) {
        us[RHO] = uL[RHO] * (SL[i] - vxl) / (SL[i] - vs);
        for (nv = VX1; nv <= VX3; nv++)
          us[nv] = (nv == vn) ? us[RHO] * vs : us[RHO] * vL[nv];
        us[PRS] = uL[PRS] / vL[RHO]
                + (vs - vxl) * (vs + vL[PRS] / (vL[RHO] * (SL[i] - vxl)));
        us[PRS] *= us[RHO];
        for (nv = 0; nv < NFLX; nv++) f[nv] = FL[nv] + SL[i] * (us[nv] - uL[nv]);
        pr[i] = pL[i];
      } else {
        us[RHO] = uR[RHO] * (SR[i] - vxr) / (SR[i] - vs);
        for (nv = VX1; nv <= VX3; nv++)
          us[nv] = (nv == vn) ? us[RHO] * vs : us[RHO] * vR[nv];
        us[PRS] = uR[PRS] / vR[RHO]
                + (vs - vxr) * (vs + vR[PRS] / (vR[RHO] * (SR[i] - vxr)));
        us[PRS] *= us[RHO];
        for (nv = 0; nv < NFLX; nv++) f[nv] = FR[nv] + SR[i] * (us[nv] - uR[nv]);
        pr[i] = pR[i];
      }
    }
    /* passive scalars: upwind on the density flux (adv_flux.c:47) */
    if (nvar > NFLX) {
      const double *ts = f[RHO] > 0.0 ? vL : vR;
      for (nv = NFLX; nv < nvar; nv++) f[nv] = f[RHO] * ts[nv];
    }
  }

  /* right-hand side (rhs.c:188-209, Cartesian) and update */
  for (i = nbeg; i <= nend; i++) {
    double scrh = dt / s->dx[d][i];
    for (nv = 0; nv < nvar; nv++)
      R(rhs, i, nv) = -scrh * (R(fl, i, nv) - R(fl, i - 1, nv));
    R(rhs, i, vn) -= scrh * (pr[i] - pr[i - 1]);
  }
  for (i = nbeg; i <= nend; i++) {
    size_t c = base + i * stride;
    for (nv = 0; nv < nvar; nv++) s->U[c * nvar + nv] += R(rhs, i, nv);
  }

  /* inverse time step (update_stage.c:303-324) */
  if (stage == 1) {
    if (s->c.dims > 1) {
      for (i = nbeg; i <= nend; i++) {
        size_t c = base + i * stride;
        s->Cdt[c] += 0.5 * (cmax[i - 1] + cmax[i]) * s->inv_dx[d][i] * 1.0;
      }
    } else {
      for (i = nbeg - 1; i <= nend; i++)
        s->invDt_hyp = MAXD(s->invDt_hyp, cmax[i] * s->inv_dx[d][i]);
    }
  }
}

static void update_stage(or_sim *s, int stage, double dt)
{
  int d, i, j, k;
  size_t nc = (size_t)s->ntot[0] * s->ntot[1] * s->ntot[2];
  if (stage == 1) memset(s->Cdt, 0, nc * sizeof(double));
  for (d = 0; d < s->c.dims; d++) {
    int lo[3], hi[3];
    for (int q = 0; q < 3; q++) { lo[q] = s->beg[q]; hi[q] = s->end[q]; }
    lo[d] = hi[d] = 0;
    for (k = lo[2]; k <= hi[2]; k++)
    for (j = lo[1]; j <= hi[1]; j++)
    for (i = lo[0]; i <= hi[0]; i++)
      row_sweep(s, d, k, j, i, stage, dt);
  }
  if (stage == 1 && s->c.dims > 1) {
    for (k = s->beg[2]; k <= s->end[2]; k++)
    for (j = s->beg[1]; j <= s->end[1]; j++)
    for (i = s->beg[0]; i <= s->end[0]; i++)
      s->invDt_hyp = MAXD(s->invDt_hyp, s->Cdt[cidx(s, k, j, i)]);
    s->invDt_hyp /= (double)(s->c.dims);
  }
}

static void prim_to_cons_dom(or_sim *s)
{
  int i, j, k, nv, nvar = s->c.nvar;
  size_t nc = (size_t)s->ntot[0] * s->ntot[1] * s->ntot[2];
  double gmm1 = s->c.gamma - 1.0, v[NVMAX];
  for (k = s->beg[2]; k <= s->end[2]; k++)
  for (j = s->beg[1]; j <= s->end[1]; j++)
  for (i = s->beg[0]; i <= s->end[0]; i++) {
    size_t c = cidx(s, k, j, i);
    for (nv = 0; nv < nvar; nv++) v[nv] = s->V[nv * nc + c];
    prim_to_cons(v, &s->U[c * nvar], nvar, gmm1);
  }
}

static int cons_to_prim_dom(or_sim *s)
{
  int i, j, k, nv, nvar = s->c.nvar, flags = 0;
  size_t nc = (size_t)s->ntot[0] * s->ntot[1] * s->ntot[2];
  double gmm1 = s->c.gamma - 1.0, v[NVMAX];
  for (k = s->beg[2]; k <= s->end[2]; k++)
  for (j = s->beg[1]; j <= s->end[1]; j++)
  for (i = s->beg[0]; i <= s->end[0]; i++) {
    size_t c = cidx(s, k, j, i);
    flags |= cons_to_prim(&s->U[c * nvar], v, nvar, gmm1);
    for (nv = 0; nv < nvar; nv++) s->V[nv * nc + c] = v[nv];
  }
  return flags;
}

/* RK2 AdvanceStep (rk_step.c:29-384) */
static int advance_step(or_sim *s)
{
  int i, j, k, nv, nvar = s->c.nvar, flags;
  boundary(s);
  prim_to_cons_dom(s);
  for (k = s->beg[2]; k <= s->end[2]; k++)
  for (j = s->beg[1]; j <= s->end[1]; j++)
  for (i = s->beg[0]; i <= s->end[0]; i++) {
    size_t c = cidx(s, k, j, i);
    for (nv = 0; nv < nvar; nv++) s->U0[c * nvar + nv] = s->U[c * nvar + nv];
  }
  update_stage(s, 1, s->g_dt);
  flags = cons_to_prim_dom(s);
  boundary(s);
  update_stage(s, 2, s->g_dt);
  for (k = s->beg[2]; k <= s->end[2]; k++)
  for (j = s->beg[1]; j <= s->end[1]; j++)
  for (i = s->beg[0]; i <= s->end[0]; i++) {
    size_t c = cidx(s, k, j, i);
    for (nv = 0; nv < nvar; nv++)
      s->U[c * nvar + nv] = 0.5 * s->U0[c * nvar + nv] + 0.5 * s->U[c * nvar + nv];
  }
  flags |= cons_to_prim_dom(s);
  return flags;
}

/* NextTimeStep (main.c:521-697) for the hyperbolic-only / BLONDIN case */
static int next_time_step(or_sim *s, double *dtnext_out)
{
  double dt_hyp = 1.0 / s->invDt_hyp, dtnext;
  dt_hyp *= s->c.cfl;
  dtnext = dt_hyp;
  if (s->c.cooling) dtnext = MIND(dtnext, s->dt_cool);
  dtnext = MIND(dtnext, s->c.cfl_max_var * s->g_dt);
  if (dtnext < s->c.first_dt * 1.e-9) return 1;
  if (s->c.cfl_max_var == 1.0) dtnext = s->g_dt;
  *dtnext_out = dtnext;
  return 0;
}

int or_run(or_sim *s, int nsteps)
{
  int n;
  if (s->hist_cap < nsteps) {
    free(s->hist_dt); free(s->hist_inv);
    s->hist_dt = calloc(nsteps, sizeof(double));
    s->hist_inv = calloc(nsteps, sizeof(double));
    s->hist_cap = nsteps;
  }
  s->nhist = 0;
  for (n = 0; n < nsteps; n++) {
    int last = 0, flags;
    if ((s->g_time + s->g_dt) >= s->c.tstop * (1.0 - 1.e-8)) {
      s->g_dt = s->c.tstop - s->g_time;
      last = 1;
    }
    /* Integrate (main.c:383-497) */
    if (!s->c.cooling || (s->step - 1) % 2 == 1) {
      s->invDt_hyp = 0.0;
      s->dt_cool = 1.e38;
    }
    flags = advance_step(s);
    if (flags & 64) s->fail |= flags;
    s->hist_dt[s->nhist] = s->g_dt;
    s->hist_inv[s->nhist] = s->invDt_hyp;
    s->nhist++;
    s->g_time += s->g_dt;
    if (!s->c.cooling || s->step % 2 == 1) {
      double dtn;
      if (next_time_step(s, &dtn)) return 1;
      s->g_dt = dtn;
    }
    s->step++;
    if (last) break;
  }
  return (s->fail & 64) ? 2 : 0;
}
