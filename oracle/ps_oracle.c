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
 *   spherical geom. Src/set_geometry.c:62-250, Src/States/plm_coeffs.c:30-74
 *   curvilinear RHS Src/MHD/rhs.c:234-351, 423-630, Src/MHD/rhs_source.c:101-420
 *   line force      Src/LineDriven/line_connect.c:267-320 (xi init),
 *                   504-777 (VGradCalc, bilinear), 815-903 (LineForce)
 *   cooling         Src/Cooling/BLONDIN/cooling.c:50-319
 *   split source    Src/split_source.c:28-79, Strang order Src/main.c:479-485
 * The wind problem (Init, UserDefBoundary, BodyForceVector) follows the
 * problem file oracle/ref_cfg/wind2d/init.c used for the reference build.
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
#define OR_FLAG_MINMOD 1   /* FLAG_MINMOD (Src/pluto.h:212) */
#define OR_FLAG_HLL    4   /* FLAG_HLL (Src/pluto.h:214) */
#define OR_FLAG_ENTROPY 8  /* FLAG_ENTROPY (Src/pluto.h:215) */
#define ABS_MIN(a, b) (fabs(a) < fabs(b) ? (a) : (b))

static const double small_density = 1.e-12;
static const double small_pressure = 1.e-12;

/* physical constants of Src/pluto.h:296-321 */
#define C_AMU    1.66053886e-24
#define C_C      2.99792458e10
#define C_G      6.6726e-8
#define C_KB     1.3806505e-16
#define C_MP     1.67262171e-24
#define C_PI     3.14159265358979
#define C_RGAS   8.3144598e7
#define C_SIGMAT 6.6524e-25

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
  /* curvilinear geometry and PLM weights (set_geometry.c, plm_coeffs.c) */
  double *xgc[3], *rt, *sp, *sn, *dmu, *dVr;
  double *pcp[3], *pcm[3], *pwp[3], *pwm[3], *pdp[3], *pdm[3];
  double *dV;            /* [k][j][i]                      */
  double *Ax1, *Ax2;     /* [k][j][i+1], [k][j+1][i] faces */
  double *rvc;           /* row workspace: face-averaged / centred state */
  /* line-driven wind */
  int na;
  double *Fr, *Ft, *Fp;            /* [a][k][j][i] */
  int nm;                          /* tabulated force multiplier: points */
  double *t_fit, *m_fit;           /* log10 t [nm]; log10 M [nm][k][j][i] */
  double *xi_s, *tr_s;             /* sirocco_xi, sirocco_t_r */
  double *pre;                     /* 6 prefactor arrays (file order) or NULL: all 1 */
  unsigned char *flag;             /* FLAG_MINMOD bits of FlagShock, [k][j][i] */
  double *dvds, *roff, *toff, *moff; /* [a][k][j][i] */
  double *x11[2], *x22[2];
  int dvds_ready;
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

/* Geometry factors (Src/set_geometry.c:62-240) and PLM weights
 * (Src/States/plm_coeffs.c:30-74, non-HIGH_ORDER branch). */
static void build_geometry(or_sim *s)
{
  int i, j, k, d;
  int n0 = s->ntot[0], n1 = s->ntot[1], n2 = s->ntot[2];
  const int sph = s->c.geometry == OR_SPHERICAL;
  double *x1 = s->x[0], *dx1 = s->dx[0], *x1p = s->xr[0], *x1m = s->xl[0];
  double *x2 = s->x[1], *x2p = s->xr[1], *x2m = s->xl[1];
  for (d = 0; d < 3; d++) s->xgc[d] = calloc(s->ntot[d], sizeof(double));
  s->rt = calloc(n0, sizeof(double));
  s->dVr = calloc(n0, sizeof(double));
  s->sp = calloc(n1, sizeof(double));
  s->sn = calloc(n1, sizeof(double));
  s->dmu = calloc(n1, sizeof(double));
  for (i = 0; i < n0; i++) {
    double xL = x1m[i], xR = x1p[i];
    if (sph) {
      s->xgc[0][i] = x1[i] + 2.0 * x1[i] * dx1[i] * dx1[i] /
                                (12.0 * x1[i] * x1[i] + dx1[i] * dx1[i]);
      s->rt[i] = (xR * xR * xR - xL * xL * xL) / (xR * xR - xL * xL) / 1.5;
    } else {
      s->xgc[0][i] = x1[i];
      s->rt[i] = x1[i];
    }
    s->dVr[i] = fabs(x1p[i] * x1p[i] * x1p[i] - x1m[i] * x1m[i] * x1m[i]) / 3.0;
  }
  for (j = 0; j < n1; j++) {
    double xL = x2m[j], xR = x2p[j];
    if (sph) {
      s->xgc[1][j] = sin(xR) - sin(xL) + xL * cos(xL) - xR * cos(xR);
      s->xgc[1][j] /= cos(xL) - cos(xR);
      s->sp[j] = fabs(sin(xR));
      s->sn[j] = fabs(sin(x2[j]));
      s->dmu[j] = fabs(cos(xL) - cos(xR));
    } else {
      s->xgc[1][j] = x2[j];
    }
  }
  for (k = 0; k < n2; k++) s->xgc[2][k] = s->x[2][k];
  if (sph) {
    /* 2-D spherical: dV = dVr*dmu, A1 = rp^2*dmu, A2 = |r|*dr*|sin(th_p)| */
    s->dV = calloc((size_t)n2 * n1 * n0, sizeof(double));
    s->Ax1 = calloc((size_t)n2 * n1 * (n0 + 1), sizeof(double));
    s->Ax2 = calloc((size_t)n2 * (n1 + 1) * n0, sizeof(double));
    for (k = 0; k < n2; k++)
    for (j = 0; j < n1; j++) {
      double dmu = fabs(cos(x2m[j]) - cos(x2p[j]));
      for (i = 0; i < n0; i++) {
        double dVr = fabs(x1p[i] * x1p[i] * x1p[i] - x1m[i] * x1m[i] * x1m[i]) / 3.0;
        s->dV[((size_t)k * n1 + j) * n0 + i] = dVr * dmu;
      }
      for (i = -1; i < n0; i++) {
        double a = (i == -1) ? x1m[0] * x1m[0] * dmu : x1p[i] * x1p[i] * dmu;
        s->Ax1[((size_t)k * n1 + j) * (n0 + 1) + (i + 1)] = a;
      }
    }
    for (k = 0; k < n2; k++)
    for (j = -1; j < n1; j++)
    for (i = 0; i < n0; i++) {
      double a = (j == -1) ? fabs(x1[i]) * dx1[i] * fabs(sin(x2m[0]))
                           : fabs(x1[i]) * dx1[i] * fabs(sin(x2p[j]));
      s->Ax2[((size_t)k * (n1 + 1) + (j + 1)) * n0 + i] = a;
    }
  }
  for (d = 0; d < 3; d++) {
    int nt = s->ntot[d];
    double *dx = s->dx[d], *xgc = s->xgc[d], *xr = s->xr[d];
    s->pcp[d] = calloc(nt, sizeof(double));
    s->pcm[d] = calloc(nt, sizeof(double));
    s->pwp[d] = calloc(nt, sizeof(double));
    s->pwm[d] = calloc(nt, sizeof(double));
    s->pdp[d] = calloc(nt, sizeof(double));
    s->pdm[d] = calloc(nt, sizeof(double));
    for (i = 1; i <= nt - 2; i++) {
      s->pwp[d][i] = dx[i] / (xgc[i + 1] - xgc[i]);
      s->pwm[d][i] = dx[i] / (xgc[i] - xgc[i - 1]);
      s->pcp[d][i] = (xgc[i + 1] - xgc[i]) / (xr[i] - xgc[i]);
      s->pcm[d][i] = (xgc[i] - xgc[i - 1]) / (xgc[i] - xr[i - 1]);
      s->pdp[d][i] = (xr[i] - xgc[i]) / dx[i];
      s->pdm[d][i] = (xgc[i] - xr[i - 1]) / dx[i];
    }
  }
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
    /* GetNghost (Src/get_nghost.c:15-60): 2 for PLM, 3 with MULTID */
    s->ngh[d] = (d < cfg->dims) ? (cfg->shock_flattening ? 3 : 2) : 0;
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
  s->rvc = calloc((size_t)(nmax + 2) * NVMAX, sizeof(double));
  build_geometry(s);
  s->flag = calloc(ncell, 1);
  s->xi_s = calloc(ncell, sizeof(double));
  s->tr_s = calloc(ncell, sizeof(double));
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
    free(s->inv_dx[d]); free(s->xgc[d]);
    free(s->pcp[d]); free(s->pcm[d]); free(s->pwp[d]); free(s->pwm[d]);
    free(s->pdp[d]); free(s->pdm[d]);
  }
  free(s->rt); free(s->sp); free(s->sn); free(s->dmu); free(s->dVr);
  free(s->dV); free(s->Ax1); free(s->Ax2); free(s->rvc);
  free(s->Fr); free(s->Ft); free(s->Fp); free(s->xi_s); free(s->tr_s); free(s->pre);
  free(s->flag);
  free(s->t_fit); free(s->m_fit);
  free(s->dvds); free(s->roff); free(s->toff); free(s->moff);
  free(s->x11[0]); free(s->x11[1]); free(s->x22[0]); free(s->x22[1]);
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
    case 4: return s->xgc[dir];
    default: return s->dx[dir];
  }
}

const double *or_sirocco_xi(const or_sim *s) { return s->xi_s; }

/* read_sirocco_heatcool with flag 1 (line_connect.c:267-497) as data:
 * sirocco_xi, sirocco_t_r and the prefactor arrays (file order comp_h,
 * comp_c, xray_h, brem_c, line_c, xi_ion), each over the total box; NULL
 * keeps that part. */
void or_set_sirocco(or_sim *s, const double *xi, const double *t_r, const double *pre)
{
  size_t nc = (size_t)s->ntot[0] * s->ntot[1] * s->ntot[2];
  if (xi) memcpy(s->xi_s, xi, nc * sizeof(double));
  if (t_r) memcpy(s->tr_s, t_r, nc * sizeof(double));
  if (pre) {
    if (!s->pre) s->pre = malloc(6 * nc * sizeof(double));
    memcpy(s->pre, pre, 6 * nc * sizeof(double));
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

/* prim_to_cons is defined below; the floors need it */
static inline void prim_to_cons(const double *v, double *u, int nvar, double gmm1);

#define UNIT_P(s) ((s)->c.unit_density * (s)->c.unit_velocity * (s)->c.unit_velocity)
#define UNIT_T(s) ((s)->c.unit_length / (s)->c.unit_velocity)
#define UNIT_A(s) ((s)->c.unit_velocity * (s)->c.unit_velocity / (s)->c.unit_length)
#define KELVIN_OF(s) ((s)->c.unit_velocity * (s)->c.unit_velocity * C_AMU / C_KB)

/* Init() of the wind problem at one point (oracle/ref_cfg/wind2d/init.c) */
static void wind_init_point(const or_sim *s, double *v, double x1, double x2)
{
  double gm_cgs = C_G * s->c.cent_mass;
  double mu = s->c.mu, T = s->c.t_iso;
  double r = x1 * s->c.unit_length;
  double cs2 = C_RGAS * T / mu;
  double tt = tan(x2);
  double rho_d = s->c.rho_0 * exp(-gm_cgs / (2.0 * cs2 * r * tt * tt)) / s->c.unit_density;
  double rho_a = s->c.dfloor / s->c.unit_density;
  v[VX1] = 0.0;
  v[VX2] = 0.0;
  if (rho_d > rho_a) {
    v[RHO] = rho_d;
    v[NFLX] = 1.0;
  } else {
    v[RHO] = rho_a;
    v[NFLX] = 0.0;
  }
  v[VX3] = sqrt(gm_cgs / r) * sin(x2) / s->c.unit_velocity;
  v[PRS] = v[RHO] * T / (KELVIN_OF(s) * mu);
}

static void compute_entropy(or_sim *s);

void or_init_wind(or_sim *s)
{
  int i, j, k, nv;
  size_t nc = (size_t)s->ntot[0] * s->ntot[1] * s->ntot[2];
  double v[NVMAX];
  /* Startup(): Init() on every cell of the total box at the centroids */
  for (k = 0; k < s->ntot[2]; k++)
  for (j = 0; j < s->ntot[1]; j++)
  for (i = 0; i < s->ntot[0]; i++) {
    for (nv = 0; nv < NVMAX; nv++) v[nv] = 0.0;
    wind_init_point(s, v, s->xgc[0][i], s->xgc[1][j]);
    for (nv = 0; nv < s->c.nvar; nv++) s->V[nv * nc + cidx(s, k, j, i)] = v[nv];
  }
  or_wind_reset(s);
}

/* The start of a wind run from the state in s->V (set by or_init_wind, or
 * by the caller, e.g. the reference's own initial snapshot of a problem
 * whose Init this oracle does not restate): read_sirocco_heatcool(flag = 0)
 * and Startup's ComputeEntropy. */
void or_wind_reset(or_sim *s)
{
  int i, j, k;
  size_t nc = (size_t)s->ntot[0] * s->ntot[1] * s->ntot[2];
  /* read_sirocco_heatcool(flag = 0): frozen xi and radiation temperature */
  for (k = s->beg[2]; k <= s->end[2]; k++)
  for (j = s->beg[1]; j <= s->end[1]; j++)
  for (i = s->beg[0]; i <= s->end[0]; i++) {
    size_t c = cidx(s, k, j, i);
    double rho = s->V[RHO * nc + c] * s->c.unit_density;
    double r = s->x[0][i] * s->c.unit_length;
    double nH = rho / (1.43 * C_MP);
    double lx = s->c.l_star * s->c.f_x;
    s->xi_s[c] = lx / nH / (r * r);
    s->tr_s[c] = s->c.t_x;
  }
  s->dvds_ready = 0;
  if (s->c.entropy_switch) compute_entropy(s);   /* Startup's Boundary */
}

void or_set_mfit(or_sim *s, int npoints, const double *t_fit, const double *m_fit)
{
  size_t i, nc = (size_t)s->ntot[0] * s->ntot[1] * s->ntot[2];
  free(s->t_fit); free(s->m_fit);
  s->nm = npoints;
  s->t_fit = malloc((size_t)npoints * sizeof(double));
  s->m_fit = malloc((size_t)npoints * nc * sizeof(double));
  /* the reader keeps log10 of what the file holds (line_connect.c:211, 228) */
  for (i = 0; i < (size_t)npoints; i++) s->t_fit[i] = log10(t_fit[i]);
  for (i = 0; i < (size_t)npoints * nc; i++) s->m_fit[i] = log10(m_fit[i]);
}

void or_set_flux(or_sim *s, int nangles, const double *fr, const double *ft, const double *fp)
{
  size_t nc = (size_t)s->ntot[0] * s->ntot[1] * s->ntot[2];
  size_t n = nc * (size_t)nangles;
  free(s->Fr); free(s->Ft); free(s->Fp);
  free(s->dvds); free(s->roff); free(s->toff); free(s->moff);
  s->na = nangles;
  s->Fr = malloc(n * sizeof(double));
  s->Ft = malloc(n * sizeof(double));
  s->Fp = malloc(n * sizeof(double));
  memcpy(s->Fr, fr, n * sizeof(double));
  memcpy(s->Ft, ft, n * sizeof(double));
  memcpy(s->Fp, fp, n * sizeof(double));
  s->dvds = calloc(n, sizeof(double));
  s->roff = calloc(n, sizeof(double));
  s->toff = calloc(n, sizeof(double));
  s->moff = calloc(n, sizeof(double));
  s->dvds_ready = 0;
}

/* UserDefBoundary(side == 0) of the wind problem: density and pressure
 * floors on every cell, with the conservative state of a repaired cell
 * rebuilt (PrimToCons3D on that cell). */
static void wind_floors(or_sim *s)
{
  int i, j, k, nv, nvar = s->c.nvar;
  size_t nc = (size_t)s->ntot[0] * s->ntot[1] * s->ntot[2];
  double mu = s->c.mu, K = KELVIN_OF(s);
  double dfloor = s->c.dfloor / s->c.unit_density;
  double tfloor = 5.e2;
  double pfloor = dfloor * tfloor / (K * mu);
  double gmm1 = s->c.gamma - 1.0, v[NVMAX];
  for (k = 0; k < s->ntot[2]; k++)
  for (j = 0; j < s->ntot[1]; j++)
  for (i = 0; i < s->ntot[0]; i++) {
    size_t c = cidx(s, k, j, i);
    double *V = s->V;
    int convert = 0;
    if (V[RHO * nc + c] < dfloor) {
      double cs, dfact, temp;
      if (V[RHO * nc + c] < 0.0) V[RHO * nc + c] = dfloor;
      cs = sqrt(s->c.gamma * V[PRS * nc + c] / V[RHO * nc + c]);
      dfact = V[RHO * nc + c] / dfloor;
      V[RHO * nc + c] = dfloor;
      V[VX1 * nc + c] = dfact * V[VX1 * nc + c];
      V[VX2 * nc + c] = dfact * V[VX2 * nc + c];
      V[VX3 * nc + c] = dfact * V[VX3 * nc + c];
      V[PRS * nc + c] = cs * cs * V[RHO * nc + c] / s->c.gamma;
      temp = V[PRS * nc + c] / V[RHO * nc + c] * K * mu;
      if (temp < tfloor) V[PRS * nc + c] = V[RHO * nc + c] * tfloor / (K * mu);
      V[NFLX * nc + c] = 0.0;
      convert = 1;
    }
    if (V[PRS * nc + c] < pfloor) {
      V[PRS * nc + c] = pfloor;
      convert = 1;
    }
    if (convert) {
      for (nv = 0; nv < nvar; nv++) v[nv] = V[nv * nc + c];
      prim_to_cons(v, &s->U[c * nvar], nvar, gmm1);
    }
  }
}

/* ComputeEntropy (Src/entropy_switch.c:14-37 with Entropy, Src/EOS/Ideal/
 * eos.c:77-103): s = p / rho^gamma over the total box, into the last
 * variable. */
static void compute_entropy(or_sim *s)
{
  size_t c, nc = (size_t)s->ntot[0] * s->ntot[1] * s->ntot[2];
  double *S = s->V + (size_t)(s->c.nvar - 1) * nc;
  for (c = 0; c < nc; c++) S[c] = s->V[PRS * nc + c] / pow(s->V[RHO * nc + c], s->c.gamma);
}

static void boundary(or_sim *s)
{
  int side, nv, i, j, k;
  int nvar = s->c.nvar;
  if (s->c.floors) wind_floors(s);
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
      } else if (type == OR_BC_USERDEF && side == 0) {
        /* wind problem, X1_BEG: copy the first active cell, inflow only */
        src[0] = s->beg[0];
        val = s->V[vidx(s, nv, src[2], src[1], src[0])];
        if (nv == VX1) val = MIND(val, 0.0);
        s->V[vidx(s, nv, k, j, i)] = val;
        continue;
      } else if (type == OR_BC_USERDEF && side == 1) {
        /* production wind, X1_END: copy the last active cell, outflow only
         * (Test_Problems/LineDrivenWind/cv_idl/init.c:331-340) */
        src[0] = s->end[0];
        val = s->V[vidx(s, nv, src[2], src[1], src[0])];
        if (nv == VX1) val = MAXD(val, 0.0);
        s->V[vidx(s, nv, k, j, i)] = val;
        continue;
      } else if (type == OR_BC_USERDEF && side == 2) {
        /* production wind, X2_BEG: every variable from the mirrored active
         * row, v_theta times -1, then density and pressure from the first
         * active row (cv_idl/init.c:343-356) */
        src[1] = (nv == RHO || nv == PRS) ? s->beg[1] : 2 * s->beg[1] - 1 - j;
        val = s->V[vidx(s, nv, src[2], src[1], src[0])];
        if (nv == VX2) val *= -1.0;
        s->V[vidx(s, nv, k, j, i)] = val;
        continue;
      } else {
        continue;
      }
      val = s->V[vidx(s, nv, src[2], src[1], src[0])];
      if (type == OR_BC_OUTFLOW || type == OR_BC_PERIODIC)
        s->V[vidx(s, nv, k, j, i)] = val;
      else
        s->V[vidx(s, nv, k, j, i)] = vsign[nv] * val;
    }
  }
  if (s->c.entropy_switch) compute_entropy(s);   /* boundary.c:487-493 */
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

/* returns nonzero flag bits on failure (64 = cons2prim fail).  entr: index
 * of the entropy variable (ENTROPY_SWITCH) or -1; use_entropy: the zone is
 * tagged FLAG_ENTROPY, p = (rho s) rho^(gamma-1) (mappers.c:185-221). */
static inline int cons_to_prim(double *u, double *v, int nvar, double gmm1, int entr,
                               int use_entropy)
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
  if (use_entropy) {
    double rhog1 = pow(rho, gmm1);
    v[PRS] = u[entr] * rhog1;
    if (v[PRS] < 0.0) {
      v[PRS] = small_pressure;
      flag |= 64;
    }
    u[PRS] = v[PRS] / gmm1 + kin;   /* redefine energy */
  } else {
    v[PRS] = gmm1 * (u[PRS] - kin);
    if (v[PRS] < 0.0) {
      v[PRS] = small_pressure;
      u[PRS] = v[PRS] / gmm1 + kin;
      flag |= 64;
    }
    if (entr >= 0) u[entr] = v[PRS] / pow(rho, gmm1);
  }
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

/* Limiters on irregular or curvilinear grids (Src/States/plm_coeffs.h:128-150) */
static inline double limit_general(int lim, double dvp, double dvm, double cp, double cm)
{
  double dv;
  if (lim == OR_LIM_MC) {
    if (dvp * dvm > 0.0) {
      double qc = 0.5 * ((dvm) + (dvp)), scrh = ABS_MIN((dvp) * cp, (dvm) * cm);
      dv = ABS_MIN(qc, scrh);
    } else dv = 0.0;
  } else if (lim == OR_LIM_VL) {
    dv = (dvp * dvm > 0.0 ? (dvp) * (dvm) * (cp * (dvm) + cm * (dvp)) /
                                ((dvp) * (dvp) + (dvm) * (dvm) + (cp + cm - 2.0) * (dvp) * (dvm))
                          : 0.0);
  } else {
    dv = (dvp * dvm > 0.0 ? ABS_MIN(dvp, dvm) : 0.0);
  }
  return dv;
}

/* PLM on characteristic variables for one cell (plm_states.c:481-746, the
 * CHAR_LIMITING == YES States(), HD with an energy equation): primitive
 * eigenvectors (HD/eigenv.c:92-240, PrimEigenvectors), projection of the
 * one-sided differences (eigenv.c:575-617, PrimToChar), limiting of each
 * characteristic difference, back-projection, the monotonicity bound in
 * primitive variables, and the passive scalars limited as primitives.
 * dR = v[i+1]-v[i], dL = v[i]-v[i-1]; general grid weights or the uniform
 * Cartesian ones (cp = cm = 2, wp = wm = 1, dp = dm = 1/2). */
static void char_states(int nvar, int d, int lim, int general, double gam, const double *v,
                        const double *dR, const double *dL, double cp, double cm, double wp,
                        double wm, double dp, double dm, int minmod, double *vp, double *vm)
{
  const int nflx = 5, vn = VX1 + d;
  const int vt = d == 0 ? VX2 : (d == 1 ? VX3 : VX1);
  const int vb = d == 0 ? VX3 : (d == 1 ? VX1 : VX2);
  double L[5][8], Rm[8][5], dvp[8], dvm[8], dwp[8], dwm[8], dwl[8], dvl[8];
  int k, nv;
  double cs2, cs, rhocs, rho_cs;
  memset(L, 0, sizeof(L));
  memset(Rm, 0, sizeof(Rm));
  cs2 = gam * v[PRS] / v[RHO];             /* SoundSpeed2, IDEAL (eos.c:16-42) */
  cs = sqrt(cs2);
  rhocs = v[RHO] * cs;
  rho_cs = v[RHO] / cs;
  Rm[RHO][0] = 0.5 * rho_cs;  Rm[vn][0] = -0.5;  Rm[PRS][0] = 0.5 * rhocs;
  Rm[RHO][1] = 0.5 * rho_cs;  Rm[vn][1] = 0.5;   Rm[PRS][1] = 0.5 * rhocs;
  Rm[RHO][2] = 1.0;  Rm[vt][3] = 1.0;  Rm[vb][4] = 1.0;
  L[0][vn] = -1.0;  L[0][PRS] = 1.0 / rhocs;
  L[1][vn] = 1.0;   L[1][PRS] = 1.0 / rhocs;
  L[2][RHO] = 1.0;  L[3][vt] = 1.0;  L[4][vb] = 1.0;
  L[2][PRS] = -1.0 / cs2;
  for (nv = 0; nv < nvar; nv++) {
    dvp[nv] = general ? dR[nv] * wp : dR[nv];
    dvm[nv] = general ? dL[nv] * wm : dL[nv];
  }
  /* PrimToChar */
  dwm[0] = L[0][vn] * dvm[vn] + L[0][PRS] * dvm[PRS];
  dwm[1] = L[1][vn] * dvm[vn] + L[1][PRS] * dvm[PRS];
  dwm[2] = dvm[RHO] + L[2][PRS] * dvm[PRS];
  dwm[3] = dvm[vt];
  dwm[4] = dvm[vb];
  dwp[0] = L[0][vn] * dvp[vn] + L[0][PRS] * dvp[PRS];
  dwp[1] = L[1][vn] * dvp[vn] + L[1][PRS] * dvp[PRS];
  dwp[2] = dvp[RHO] + L[2][PRS] * dvp[PRS];
  dwp[3] = dvp[vt];
  dwp[4] = dvp[vb];
  for (k = nflx; k--;) {
    if (minmod)   /* SHOCK_FLATTENING MULTID, FLAG_MINMOD (plm_states.c:617-620) */
      dwl[k] = (dwp[k] * dwm[k] > 0.0 ? ABS_MIN(dwp[k], dwm[k]) : 0.0);
    else
      dwl[k] = general ? limit_general(lim, dwp[k], dwm[k], cp, cm) : limit(lim, dwp[k], dwm[k]);
  }
  for (nv = nflx; nv--;) {
    double dc = 0.0;
    for (k = 0; k < nflx; k++) dc += dwl[k] * Rm[nv][k];
    if (dvp[nv] * dvm[nv] > 0.0) {
      double d2v = ABS_MIN(cp * dvp[nv], cm * dvm[nv]);
      dvl[nv] = (d2v * dc > 0.0 ? (fabs(d2v) < fabs(dc) ? d2v : dc) : 0.0);
    } else dvl[nv] = 0.0;
  }
  for (nv = nflx; nv < nvar; nv++)
    dvl[nv] = general ? limit_general(lim, dvp[nv], dvm[nv], cp, cm) : limit(lim, dvp[nv], dvm[nv]);
  for (nv = nvar; nv--;) {
    vp[nv] = v[nv] + dvl[nv] * dp;
    vm[nv] = v[nv] - dvl[nv] * dm;
  }
}

/* ------------------------------------------------------------------ */
/* line force (Src/LineDriven/line_connect.c)                         */
/* ------------------------------------------------------------------ */

#define AIDX(s, a, c) ((size_t)(a) * (size_t)(s)->ntot[0] * (s)->ntot[1] * (s)->ntot[2] + (c))

static void bilinear(const double x11[2], const double x22[2], const double v11[2],
                     const double v12[2], const double v21[2], const double v22[2],
                     const double test[2], double ans[2])
{
  double fracx1 = (test[0] - x11[0]) / (x22[0] - x11[0]);
  double fracx2 = (test[1] - x11[1]) / (x22[1] - x11[1]);
  double temp1 = (1.0 - fracx1) * v11[0] + fracx1 * v21[0];
  double temp2 = (1.0 - fracx1) * v12[0] + fracx1 * v22[0];
  ans[0] = (1.0 - fracx2) * temp1 + fracx2 * temp2;
  temp1 = (1.0 - fracx1) * v11[1] + fracx1 * v21[1];
  temp2 = (1.0 - fracx1) * v12[1] + fracx1 * v22[1];
  ans[1] = (1.0 - fracx2) * temp1 + fracx2 * temp2;
}

/* VGradCalc (line_connect.c:504-742): dv/ds along every flux bin.  Returns
 * nonzero if a NaN appears (the reference exits the program there). */
static int vgrad_calc(or_sim *s)
{
  int i, j, k, a;
  size_t nc = (size_t)s->ntot[0] * s->ntot[1] * s->ntot[2];
  const double UL = s->c.unit_length, UV = s->c.unit_velocity;
  double *x1 = s->x[0], *x2 = s->x[1];
  double *V1 = s->V + VX1 * nc, *V2 = s->V + VX2 * nc;
  if (!s->dvds_ready) {
    for (a = 0; a < 2; a++) {
      free(s->x11[a]); free(s->x22[a]);
      s->x11[a] = calloc(nc, sizeof(double));
      s->x22[a] = calloc(nc, sizeof(double));
    }
    for (a = 0; a < s->na; a++) {
      for (k = s->beg[2]; k <= s->end[2]; k++)
      for (j = s->beg[1]; j <= s->end[1]; j++)
      for (i = s->beg[0]; i <= s->end[0]; i++) {
        size_t c = cidx(s, k, j, i), q = AIDX(s, a, c);
        double maxds, mod_flux;
        s->x11[0][c] = (x1[i - 1] + x1[i]) / 2.0 * UL;
        s->x11[1][c] = (x2[j - 1] + x2[j]) / 2.0;
        s->x22[0][c] = (x1[i + 1] + x1[i]) / 2.0 * UL;
        s->x22[1][c] = (x2[j + 1] + x2[j]) / 2.0;
        maxds = fabs(s->x22[0][c] - s->x11[0][c]);
        if (maxds > (x1[i] * UL * fabs(s->x22[1][c] - s->x11[1][c])))
          maxds = x1[i] * UL * fabs(s->x22[1][c] - s->x11[1][c]);
        maxds /= 2.0;
        mod_flux = sqrt(pow(s->Fr[q], 2) + pow(s->Ft[q], 2) + pow(s->Fp[q], 2));
        if (mod_flux == 0.0) {
          s->moff[q] = -999;
        } else {
          double x = x1[i] * sin(x2[j]) * UL;
          double z = x1[i] * cos(x2[j]) * UL;
          double th = (a + 0.5) * (2.0 * C_PI) / 36.0;
          double dx1 = maxds * sin(th), dx2 = maxds * cos(th);
          double ds = sqrt(dx1 * dx1 + dx2 * dx2);
          s->roff[q] = sqrt((x + dx1) * (x + dx1) + (z + dx2) * (z + dx2));
          s->toff[q] = atan((x + dx1) / (z + dx2));
          s->moff[q] = ds;
        }
      }
    }
    s->dvds_ready = 1;
  }
  for (a = 0; a < s->na; a++) {
    for (k = s->beg[2]; k <= s->end[2]; k++)
    for (j = s->beg[1]; j <= s->end[1]; j++)
    for (i = s->beg[0]; i <= s->end[0]; i++) {
      size_t c = cidx(s, k, j, i), q = AIDX(s, a, c);
      size_t cjm = cidx(s, k, j - 1, i), cjp = cidx(s, k, j + 1, i);
      double v11[2], v12[2], v21[2], v22[2], x11[2], x22[2], loc[2], ans1[2], ans2[2];
      double vx1, vz1, ds;
      v11[0] = (V1[cjm - 1] + V1[cjm] + V1[c - 1] + V1[c]) / 4.0;
      v11[1] = (V2[cjm - 1] + V2[cjm] + V2[c - 1] + V2[c]) / 4.0;
      v12[0] = (V1[cjp - 1] + V1[c - 1] + V1[cjp] + V1[c]) / 4.0;
      v12[1] = (V2[cjp - 1] + V2[c - 1] + V2[cjp] + V2[c]) / 4.0;
      v22[0] = (V1[cjp] + V1[cjp + 1] + V1[c + 1] + V1[c]) / 4.0;
      v22[1] = (V2[cjp] + V2[cjp + 1] + V2[c + 1] + V2[c]) / 4.0;
      v21[0] = (V1[c + 1] + V1[cjm + 1] + V1[cjm] + V1[c]) / 4.0;
      v21[1] = (V2[c + 1] + V2[cjm + 1] + V2[cjm] + V2[c]) / 4.0;
      x11[0] = s->x11[0][c]; x11[1] = s->x11[1][c];
      x22[0] = s->x22[0][c]; x22[1] = s->x22[1][c];
      loc[0] = x1[i] * UL;
      loc[1] = x2[j];
      bilinear(x11, x22, v11, v12, v21, v22, loc, ans1);
      vx1 = (ans1[0] * UV * sin(x2[j]) + ans1[1] * UV * cos(x2[j]));
      vz1 = (ans1[0] * UV * cos(x2[j]) - ans1[1] * UV * sin(x2[j]));
      loc[0] = s->roff[q];
      loc[1] = s->toff[q];
      ds = s->moff[q];
      if (ds == -999) {
        s->dvds[q] = -999;
      } else {
        double vx2, vz2, th, v1, v2;
        bilinear(x11, x22, v11, v12, v21, v22, loc, ans2);
        vx2 = (ans2[0] * UV * sin(loc[1]) + ans2[1] * UV * cos(loc[1]));
        vz2 = (ans2[0] * UV * cos(loc[1]) - ans2[1] * UV * sin(loc[1]));
        th = (a + 0.5) * (2.0 * C_PI) / 36.0;
        v1 = sin(th) * vx1 + cos(th) * vz1;
        v2 = sin(th) * vx2 + cos(th) * vz2;
        s->dvds[q] = fabs((v2 - v1) / ds);
      }
      if (s->dvds[q] != s->dvds[q]) return 1;
    }
  }
  return 0;
}

/* linterp (line_connect.c:778-808): first index whose abscissa is not
 * below x by a linear scan, 10^ of the linear interpolant of log10 M, ends
 * clamped */
static double or_linterp(double x, const double *xa, const double *ya, size_t ystride, int n)
{
  int idx = 0;
  double result;
  while (idx < n && xa[idx] < x) idx++;
  if (idx == 0) {
    result = pow(10.0, ya[0]);
  } else if (idx >= n) {
    result = pow(10.0, ya[(size_t)(n - 1) * ystride]);
  } else {
    double x_low = xa[idx - 1], x_high = xa[idx];
    double y_low = ya[(size_t)(idx - 1) * ystride], y_high = ya[(size_t)idx * ystride];
    double slope = (y_high - y_low) / (x_high - x_low);
    result = pow(10.0, y_low + slope * (x - x_low));
  }
  if (isnan(result)) result = 0.0;
  return result;
}

/* LineForce (line_connect.c:815-903): power-law force multiplier, or the
 * cell's tabulated M(t) when KRAD and ALPHARAD are both 999 */
static void line_force(const or_sim *s, const double *v, size_t c, double *grad)
{
  const double sigma_e = C_SIGMAT / C_AMU / 1.18;
  double rho = v[RHO] * s->c.unit_density;
  double mu = s->c.mu, krad = s->c.krad, alpharad = s->c.alpharad;
  double M_max = 4400.;
  double T = v[PRS] / v[RHO] * KELVIN_OF(s) * mu;
  double v_th = sqrt((2.0 * C_KB * T) / C_MP);
  double UA = UNIT_A(s);
  int a;
  grad[0] = 0.0;
  grad[1] = 0.0;
  grad[2] = 0.0;
  for (a = 0; a < s->na; a++) {
    size_t q = AIDX(s, a, c);
    double flux_r = s->Fr[q], flux_t = s->Ft[q], M_UV;
    if (s->dvds[q] > 0.0) {
      double t_UV = sigma_e * rho * v_th / s->dvds[q];
      if (krad == 999 && alpharad == 999) {
        size_t nc = (size_t)s->ntot[0] * s->ntot[1] * s->ntot[2];
        M_UV = s->nm > 0 ? or_linterp(log10(t_UV), s->t_fit, s->m_fit + c, nc, s->nm) : 0.0;
      } else {
        M_UV = krad * pow(t_UV, alpharad);
      }
      if (M_UV > M_max) M_UV = M_max;
    } else {
      M_UV = 0.0;
    }
    grad[0] += ((1.0 + M_UV) * sigma_e * flux_r / C_C) / UA;
    grad[1] += ((1.0 + M_UV) * sigma_e * flux_t / C_C) / UA;
  }
}

/* Curvilinear right-hand side of one row: total flux times area, flux
 * difference over the volume, pressure gradient, angular-momentum form of
 * the phi momentum (rhs.c:234-351, 423-630), then the geometric, gravity
 * and line-force sources (rhs_source.c:101-420) with the face-averaged
 * state in x1 and the cell-centred state in x2. */
static void sph_rhs(or_sim *s, int d, int k0, int j0, int i0, double dt)
{
  int nvar = s->c.nvar, nbeg = s->beg[d], nend = s->end[d], i, nv;
  int n0 = s->ntot[0], n1 = s->ntot[1];
  double *fl = s->rflux, *rhs = s->rrhs, *pr = s->rpress, *vp = s->rvp, *vm = s->rvm;
  double *v = s->rv;
  double fA[2][NVMAX];
  double gm_code = C_G * s->c.cent_mass /
                   (s->c.unit_length * s->c.unit_velocity * s->c.unit_velocity);
  size_t nc = (size_t)s->ntot[0] * s->ntot[1] * s->ntot[2];
  (void)nc;
  for (i = nbeg; i <= nend; i++) {
    int ii = d == 0 ? i : i0, jj = d == 1 ? i : j0;
    size_t c = cidx(s, k0, jj, ii);
    double dtdV = dt / s->dV[c], dtdl, vc[NVMAX], grad[3], g0;
    for (int side = 0; side < 2; side++) {
      int f = i - 1 + side; /* face f+1/2 */
      double A;
      if (d == 0) A = s->Ax1[((size_t)k0 * n1 + j0) * (n0 + 1) + (f + 1)];
      else        A = s->Ax2[((size_t)k0 * (n1 + 1) + (f + 1)) * n0 + i0];
      for (nv = 0; nv < nvar; nv++) fA[side][nv] = R(fl, f, nv) * A;
      if (d == 0) fA[side][VX3] *= fabs(s->xr[0][f]);
      else        fA[side][VX3] *= fabs(s->sp[f]);
    }
    if (d == 0) dtdl = dt / s->dx[0][i];
    else        dtdl = dt / s->dx[1][i] * (1.0 / s->rt[i0]);
    for (nv = 0; nv < nvar; nv++) R(rhs, i, nv) = -dtdV * (fA[1][nv] - fA[0][nv]);
    R(rhs, i, VX1 + d) -= dtdl * (pr[i] - pr[i - 1]);
    if (d == 0) R(rhs, i, VX3) /= fabs(s->x[0][i]);
    else        R(rhs, i, VX3) /= fabs(s->sn[i]);

    if (d == 0) {
      double r_1 = 1.0 / s->x[0][i], vphi, Sm;
      for (nv = 0; nv < nvar; nv++) vc[nv] = 0.5 * (R(vp, i, nv) + R(vm, i, nv));
      vphi = vc[VX3];
      Sm = vc[RHO] * (vc[VX2] * vc[VX2] + vphi * vphi);
      R(rhs, i, VX1) += dt * Sm * r_1;
      if (s->c.body_force) {
        g0 = -1.0 * gm_code / (s->x[0][i] * s->x[0][i]);
        R(rhs, i, VX1) += dt * vc[RHO] * g0;
        R(rhs, i, PRS) += dt * 0.5 * (R(fl, i, RHO) + R(fl, i - 1, RHO)) * g0;
      }
      if (s->c.line_force) {
        line_force(s, vc, c, grad);
        R(rhs, i, VX1) += dt * vc[RHO] * grad[0];
        R(rhs, i, PRS) += dt * 0.5 * (R(fl, i, RHO) + R(fl, i - 1, RHO)) * grad[0];
      }
    } else {
      double r_1 = 1.0 / s->rt[i0], ct = 1.0 / tan(s->x[1][i]), vphi, Sm;
      for (nv = 0; nv < nvar; nv++) vc[nv] = R(v, i, nv);
      vphi = vc[VX3];
      Sm = vc[RHO] * (-vc[VX2] * vc[VX1] + ct * vphi * vphi);
      Sm += 0.0 - ct * 0.0;
      R(rhs, i, VX2) += dt * Sm * r_1;
      if (s->c.body_force) {
        double g1 = 0.0, g2 = 0.0;
        R(rhs, i, VX2) += dt * vc[RHO] * g1;
        R(rhs, i, PRS) += dt * 0.5 * (R(fl, i, RHO) + R(fl, i - 1, RHO)) * g1;
        R(rhs, i, VX3) += dt * vc[RHO] * g2;
        R(rhs, i, PRS) += dt * vc[RHO] * vc[VX3] * g2;
      }
      if (s->c.line_force) {
        line_force(s, vc, c, grad);
        R(rhs, i, VX2) += dt * vc[RHO] * grad[1];
        R(rhs, i, PRS) += dt * 0.5 * (R(fl, i, RHO) + R(fl, i - 1, RHO)) * grad[1];
        R(rhs, i, VX3) += dt * vc[RHO] * grad[2];
        R(rhs, i, PRS) += dt * vc[RHO] * vc[VX3] * grad[2];
      }
    }
  }
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
    const int minmod = s->c.shock_flattening && (s->flag[base + i * stride] & OR_FLAG_MINMOD);
    if (s->c.char_limiting) {
      const int general = s->c.geometry != OR_CARTESIAN;
      char_states(nvar, d, s->c.limiter, general, gam, &R(v, i, 0), &R(dvv, i, 0),
                  &R(dvv, i - 1, 0), general ? s->pcp[d][i] : 2.0, general ? s->pcm[d][i] : 2.0,
                  general ? s->pwp[d][i] : 1.0, general ? s->pwm[d][i] : 1.0,
                  general ? s->pdp[d][i] : 0.5, general ? s->pdm[d][i] : 0.5, minmod,
                  &R(vp, i, 0), &R(vm, i, 0));
    } else if (minmod) {   /* plm_states.c:176-193 */
      const int general = s->c.geometry != OR_CARTESIAN;
      double wp = general ? s->pwp[d][i] : 1.0, wm = general ? s->pwm[d][i] : 1.0;
      double dp = general ? s->pdp[d][i] : 0.5, dm = general ? s->pdm[d][i] : 0.5;
      for (nv = 0; nv < nvar; nv++) {
        double dvp = general ? R(dvv, i, nv) * wp : R(dvv, i, nv);
        double dvm = general ? R(dvv, i - 1, nv) * wm : R(dvv, i - 1, nv);
        double dvl = (dvp * dvm > 0.0 ? ABS_MIN(dvp, dvm) : 0.0);
        R(vp, i, nv) = R(v, i, nv) + dvl * dp;
        R(vm, i, nv) = R(v, i, nv) - dvl * dm;
      }
    } else if (s->c.geometry == OR_CARTESIAN) {
      for (nv = 0; nv < nvar; nv++) {
        double dvp = R(dvv, i, nv), dvm = R(dvv, i - 1, nv);
        double dvl = limit(s->c.limiter, dvp, dvm);
        R(vp, i, nv) = R(v, i, nv) + dvl * 0.5;
        R(vm, i, nv) = R(v, i, nv) - dvl * 0.5;
      }
    } else {
      double cp = s->pcp[d][i], cm = s->pcm[d][i], wp = s->pwp[d][i], wm = s->pwm[d][i];
      double dp = s->pdp[d][i], dm = s->pdm[d][i];
      for (nv = 0; nv < nvar; nv++) {
        double dvp = R(dvv, i, nv) * wp, dvm = R(dvv, i - 1, nv) * wm;
        double dvl = limit_general(s->c.limiter, dvp, dvm, cp, cm);
        R(vp, i, nv) = R(v, i, nv) + dvl * dp;
        R(vm, i, nv) = R(v, i, nv) - dvl * dm;
      }
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
    } else if (s->c.solver == OR_HLL ||
               (s->c.shock_flattening && ((s->flag[base + i * stride] & OR_FLAG_HLL) ||
                                          (s->flag[base + (i + 1) * stride] & OR_FLAG_HLL)))) {
      /* HLL, or HLLC's switch to HLL next to a shocked zone (hllc.c:93-104) */
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

  if (s->c.geometry == OR_CARTESIAN) {
    /* right-hand side (rhs.c:188-209, Cartesian) */
    for (i = nbeg; i <= nend; i++) {
      double scrh = dt / s->dx[d][i];
      for (nv = 0; nv < nvar; nv++)
        R(rhs, i, nv) = -scrh * (R(fl, i, nv) - R(fl, i - 1, nv));
      R(rhs, i, vn) -= scrh * (pr[i] - pr[i - 1]);
    }
  } else {
    sph_rhs(s, d, k0, j0, i0, dt);
  }
  for (i = nbeg; i <= nend; i++) {
    size_t c = base + i * stride;
    for (nv = 0; nv < nvar; nv++) s->U[c * nvar + nv] += R(rhs, i, nv);
  }

  /* inverse time step (update_stage.c:303-324) */
  if (stage == 1) {
    if (s->c.dims > 1) {
      double r_1 = 1.0;
      if (s->c.geometry == OR_SPHERICAL && d == 1) r_1 = 1.0 / s->x[0][i0];
      for (i = nbeg; i <= nend; i++) {
        size_t c = base + i * stride;
        double inv_dl = (s->c.geometry == OR_SPHERICAL && d == 1) ? s->inv_dx[d][i] * r_1
                                                                  : s->inv_dx[d][i];
        s->Cdt[c] += 0.5 * (cmax[i - 1] + cmax[i]) * inv_dl * 1.0;
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
  if (s->c.line_force && vgrad_calc(s)) s->fail |= 1024;
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
    const int entr = s->c.entropy_switch ? nvar - 1 : -1;
    flags |= cons_to_prim(&s->U[c * nvar], v, nvar, gmm1, entr,
                          entr >= 0 && (s->flag[c] & OR_FLAG_ENTROPY));
    for (nv = 0; nv < nvar; nv++) s->V[nv * nc + c] = v[nv];
  }
  return flags;
}

/* ------------------------------------------------------------------ */
/* BLONDIN heating/cooling (Src/Cooling/BLONDIN/cooling.c:50-319)      */
/* ------------------------------------------------------------------ */

typedef struct {
  double xi, sqxi, sqsqxi, nH, n, tx, E, hc_init, dt_share;
  double comp_c_pre, comp_h_pre, line_c_pre, brem_c_pre, xray_h_pre;
} bl_ctx;

static double bl_ne_rat(double T)
{
  double ne_ratio;
  if (T < 1.5e4) {
    ne_ratio = 1e-2 + pow(10, (-51.59417133 + 12.27740153 * log10(T)));
  } else if (T >= 1.5e4 && T < 3.3e4) {
    ne_ratio = pow(10, (-3.80749689 + 0.86092628 * log10(T)));
  } else {
    ne_ratio = 1.21;
  }
  return ne_ratio;
}

static double bl_heatcool(const bl_ctx *b, double T)
{
  double sqT = sqrt(T);
  double ne = b->nH * bl_ne_rat(T);
  double comp_heat = b->comp_h_pre * (8.9e-36 * b->xi * b->tx);
  double comp_cool = b->comp_c_pre * (8.9e-36 * b->xi * (4.0 * T));
  double xray_heat = b->xray_h_pre * (1.5e-21 * (b->sqsqxi / sqT));
  double line_cool = b->line_c_pre * ((1e-16 * exp(-1.3e5 / T) / b->sqxi / T) +
                                      fmin(fmin(1e-24, 5e-27 * sqT), 1.5e-17 / T));
  double brem_cool = b->brem_c_pre * (3.3e-27 * sqT);
  return b->nH * (ne * comp_heat + b->nH * xray_heat - ne * comp_cool - ne * line_cool -
                  ne * brem_cool);
}

static double bl_zfunc(const bl_ctx *b, double temp)
{
  return (temp * b->n * C_KB / (2.0 / 3.0)) - b->E -
         b->dt_share * (b->hc_init + bl_heatcool(b, temp)) / 2.0;
}

/* which: 0 = zfunc, 1 = heatcool */
static double bl_func(const bl_ctx *b, int which, double x)
{
  return which == 0 ? bl_zfunc(b, x) : bl_heatcool(b, x);
}

/* Brent's method as in the reference (ITMAX 100, EPS 3e-8) */
static double bl_zbrent(const bl_ctx *bc, int which, double x1, double x2, double tol)
{
  const double EPS = 3.0e-8;
  int iter;
  double a = x1, b = x2, c = x2;
  double d = 0.0, e = 0.0;
  double fa = bl_func(bc, which, a), fb = bl_func(bc, which, b), fc = fb;
  double p, q, r, sv, tol1, xm;
  if (fb * fa > 0.0) return b;
  for (iter = 1; iter <= 100; iter++) {
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
    tol1 = 2.0 * EPS * fabs(b) + 0.5 * tol;
    xm = 0.5 * (c - b);
    if (fabs(xm) <= tol1 || fb == 0.0) return b;
    if (fabs(e) >= tol1 && fabs(fa) > fabs(fb)) {
      sv = fb / fa;
      if (a == c) {
        p = 2.0 * xm * sv;
        q = 1.0 - sv;
      } else {
        q = fa / fc;
        r = fb / fc;
        p = sv * (2.0 * xm * q * (q - r) - (b - a) * (r - 1.0));
        q = (q - 1.0) * (r - 1.0) * (sv - 1.0);
      }
      if (p > 0.0) q = -q;
      p = fabs(p);
      double min1 = 3.0 * xm * q - fabs(tol1 * q);
      double min2 = fabs(e * q);
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

/* ------------------------------------------------------------------ */
/* ODE cooling path: CoolingSource with the production problem's Radiat */
/* (Test_Problems/LineDrivenWind/cv_idl/cooling_source.c:50-246,       */
/* radiat.c:21-142) and the integrators of Src/Cooling/                */
/* cooling_ode_solver.c (SolveODE_RKF12 265-324, SolveODE_CK45 26-218) */
/* ------------------------------------------------------------------ */

#define OR_MAX_COOLING_RATE 0.1   /* g_maxCoolingRate (Src/globals.h:104) */
#define OR_MIN_COOLING_TEMP 1.e4  /* g_minCoolingTemp as Radiat sets it */

/* MeanMolecularWeight with COOLING == TABULATED (Src/mean_mol_weight.c:
 * 138-141) and the default mass fractions (Src/pluto.h:692-720) */
static double mu_tabulated(void)
{
  const double AH = 1.008, AHe = 4.004, AZ = 30.0;
  const double xH = 0.7110, xHe = 0.2741;
  const double xZ = (1.0 - xH - xHe);
  const double fHe = (xHe / AHe * AH / xH), fZ = (xZ / AZ * AH / xH);
  return (AH + fHe * AHe + fZ * AZ) / (2.0 + 3.0 * fHe + fZ * (1.0 + AZ * 0.5));
}

typedef struct {
  double x1, time, xi_s, tr_s;
  double ch, cc, xh, lc, bc;
} ode_cell;

/* Radiat: d(rho e)/dt in code units for the state v (v[re] = rho e); may
 * floor v[re] (radiat.c:58-62).  Returns 0, or 1 on a NaN temperature. */
static int ode_radiat(const or_sim *s, const ode_cell *oc, double *v, int re, double *rhs)
{
  double mu = s->c.mu, lx = s->c.l_star * s->c.f_x;
  double r = oc->x1 * s->c.unit_length;
  double rho = v[RHO] * s->c.unit_density;
  double nH = rho / (1.43 * C_MP), ne, T, prs, xi, tx, sqT, sqxi, sqsqxi;
  double E_cost = s->c.unit_length / s->c.unit_density / pow(s->c.unit_velocity, 3.0);
  double comp_heat, comp_cool, xray_heat, line_cool, brem_cool, lambda;
  prs = v[re] * (s->c.gamma - 1.0);
  if (prs < 0.0) {
    prs = small_pressure;
    v[re] = prs / (s->c.gamma - 1.0);
  }
  T = prs / v[RHO] * KELVIN_OF(s) * mu;
  if (T != T) {
    *rhs = 0.0;
    return 1;
  }
  if (T < OR_MIN_COOLING_TEMP) {
    *rhs = 0.0;
    return 0;
  }
  if (oc->time < 3.0) {
    xi = lx / nH / r / r;
    tx = s->c.t_x;
  } else {
    xi = oc->xi_s;
    tx = oc->tr_s;
  }
  sqT = sqrt(T);
  sqxi = sqrt(xi);
  sqsqxi = pow(xi, 0.25);
  ne = 1.21 * nH;   /* PY_CONNECT is not defined */
  comp_heat = oc->ch * (8.9e-36 * xi * tx);
  comp_cool = oc->cc * (8.9e-36 * xi * (4.0 * T));
  xray_heat = oc->xh * (1.5e-21 * (sqsqxi / sqT));
  line_cool = oc->lc * ((1e-16 * exp(-1.3e5 / T) / sqxi / T) +
                        fmin(fmin(1e-24, 5e-27 * sqT), 1.5e-17 / T));
  brem_cool = oc->bc * (3.3e-27 * sqT);
  lambda = nH * (ne * comp_heat + nH * xray_heat - ne * comp_cool - ne * line_cool -
                 ne * brem_cool);
  *rhs = v[NFLX] > 0.01 ? lambda * E_cost : 0.0;   /* v[TRC] */
  *rhs *= 1.0 - 1.0 / cosh(pow(T / OR_MIN_COOLING_TEMP, 12));
  return 0;
}

/* SolveODE_RKF12 for the one variable rho e: 2nd-order solution into
 * v2[re], returns the scaled difference to the 1st-order one */
static double ode_rkf12(const or_sim *s, const ode_cell *oc, const double *v0, double k1,
                        double *v2, int re, double dt, int *bad)
{
  double v1[NVMAX + 1], k2, v1st, vscal;
  int nv;
  for (nv = 0; nv <= re; nv++) v1[nv] = v0[nv];
  v1[re] = v0[re] + 0.5 * dt * k1;
  *bad |= ode_radiat(s, oc, v1, re, &k2);
  v2[re] = v0[re] + dt * k2;
  v1st = v0[re] + dt * k1;
  vscal = fabs(v0[re]) + dt * fabs(k1);
  return fabs(v2[re] - v1st) / fabs(vscal);
}

/* SolveODE_CK45 for rho e: Cash-Karp 4(5) with adaptive substeps until dt
 * is covered; v5[re] gets the result, the return value is the suggested
 * next step.  As in the reference, an accepted substep grows the step by
 * the cap 5 (the error used for the growth is reset to 1e-18 first). */
static double ode_ck45(const or_sim *s, const ode_cell *oc, const double *v0_in, double k1_in,
                       double *v5, int re, double dt, double tol, int *bad)
{
  const double c1 = 37.0 / 378.0, c3 = 250.0 / 621.0, c4 = 125.0 / 594.0,
               c6 = 512.0 / 1771.0;
  const double c2 = 0.0, c5 = 0.0;
  const double cs1 = 2825.0 / 27648.0, cs2 = 0.0, cs3 = 18575.0 / 48384.0,
               cs4 = 13525.0 / 55296.0, cs5 = 277.0 / 14336.0, cs6 = 0.25;
  const double b21 = 0.2;
  const double b31 = 3.0 / 40.0, b32 = 9.0 / 40.0;
  const double b41 = 0.3, b42 = -0.9, b43 = 1.2;
  const double b51 = -11.0 / 54.0, b52 = 2.5, b53 = -70.0 / 27.0, b54 = 35.0 / 27.0;
  const double b61 = 1631.0 / 55296.0, b62 = 175.0 / 512.0, b63 = 575.0 / 13824.0,
               b64 = 44275.0 / 110592.0, b65 = 253.0 / 4096.0;
  double v0[NVMAX + 1], v1[NVMAX + 1], k1 = k1_in, k2, k3, k4, k5, k6, v4, err, scrh;
  double t = 0.0, tend = dt;
  int nv, ksub = 0;
  for (nv = 0; nv <= re; nv++) v0[nv] = v1[nv] = v0_in[nv];
  for (;;) {
    v1[re] = v0[re] + dt * b21 * k1;
    *bad |= ode_radiat(s, oc, v1, re, &k2);
    v1[re] = v0[re] + dt * (b31 * k1 + b32 * k2);
    *bad |= ode_radiat(s, oc, v1, re, &k3);
    v1[re] = v0[re] + dt * (b41 * k1 + b42 * k2 + b43 * k3);
    *bad |= ode_radiat(s, oc, v1, re, &k4);
    v1[re] = v0[re] + dt * (b51 * k1 + b52 * k2 + b53 * k3 + b54 * k4);
    *bad |= ode_radiat(s, oc, v1, re, &k5);
    v1[re] = v0[re] + dt * (b61 * k1 + b62 * k2 + b63 * k3 + b64 * k4 + b65 * k5);
    *bad |= ode_radiat(s, oc, v1, re, &k6);
    v5[re] = v0[re] + dt * (c1 * k1 + c2 * k2 + c3 * k3 + c4 * k4 + c5 * k5 + c6 * k6);
    v4 = v0[re] + dt * (cs1 * k1 + cs2 * k2 + cs3 * k3 + cs4 * k4 + cs5 * k5 + cs6 * k6);
    scrh = fabs(v0[re]) + dt * fabs(k1);
    err = 0.0;
    {
      double e1 = fabs(v5[re] - v4) / fabs(scrh);
      err = MAXD(err, e1);
    }
    err /= tol;
    if (err < 1.0) {
      double dt_grow;
      ksub++;
      err = MAXD(0.0, 1.e-18);
      t += dt;
      dt_grow = 0.9 * dt * pow(err, -0.2);
      dt_grow = MIND(dt_grow, 5.0 * dt);
      dt = dt_grow;
      if (fabs(t / tend - 1.0) < 1.e-9) break;
      if (dt > (tend - t)) dt = tend - t;
      v0[re] = v5[re];
      *bad |= ode_radiat(s, oc, v0, re, &k1);
      if (ksub > 1000) {
        *bad |= 2;
        break;
      }
    } else {
      double dt_shrink = 0.9 * dt * pow(err, -0.25);
      dt = MAXD(dt_shrink, 0.05 * dt);
    }
  }
  return dt;
}

/* CoolingSource over the active cells: integrate d(rho e)/dt = Radiat from
 * 0 to dt (RKF12 when not stiff and accurate, else adaptive CK45 from a
 * rough first step), floor at g_minCoolingTemp for gas that crossed it,
 * and lower dt_cool to dt * g_maxCoolingRate / |p1/p0 - 1|. */
static void ode_cooling(or_sim *s, double dt, double t)
{
  int i, j, k, nv, nvar = s->c.nvar, re = nvar;
  size_t nc = (size_t)s->ntot[0] * s->ntot[1] * s->ntot[2];
  const double min_tol = 2.e-5, gm1 = s->c.gamma - 1.0, mu0 = mu_tabulated();
  ode_cell oc;
  oc.time = t;
  oc.ch = oc.cc = oc.xh = oc.lc = oc.bc = 1.0;
  for (k = s->beg[2]; k <= s->end[2]; k++)
  for (j = s->beg[1]; j <= s->end[1]; j++)
  for (i = s->beg[0]; i <= s->end[0]; i++) {
    size_t c = cidx(s, k, j, i);
    double v0[NVMAX + 1], v1[NVMAX + 1], k1, err = 0.0, prs, T0, T1, scrh;
    int stiff, bad = 0;
    oc.x1 = s->x[0][i];
    oc.xi_s = s->xi_s[c];
    oc.tr_s = s->tr_s[c];
    if (s->pre) {
      oc.ch = s->pre[0 * nc + c];
      oc.cc = s->pre[1 * nc + c];
      oc.xh = s->pre[2 * nc + c];
      oc.bc = s->pre[3 * nc + c];
      oc.lc = s->pre[4 * nc + c];
    }
    for (nv = 0; nv < nvar; nv++) v0[nv] = v1[nv] = s->V[nv * nc + c];
    prs = v0[PRS];
    T0 = v0[PRS] / v0[RHO] * KELVIN_OF(s) * mu0;
    v0[re] = v1[re] = prs / gm1;
    if (T0 <= 0.0) {
      s->fail |= 1024;
      return;
    }
    bad |= ode_radiat(s, &oc, v0, re, &k1);
    stiff = (fabs(k1) > 0.5 / dt ? 1 : 0);
    if (!stiff) {
      err = ode_rkf12(s, &oc, v0, k1, v1, re, dt, &bad);
      err /= min_tol;
    }
    if (stiff || err > 1.0) {
      double dt1, dts, t1 = 0.0;
      int done = 0;
      dt1 = 0.5 / (fabs(k1) + 1.0 / dt);
      do {
        if ((t1 + dt1) >= dt) {
          dt1 = dt - t1;
          done = 1;
        }
        dts = ode_ck45(s, &oc, v0, k1, v1, re, dt1, min_tol, &bad);
        t1 += dt1;
        dt1 = dts;
        if (done) break;
        for (nv = 0; nv <= re; nv++) v0[nv] = v1[nv];
        bad |= ode_radiat(s, &oc, v0, re, &k1);
      } while (!done);
    }
    if (bad) {
      s->fail |= 1024;
      return;
    }
    prs = v1[re] * gm1;
    T1 = prs / v1[RHO] * KELVIN_OF(s) * mu0;
    if (prs < 0.0) prs = small_pressure;
    if (T1 < OR_MIN_COOLING_TEMP && T0 > OR_MIN_COOLING_TEMP)
      prs = OR_MIN_COOLING_TEMP * v1[RHO] / (KELVIN_OF(s) * mu0);
    err = fabs(prs / s->V[PRS * nc + c] - 1.0);
    scrh = dt * OR_MAX_COOLING_RATE / err;
    s->dt_cool = MIND(s->dt_cool, scrh);
    s->V[PRS * nc + c] = prs;
  }
}

void or_cooling(or_sim *s, double dt, double t)
{
  int i, j, k;
  size_t nc = (size_t)s->ntot[0] * s->ntot[1] * s->ntot[2];
  double lx = s->c.l_star * s->c.f_x, mu = s->c.mu;
  double g_minCoolingTemp = 1.e4;
  bl_ctx b;
  if (s->c.cooling == 2) {
    ode_cooling(s, dt, t);
    return;
  }
  memset(&b, 0, sizeof(b));
  b.dt_share = dt * UNIT_T(s);
  b.comp_c_pre = b.comp_h_pre = b.line_c_pre = b.brem_c_pre = b.xray_h_pre = 1.0;
  for (k = s->beg[2]; k <= s->end[2]; k++)
  for (j = s->beg[1]; j <= s->end[1]; j++)
  for (i = s->beg[0]; i <= s->end[0]; i++) {
    size_t c = cidx(s, k, j, i);
    if (s->pre) {   /* cooling.c:73-79 */
      b.comp_h_pre = s->pre[0 * nc + c];
      b.comp_c_pre = s->pre[1 * nc + c];
      b.xray_h_pre = s->pre[2 * nc + c];
      b.brem_c_pre = s->pre[3 * nc + c];
      b.line_c_pre = s->pre[4 * nc + c];
    }
    double r = s->x[0][i] * s->c.unit_length;
    double rho = s->V[RHO * nc + c] * s->c.unit_density;
    double p = s->V[PRS * nc + c], T, T_f, t_l, t_u, test, E_f, p_f;
    T = p / s->V[RHO * nc + c] * KELVIN_OF(s) * mu;
    (void)T;
    b.E = (p * UNIT_P(s)) / (s->c.gamma - 1);
    b.nH = rho / (1.43 * C_MP);
    if (s->c.xi_const > 0.0) {
      b.xi = s->c.xi_const;
      b.tx = s->c.t_x;
    } else if (t <= 3.0) {
      b.xi = lx / b.nH / r / r;
      b.tx = s->c.t_x;
    } else {
      b.xi = s->xi_s[c];
      b.tx = s->tr_s[c];
    }
    b.n = rho / (mu * C_MP);
    T = b.E * (2.0 / 3.0) / (b.n * C_KB);
    if (T < g_minCoolingTemp) continue;
    b.sqxi = sqrt(b.xi);
    b.sqsqxi = pow(b.xi, 0.25);
    b.hc_init = bl_heatcool(&b, T);
    t_l = T * 0.9;
    t_u = T * 1.1;
    test = bl_zfunc(&b, t_l) * bl_zfunc(&b, t_u);
    while (test > 0 && test == test) {
      t_l *= 0.9;
      t_u *= 1.1;
      test = bl_zfunc(&b, t_l) * bl_zfunc(&b, t_u);
    }
    if (test != test) {
      T_f = T;
    } else {
      double hc_final;
      T_f = bl_zbrent(&b, 0, t_l, t_u, 1.0);
      hc_final = bl_heatcool(&b, T_f);
      if (hc_final * b.hc_init < 0.0) T_f = bl_zbrent(&b, 1, fmin(T_f, T), fmax(T_f, T), 1.0);
    }
    T_f = MAXD(T_f, g_minCoolingTemp);
    E_f = T_f / (2.0 / 3.0) * (b.n * C_KB);
    p_f = E_f * (s->c.gamma - 1) / UNIT_P(s);
    s->V[PRS * nc + c] = p_f;
  }
}

/* One BLONDIN solve for a (n_H, T, xi, T_x, dt) tuple, prefactors 1
 * (cooling.c:95-162 with the per-cell quantities given): the thermal
 * energy is E = T n kB / (2/3) with n = n_H 1.43 / mu, and the result is
 * T_f after the 1e4 K floor; T below 1e4 K is returned unchanged.  This is
 * how the surrogate's training pairs and its fallback are defined. */
double or_blondin_point(double nH, double T, double xi, double tx, double dt_s, double mu)
{
  bl_ctx b;
  double t_l, t_u, test, T_f;
  memset(&b, 0, sizeof(b));
  b.comp_c_pre = b.comp_h_pre = b.line_c_pre = b.brem_c_pre = b.xray_h_pre = 1.0;
  if (T < 1.e4) return T;
  b.dt_share = dt_s;
  b.nH = nH;
  b.n = nH * 1.43 / mu;
  b.E = T * b.n * C_KB / (2.0 / 3.0);
  b.xi = xi;
  b.tx = tx;
  b.sqxi = sqrt(b.xi);
  b.sqsqxi = pow(b.xi, 0.25);
  b.hc_init = bl_heatcool(&b, T);
  t_l = T * 0.9;
  t_u = T * 1.1;
  test = bl_zfunc(&b, t_l) * bl_zfunc(&b, t_u);
  while (test > 0 && test == test) {
    t_l *= 0.9;
    t_u *= 1.1;
    test = bl_zfunc(&b, t_l) * bl_zfunc(&b, t_u);
  }
  if (test != test) {
    T_f = T;
  } else {
    double hc_final;
    T_f = bl_zbrent(&b, 0, t_l, t_u, 1.0);
    hc_final = bl_heatcool(&b, T_f);
    if (hc_final * b.hc_init < 0.0) T_f = bl_zbrent(&b, 1, fmin(T_f, T), fmax(T_f, T), 1.0);
  }
  return MAXD(T_f, 1.e4);
}

/* FlagShock with SHOCK_FLATTENING == MULTID (flag_shock.c:81-250): zones
 * with div v < 0 and a pressure jump sum_d |p_{+1} - p_{-1}| above
 * 5 min(p, neighbours) are shocked; they and their neighbours in every
 * active direction get FLAG_MINMOD.  Flags start from zero every step
 * (main.c:260). */
static void flag_shock(or_sim *s)
{
  int i, j, k;
  int n0 = s->ntot[0], n1 = s->ntot[1], n2 = s->ntot[2];
  int ik = s->c.dims == 3, ij = s->c.dims >= 2;
  size_t nc = (size_t)n0 * n1 * n2, sx = 1, sy = n0, sz = (size_t)n0 * n1;
  const double *vx1 = s->V + VX1 * nc, *vx2 = s->V + VX2 * nc, *vx3 = s->V + VX3 * nc;
  const double *pt = s->V + PRS * nc;
  memset(s->flag, 0, nc);
  if (s->c.entropy_switch) memset(s->flag, OR_FLAG_ENTROPY, nc);   /* flag_shock.c:146-148 */
  for (k = ik; k < n2 - ik; k++)
  for (j = ij; j < n1 - ij; j++)
  for (i = 1; i < n0 - 1; i++) {
    size_t c = cidx(s, k, j, i);
    double divv, dvx1, dvx2 = 0.0, dvx3 = 0.0, pt_min, gradp;
    if (s->c.geometry == OR_CARTESIAN) {
      dvx1 = (vx1[c + sx] - vx1[c - sx]) / s->dx[0][i];
      if (ij) dvx2 = (vx2[c + sy] - vx2[c - sy]) / s->dx[1][j];
      if (ik) dvx3 = (vx3[c + sz] - vx3[c - sz]) / s->dx[2][k];
      divv = s->c.dims == 1 ? dvx1 : (s->c.dims == 2 ? dvx1 + dvx2 : dvx1 + dvx2 + dvx3);
    } else {
      double a1p = s->Ax1[((size_t)k * n1 + j) * (n0 + 1) + (i + 1)];
      double a1m = s->Ax1[((size_t)k * n1 + j) * (n0 + 1) + i];
      double a2p = s->Ax2[((size_t)k * (n1 + 1) + (j + 1)) * n0 + i];
      double a2m = s->Ax2[((size_t)k * (n1 + 1) + j) * n0 + i];
      dvx1 = a1p * (vx1[c + sx] + vx1[c]) - a1m * (vx1[c - sx] + vx1[c]);
      dvx2 = a2p * (vx2[c + sy] + vx2[c]) - a2m * (vx2[c - sy] + vx2[c]);
      divv = (dvx1 + dvx2) / s->dV[c];
    }
    if (divv < 0.0) {
      double pmin1, pmin2 = 0.0, pmin3 = 0.0, dpx1, dpx2 = 0.0, dpx3 = 0.0;
      pt_min = pt[c];
      pmin1 = MIND(pt[c + sx], pt[c - sx]);
      if (ij) pmin2 = MIND(pt[c + sy], pt[c - sy]);
      if (ik) pmin3 = MIND(pt[c + sz], pt[c - sz]);
      pt_min = MIND(pt_min, pmin1);
      if (ij) pt_min = MIND(pt_min, pmin2);
      if (ik) pt_min = MIND(pt_min, pmin3);
      dpx1 = fabs(pt[c + sx] - pt[c - sx]);
      if (ij) dpx2 = fabs(pt[c + sy] - pt[c - sy]);
      if (ik) dpx3 = fabs(pt[c + sz] - pt[c - sz]);
      gradp = s->c.dims == 1 ? dpx1 : (s->c.dims == 2 ? dpx1 + dpx2 : dpx1 + dpx2 + dpx3);
      if (s->c.entropy_switch == 1 && gradp > 0.05 * pt_min) {   /* flag_shock.c:251-267 */
        s->flag[c] &= ~OR_FLAG_ENTROPY;
        s->flag[c - sx] &= ~OR_FLAG_ENTROPY;
        s->flag[c + sx] &= ~OR_FLAG_ENTROPY;
        if (ij) { s->flag[c + sy] &= ~OR_FLAG_ENTROPY; s->flag[c - sy] &= ~OR_FLAG_ENTROPY; }
        if (ik) { s->flag[c + sz] &= ~OR_FLAG_ENTROPY; s->flag[c - sz] &= ~OR_FLAG_ENTROPY; }
      }
      if (s->c.shock_flattening && gradp > 5.0 * pt_min) {
        s->flag[c] |= OR_FLAG_HLL;
        s->flag[c] |= OR_FLAG_MINMOD;
        s->flag[c + sx] |= OR_FLAG_MINMOD;
        s->flag[c - sx] |= OR_FLAG_MINMOD;
        if (ij) { s->flag[c - sy] |= OR_FLAG_MINMOD; s->flag[c + sy] |= OR_FLAG_MINMOD; }
        if (ik) { s->flag[c - sz] |= OR_FLAG_MINMOD; s->flag[c + sz] |= OR_FLAG_MINMOD; }
      }
    }
  }
}

/* RK2 AdvanceStep (rk_step.c:29-384) */
static int advance_step(or_sim *s)
{
  int i, j, k, nv, nvar = s->c.nvar, flags;
  boundary(s);
  if (s->c.shock_flattening || s->c.entropy_switch) flag_shock(s);
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
    /* Strang alternation of the split source (main.c:479-485) */
    if (s->c.cooling && s->step % 2 != 0) or_cooling(s, s->g_dt, s->g_time);
    flags = advance_step(s);
    if (flags & 64) s->fail |= flags;
    if (s->c.cooling && s->step % 2 == 0) or_cooling(s, s->g_dt, s->g_time);
    if (s->fail & 1024) return 3;
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
