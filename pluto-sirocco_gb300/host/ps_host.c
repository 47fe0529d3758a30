/* ps_host.c -- host-side helpers of the C ABI: grid construction and the
 * blast-wave initial condition.  Compiled with -ffp-contract=off so that
 * every value is rounded exactly as in the reference's x86-64 build.
 *
 * Reference (paths inside the reference project):
 *   SetGrid ghosts/centres   Src/set_grid.c:100-140
 *   grid patches             Src/set_grid.c:405-450 (u, l+, r)
 *   RandomSeed/RandomNumber  Src/Math_Tools/math_random.c:36-183 (PRNG_MT)
 */
#include "ps_gb300.h"

#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

extern void ps_set_error_msg(const char *msg);

int ps_grid_build(int type, int n, int ngh, double xbeg, double xend,
                  double ratio, double *x, double *xl, double *xr, double *dx)
{
  int i, ib = ngh, ie = ngh + n - 1, nt = n + 2 * ngh;
  if (n < 1 || ngh < 0 || !x || !xl || !xr || !dx) {
    ps_set_error_msg("ps_grid_build: bad arguments");
    return PS_EINVAL;
  }
  if (type == PS_GRID_UNIFORM) {
    for (i = ib; i <= ie; i++) {
      dx[i] = (xend - xbeg) / (double)(n);
      xl[i] = xbeg + (double)(i - ib) * dx[i];
      xr[i] = xl[i] + dx[i];
    }
  } else if (type == PS_GRID_LOG_INC) {
    double dy;
    if (xbeg == 0.0) {
      ps_set_error_msg("ps_grid_build: logarithmic patch needs xbeg != 0");
      return PS_EINVAL;
    }
    dy = log10((xend + fabs(xbeg) - xbeg) / fabs(xbeg));
    dy /= (double)(n);
    xl[ib] = xbeg;
    for (i = ib; i <= ie; i++) {
      dx[i] = (xl[i] + fabs(xbeg) - xbeg) * (pow(10.0, dy) - 1.0);
      xr[i] = xl[i] + dx[i];
      if (i < ie) xl[i + 1] = xr[i];
    }
  } else if (type == PS_GRID_RATIO) {
    xl[ib] = xbeg;
    dx[ib] = (xend - xbeg) * (ratio - 1.0) / (pow(ratio, (ie - ib + 1)) - 1.0);
    xr[ib] = xl[ib] + dx[ib];
    for (i = ib + 1; i <= ie; i++) {
      dx[i] = dx[i - 1] * ratio;
      xl[i] = xl[i - 1] + dx[i - 1];
      xr[i] = xl[i] + dx[i];
    }
  } else {
    ps_set_error_msg("ps_grid_build: unknown patch type");
    return PS_EINVAL;
  }
  for (i = 0; i < ngh; i++) {
    dx[i] = dx[ib];
    xl[i] = xl[ib] - (ngh - i) * dx[ib];
    xr[i] = xl[i] + dx[ib];
    dx[ie + i + 1] = dx[ie];
    xl[ie + i + 1] = xl[ie] + (i + 1) * dx[ie];
    xr[ie + i + 1] = xl[ie] + (i + 2) * dx[ie];
  }
  for (i = 0; i < nt; i++) x[i] = 0.5 * (xl[i] + xr[i]);
  return 0;
}

/* MT19937-64 (Matsumoto & Nishimura), the published algorithm behind
 * PLUTO's PRNG_MT; real numbers on [0, 1] are (x >> 11) / (2^53 - 1). */
typedef struct {
  uint64_t s[312];
  int idx;
} mt64;

static void mt64_init(mt64 *g, uint64_t seed)
{
  int i;
  g->s[0] = seed;
  for (i = 1; i < 312; i++)
    g->s[i] = 6364136223846793005ull * (g->s[i - 1] ^ (g->s[i - 1] >> 62)) + (uint64_t)i;
  g->idx = 312;
}

static uint64_t mt64_u64(mt64 *g)
{
  static const uint64_t hi = 0xFFFFFFFF80000000ull, lo = 0x7FFFFFFFull;
  static const uint64_t a = 0xB5026F5AA96619E9ull;
  uint64_t y;
  if (g->idx >= 312) {
    int i;
    for (i = 0; i < 312; i++) {
      uint64_t m = (g->s[i] & hi) | (g->s[(i + 1) % 312] & lo);
      g->s[i] = g->s[(i + 156) % 312] ^ (m >> 1) ^ ((m & 1ull) ? a : 0ull);
    }
    g->idx = 0;
  }
  y = g->s[g->idx++];
  y ^= (y >> 29) & 0x5555555555555555ull;
  y ^= (y << 17) & 0x71D67FFFEDA60000ull;
  y ^= (y << 37) & 0xFFF7EEE000000000ull;
  y ^= (y >> 43);
  return y;
}

static double mt64_unit(mt64 *g)
{
  return (double)(mt64_u64(g) >> 11) * (1.0 / 9007199254740991.0);
}

int ps_init_blast(const ps_config *cfg, const double *x1, const double *x2,
                  const double *x3, double p_amb, double p_in, double r_in,
                  double noise, long seed, double *Vc)
{
  int ngh[3], ntot[3], d, i, j, k, nv;
  size_t nc, c;
  mt64 *g;
  if (!cfg || !x1 || !x2 || !Vc || cfg->nvar < 5 || (cfg->dims == 3 && !x3)) {
    ps_set_error_msg("ps_init_blast: bad arguments");
    return PS_EINVAL;
  }
  for (d = 0; d < 3; d++) {
    ngh[d] = d < cfg->dims ? 2 : 0;
    ntot[d] = cfg->nx[d] + 2 * ngh[d];
  }
  nc = (size_t)ntot[0] * ntot[1] * ntot[2];
  for (nv = 0; nv < cfg->nvar; nv++) {
    double val = nv == 0 ? 1.0 : (nv == 4 ? p_amb : 0.0);
    for (c = 0; c < nc; c++) Vc[nv * nc + c] = val;
  }
  g = (mt64 *)malloc(sizeof(mt64));
  if (!g) return PS_ENOMEM;
  mt64_init(g, (uint64_t)seed);
  for (k = ngh[2]; k < ngh[2] + cfg->nx[2]; k++)
  for (j = ngh[1]; j < ngh[1] + cfg->nx[1]; j++)
  for (i = ngh[0]; i < ngh[0] + cfg->nx[0]; i++) {
    double rnd = mt64_unit(g), ax, ay, r2;
    c = ((size_t)k * ntot[1] + j) * ntot[0] + i;
    Vc[0 * nc + c] = 1.0 * (1.0 + (-noise + rnd * (noise - (-noise))));
    Vc[1 * nc + c] = 0.0;
    Vc[2 * nc + c] = 0.0;
    Vc[3 * nc + c] = 0.0;
    ax = x1[i] - 0.5;
    ay = x2[j] - 0.5;
    r2 = ax * ax + ay * ay;
    if (cfg->dims == 3) {
      double az = x3[k] - 0.5;
      r2 = r2 + az * az;
    }
    Vc[4 * nc + c] = (sqrt(r2) < r_in) ? p_in : p_amb;
  }
  free(g);
  return 0;
}

/* ------------------------------------------------------------------ */
/* line-driven disk wind                                               */
/* ------------------------------------------------------------------ */

#define W_AMU  1.66053886e-24
#define W_G    6.6726e-8
#define W_KB   1.3806505e-16
#define W_PI   3.14159265358979
#define W_RGAS 8.3144598e7

int ps_init_wind(const ps_config *cfg, const ps_wind *w, const double *x1,
                 const double *xl1, const double *xr1, const double *dx1,
                 const double *x2, const double *xl2, const double *xr2,
                 double *Vc)
{
  int n0, n1, i, j;
  size_t nc;
  double gm_cgs, kelvin, rho_a;
  if (!cfg || !w || !x1 || !xl1 || !xr1 || !dx1 || !x2 || !xl2 || !xr2 || !Vc ||
      cfg->dims != 2 || cfg->nvar != (cfg->entropy_switch ? 7 : 6) ||
      cfg->geometry != PS_SPHERICAL) {
    ps_set_error_msg("ps_init_wind: needs a 2-D spherical configuration with nvar = 6 "
                     "(7 with the entropy switch)");
    return PS_EINVAL;
  }
  n0 = cfg->nx[0] + 2 * PS_NGHOST(cfg);
  n1 = cfg->nx[1] + 2 * PS_NGHOST(cfg);
  nc = (size_t)n0 * n1;
  gm_cgs = W_G * w->cent_mass;
  kelvin = w->unit_velocity * w->unit_velocity * W_AMU / W_KB;
  rho_a = w->dfloor / w->unit_density;
  (void)xl1;
  (void)xr1;
  for (j = 0; j < n1; j++) {
    /* theta centroid (Src/set_geometry.c:97-99) */
    double xL = xl2[j], xR = xr2[j];
    double th = sin(xR) - sin(xL) + xL * cos(xL) - xR * cos(xR);
    th /= cos(xL) - cos(xR);
    for (i = 0; i < n0; i++) {
      /* radial centroid (Src/set_geometry.c:81-84) */
      double r1 = x1[i] + 2.0 * x1[i] * dx1[i] * dx1[i] /
                              (12.0 * x1[i] * x1[i] + dx1[i] * dx1[i]);
      double r = r1 * w->unit_length;
      double cs2 = W_RGAS * w->t_iso / w->mu;
      double tt = tan(th);
      double rho_d = w->rho_0 * exp(-gm_cgs / (2.0 * cs2 * r * tt * tt)) / w->unit_density;
      size_t c = (size_t)j * n0 + i;
      double rho, trc;
      if (rho_d > rho_a) {
        rho = rho_d;
        trc = 1.0;
      } else {
        rho = rho_a;
        trc = 0.0;
      }
      Vc[0 * nc + c] = rho;
      Vc[1 * nc + c] = 0.0;
      Vc[2 * nc + c] = 0.0;
      Vc[3 * nc + c] = sqrt(gm_cgs / r) * sin(th) / w->unit_velocity;
      Vc[4 * nc + c] = rho * w->t_iso / (kelvin * w->mu);
      Vc[5 * nc + c] = trc;
      /* ComputeEntropy of Startup's Boundary (Src/entropy_switch.c) */
      if (cfg->entropy_switch) Vc[6 * nc + c] = Vc[4 * nc + c] / pow(rho, cfg->gamma);
    }
  }
  return 0;
}

int ps_wind_synthetic_flux(const ps_config *cfg, const ps_wind *w,
                           const double *x1, const double *x2,
                           double *fr, double *ft, double *fp)
{
  int n0, n1, na, i, j, a;
  size_t nc;
  char buf[64];
  double l_uv;
  if (!cfg || !w || !x1 || !x2 || !fr || !ft || !fp || cfg->dims != 2 || w->nangles < 1 ||
      w->nangles > 64) {
    ps_set_error_msg("ps_wind_synthetic_flux: bad arguments");
    return PS_EINVAL;
  }
  const int ng = PS_NGHOST(cfg);
  n0 = cfg->nx[0] + 2 * ng;
  n1 = cfg->nx[1] + 2 * ng;
  nc = (size_t)n0 * n1;
  na = w->nangles;
  memset(fr, 0, (size_t)na * nc * sizeof(double));
  memset(ft, 0, (size_t)na * nc * sizeof(double));
  memset(fp, 0, (size_t)na * nc * sizeof(double));
  l_uv = w->l_star * w->frac_uv;
  for (j = ng; j < n1 - ng; j++) {
    a = (int)floor(x2[j] / (2 * W_PI / 36));
    if (a < 0 || a >= na) continue;
    for (i = ng; i < n0 - ng; i++) {
      double r = x1[i] * w->unit_length;
      snprintf(buf, sizeof(buf), "%.12e", l_uv / (4 * 3.141592653589793 * r * r));
      fr[(size_t)a * nc + (size_t)j * n0 + i] = strtod(buf, NULL);
    }
  }
  return 0;
}

int ps_wind_synthetic_flux_dense(const ps_config *cfg, const ps_wind *w, const double *x1,
                                 const double *x2, double *fr, double *ft, double *fp)
{
  int n0, n1, na, i, j, a;
  size_t nc;
  char buf[64];
  double l_uv;
  if (!cfg || !w || !x1 || !x2 || !fr || !ft || !fp || cfg->dims != 2 || w->nangles < 1 ||
      w->nangles > 64) {
    ps_set_error_msg("ps_wind_synthetic_flux_dense: bad arguments");
    return PS_EINVAL;
  }
  const int ng = PS_NGHOST(cfg);
  n0 = cfg->nx[0] + 2 * ng;
  n1 = cfg->nx[1] + 2 * ng;
  nc = (size_t)n0 * n1;
  na = w->nangles;
  memset(fr, 0, (size_t)na * nc * sizeof(double));
  memset(ft, 0, (size_t)na * nc * sizeof(double));
  memset(fp, 0, (size_t)na * nc * sizeof(double));
  l_uv = w->l_star * w->frac_uv;
  /* the rounded values depend on the column i and the bin offset d only:
   * tabulate them once per column (d in [-(na-1), na-1]) */
  const int nd = 2 * na - 1;
  double *tr = (double *)malloc(sizeof(double) * (size_t)nd * 2);
  if (!tr) {
    ps_set_error_msg("ps_wind_synthetic_flux_dense: out of memory");
    return PS_EINVAL;
  }
  for (i = ng; i < n0 - ng; i++) {
    const double r = x1[i] * w->unit_length;
    const double f0 = l_uv / (4 * 3.141592653589793 * r * r);
    int d;
    for (d = -(na - 1); d <= na - 1; d++) {
      const double wt = d == 0 ? 1.0 : 0.05 / (1.0 + (double)abs(d));
      const double ang = d * (2.0 * 3.141592653589793 / na);
      snprintf(buf, sizeof(buf), "%.12e", f0 * wt * cos(ang));
      tr[2 * (d + na - 1)] = strtod(buf, NULL);
      snprintf(buf, sizeof(buf), "%.12e", f0 * wt * sin(ang));
      tr[2 * (d + na - 1) + 1] = strtod(buf, NULL);
    }
    for (j = ng; j < n1 - ng; j++) {
      const int a0 = (int)floor(x2[j] / (2 * W_PI / 36));
      for (a = 0; a < na; a++) {
        const int k = a - a0 + na - 1;
        if (k < 0 || k >= nd) continue;
        fr[(size_t)a * nc + (size_t)j * n0 + i] = tr[2 * k];
        ft[(size_t)a * nc + (size_t)j * n0 + i] = tr[2 * k + 1];
      }
    }
  }
  free(tr);
  return 0;
}
