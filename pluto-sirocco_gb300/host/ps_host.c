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
