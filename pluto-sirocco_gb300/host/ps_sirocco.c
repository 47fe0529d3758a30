/* ps_sirocco.c -- readers of the files a SIROCCO radiative-transfer run
 * hands to the wind problem (Src/LineDriven/line_connect.c:43-497):
 *
 *   directional_flux_{r,theta,phi}.dat   two header lines (the second holds
 *       the number of angle bins as its third word), then one record per
 *       cell: "i j k x1[cm] x2[rad] F_0 ... F_{NA-1}"  (read_sirocco_fluxes)
 *   py_heatcool.dat   a header line, then "i j rcen[cm] thetacen vol t_e t_r
 *       xi ne heat_xray heat_comp heat_lines heat_ff cool_comp cool_lines
 *       cool_ff dens n_h"  (read_sirocco_heatcool, flag 1)
 *   prefactors.dat   a header line, then "i rcen[cm] j thetacen dens
 *       comp_h comp_c xray_h brem_c line_c xi_ion"  (same function)
 *   M_UV_data.dat   a header line whose second word is the number of
 *       points, a word and the t values, then per cell "i j x1[cm] x2[rad]
 *       M_0 ... M_{n-1}"  (read_sirocco_fluxes with KRAD = ALPHARAD = 999)
 *
 * Records are placed on the grid by their coordinates, with the reference's
 * tolerances: |1 - x1_file / UNIT_LENGTH / x1[i]| < 1e-6 and
 * |1 - x2_file / x2[j]| < 1e-6 for the fluxes, relative 1e-5 on
 * rcen / UNIT_LENGTH and thetacen for the other two files.  The reference
 * scans every cell for every record; here each coordinate is found by
 * binary search in the monotonic cell-centre arrays (the nearest centre and
 * its neighbours are tested), which gives the same placement whenever a
 * record matches one cell.  Arrays are over the total box, [j][i] (flux
 * arrays [angle][j][i]); cells without a record keep what the caller put
 * there. */
#include "ps_gb300.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

void ps_set_error_msg(const char *msg);

#define PS_LINE 65536

/* index of the active cell whose centre matches v under `ok`, or -1 */
static int find_cell(const double *x, int beg, int n, double v,
                     int (*ok)(double v, double xc, double tol), double tol)
{
  int lo = beg, hi = beg + n - 1;
  if (n <= 0) return -1;
  while (hi - lo > 1) {
    const int mid = lo + (hi - lo) / 2;
    if (x[mid] < v) lo = mid; else hi = mid;
  }
  for (int c = lo - 1; c <= hi + 1; c++) {
    if (c < beg || c > beg + n - 1) continue;
    if (ok(v, x[c], tol)) return c;
  }
  return -1;
}

/* read_sirocco_fluxes: fabs(1.0 - x_in / x[i]) < tol (x_in already in code units) */
static int match_ratio(double v, double xc, double tol) { return fabs(1.0 - v / xc) < tol; }
/* read_sirocco_heatcool: fabs((x_in - x[i]) / x_in) < tol */
static int match_rel(double v, double xc, double tol) { return fabs((v - xc) / v) < tol; }

static int fail(const char *msg)
{
  ps_set_error_msg(msg);
  return PS_EINVAL;
}

int ps_read_sirocco_fluxes(const ps_config *cfg, double unit_length, const double *x1,
                           const double *x2, const char *dir, int max_angles, double *fr,
                           double *ft, double *fp, long *matched)
{
  static const char *names[3] = {"directional_flux_r.dat", "directional_flux_theta.dat",
                                 "directional_flux_phi.dat"};
  double *out[3] = {fr, ft, fp};
  int na = -1;
  long count = 0;
  if (!cfg || !x1 || !x2 || !dir || !fr || !ft || !fp || max_angles <= 0 || !(unit_length > 0))
    return fail("ps_read_sirocco_fluxes: bad arguments");
  const int ng = PS_NGHOST(cfg), n0 = cfg->nx[0] + 2 * ng, n1 = cfg->nx[1] + 2 * ng;
  const size_t plane = (size_t)n0 * n1;
  char *line = (char *)malloc(PS_LINE);
  double *vals = (double *)malloc(sizeof(double) * (size_t)max_angles);
  if (!line || !vals) {
    free(line);
    free(vals);
    return fail("ps_read_sirocco_fluxes: out of memory");
  }
  int rc = 0;
  for (int ax = 0; ax < 3 && !rc; ax++) {
    char path[4096];
    snprintf(path, sizeof(path), "%s/%s", dir, names[ax]);
    FILE *f = fopen(path, "r");
    if (!f) {
      rc = fail("ps_read_sirocco_fluxes: a directional flux file is missing");
      break;
    }
    long nbins = -1;
    if (!fgets(line, PS_LINE, f) || !fgets(line, PS_LINE, f) ||
        sscanf(line, "%*s %*s %ld", &nbins) != 1 || nbins <= 0) {
      fclose(f);
      rc = fail("ps_read_sirocco_fluxes: flux header improperly formatted");
      break;
    }
    if (ax == 0) {
      if (nbins > max_angles) {
        fclose(f);
        rc = fail("ps_read_sirocco_fluxes: more angle bins than max_angles");
        break;
      }
      na = (int)nbins;
    } else if (nbins != na) {
      fclose(f);
      rc = fail("ps_read_sirocco_fluxes: the flux files disagree on the number of angle bins");
      break;
    }
    long ii, jj, kk;
    double x1in, x2in;
    while (fscanf(f, "%ld", &ii) == 1) {
      if (fscanf(f, "%ld %ld %le %le", &jj, &kk, &x1in, &x2in) != 4) {
        rc = fail("ps_read_sirocco_fluxes: error in reading a flux file");
        break;
      }
      for (int a = 0; a < na && !rc; a++)
        if (fscanf(f, "%le", &vals[a]) != 1)
          rc = fail("ps_read_sirocco_fluxes: error in reading a flux file");
      if (rc) break;
      const int i = find_cell(x1, ng, cfg->nx[0], x1in / unit_length, match_ratio, 1e-6);
      const int j = find_cell(x2, ng, cfg->nx[1], x2in, match_ratio, 1e-6);
      if (i < 0 || j < 0) continue;
      for (int a = 0; a < na; a++) out[ax][(size_t)a * plane + (size_t)j * n0 + i] = vals[a];
      if (ax == 0) count++;
    }
    fclose(f);
  }
  free(line);
  free(vals);
  if (rc) return rc;
  if (matched) *matched = count;
  return na;
}

int ps_read_sirocco_heatcool(const ps_config *cfg, double unit_length, const double *x1,
                             const double *x2, const char *path, double *xi, double *t_r,
                             long *matched)
{
  if (!cfg || !x1 || !x2 || !path || !xi || !t_r || !(unit_length > 0))
    return fail("ps_read_sirocco_heatcool: bad arguments");
  FILE *f = fopen(path, "r");
  if (!f) return fail("ps_read_sirocco_heatcool: cannot open the file");
  const int ng = PS_NGHOST(cfg), n0 = cfg->nx[0] + 2 * ng;
  char *line = (char *)malloc(PS_LINE);
  if (!line) {
    fclose(f);
    return fail("ps_read_sirocco_heatcool: out of memory");
  }
  long count = 0;
  int rc = 0;
  if (!fgets(line, PS_LINE, f)) rc = fail("ps_read_sirocco_heatcool: no header line");
  while (!rc && fgets(line, PS_LINE, f)) {
    int ii, jj;
    double rcen, thetacen, vol, t_e, tr, x, ne, h1, h2, h3, h4, c1, c2, c3, dens, n_h;
    const int nw = sscanf(line, "%d %d %le %le %le %le %le %le %le %le %le %le %le %le %le %le %le %le",
                          &ii, &jj, &rcen, &thetacen, &vol, &t_e, &tr, &x, &ne, &h1, &h2, &h3,
                          &h4, &c1, &c2, &c3, &dens, &n_h);
    if (nw != 18) {
      rc = fail("ps_read_sirocco_heatcool: py_heatcool file incorrectly formatted");
      break;
    }
    const int i = find_cell(x1, ng, cfg->nx[0], rcen / unit_length, match_rel, 1e-5);
    const int j = find_cell(x2, ng, cfg->nx[1], thetacen, match_rel, 1e-5);
    if (i < 0 || j < 0) continue;
    const size_t c = (size_t)j * n0 + i;
    xi[c] = x < 1.0 ? 1.0 : x;
    t_r[c] = tr < 1.e3 ? 1.e3 : tr;
    count++;
  }
  free(line);
  fclose(f);
  if (rc) return rc;
  if (matched) *matched = count;
  return 0;
}

int ps_read_sirocco_prefactors(const ps_config *cfg, double unit_length, const double *x1,
                               const double *x2, const char *path, double *pre, long *matched)
{
  if (!cfg || !x1 || !x2 || !path || !pre || !(unit_length > 0))
    return fail("ps_read_sirocco_prefactors: bad arguments");
  FILE *f = fopen(path, "r");
  if (!f) return fail("ps_read_sirocco_prefactors: cannot open the file");
  const int ng = PS_NGHOST(cfg), n0 = cfg->nx[0] + 2 * ng, n1 = cfg->nx[1] + 2 * ng;
  const size_t plane = (size_t)n0 * n1;
  char *line = (char *)malloc(PS_LINE);
  if (!line) {
    fclose(f);
    return fail("ps_read_sirocco_prefactors: out of memory");
  }
  long count = 0;
  int rc = 0;
  if (!fgets(line, PS_LINE, f)) rc = fail("ps_read_sirocco_prefactors: no header line");
  while (!rc && fgets(line, PS_LINE, f)) {
    int ii, jj;
    double rcen, thetacen, dens, v[6];
    const int nw = sscanf(line, "%d %le %d %le %le %le %le %le %le %le %le", &ii, &rcen, &jj,
                          &thetacen, &dens, &v[0], &v[1], &v[2], &v[3], &v[4], &v[5]);
    if (nw != 11) {
      rc = fail("ps_read_sirocco_prefactors: prefactor file incorrectly formatted");
      break;
    }
    const int i = find_cell(x1, ng, cfg->nx[0], rcen / unit_length, match_rel, 1e-5);
    const int j = find_cell(x2, ng, cfg->nx[1], thetacen, match_rel, 1e-5);
    if (i < 0 || j < 0) continue;
    const size_t c = (size_t)j * n0 + i;
    for (int k = 0; k < 6; k++) pre[(size_t)k * plane + c] = v[k];
    count++;
  }
  free(line);
  fclose(f);
  if (rc) return rc;
  if (matched) *matched = count;
  return 0;
}

int ps_read_m_uv_fit(const ps_config *cfg, double unit_length, const double *x1,
                     const double *x2, const char *path, int max_points, double *t_fit,
                     double *m_fit, long *matched)
{
  if (!cfg || !x1 || !x2 || !path || !t_fit || !m_fit || max_points <= 0 || !(unit_length > 0))
    return fail("ps_read_m_uv_fit: bad arguments");
  FILE *f = fopen(path, "r");
  if (!f) return fail("ps_read_m_uv_fit: cannot open the file");
  const int ng = PS_NGHOST(cfg), n0 = cfg->nx[0] + 2 * ng, n1 = cfg->nx[1] + 2 * ng;
  const size_t plane = (size_t)n0 * n1;
  char *line = (char *)malloc(PS_LINE);
  double *vals = (double *)malloc(sizeof(double) * (size_t)max_points);
  if (!line || !vals) {
    free(line);
    free(vals);
    fclose(f);
    return fail("ps_read_m_uv_fit: out of memory");
  }
  long np = -1, count = 0;
  int rc = 0;
  if (!fgets(line, PS_LINE, f) || sscanf(line, "%*s %ld", &np) != 1 || np <= 0)
    rc = fail("ps_read_m_uv_fit: header improperly formatted");
  else if (np > max_points)
    rc = fail("ps_read_m_uv_fit: more points than max_points");
  if (!rc && fscanf(f, "%*s ") != 0) rc = fail("ps_read_m_uv_fit: no t header");
  for (long k = 0; !rc && k < np; k++)
    if (fscanf(f, "%le", &t_fit[k]) != 1) rc = fail("ps_read_m_uv_fit: error in reading t");
  long ii, jj;
  double x1in, x2in;
  while (!rc && fscanf(f, "%ld ", &ii) == 1) {
    if (fscanf(f, "%ld %le %le", &jj, &x1in, &x2in) != 3) {
      rc = fail("ps_read_m_uv_fit: error in reading a record");
      break;
    }
    for (long k = 0; k < np && !rc; k++)
      if (fscanf(f, "%le", &vals[k]) != 1) rc = fail("ps_read_m_uv_fit: error in reading a record");
    if (rc) break;
    const int i = find_cell(x1, ng, cfg->nx[0], x1in / unit_length, match_ratio, 1e-6);
    const int j = find_cell(x2, ng, cfg->nx[1], x2in, match_ratio, 1e-6);
    if (i < 0 || j < 0) continue;
    for (long k = 0; k < np; k++) m_fit[(size_t)k * plane + (size_t)j * n0 + i] = vals[k];
    count++;
  }
  free(line);
  free(vals);
  fclose(f);
  if (rc) return rc;
  if (matched) *matched = count;
  return (int)np;
}
