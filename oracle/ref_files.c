/* ref_files.c -- input files of the reference's own build for the synthetic
 * wind configurations.
 *
 * TEST INFRASTRUCTURE ONLY (part of liboracle.so): used by
 * tests/golden/make_golden.py and by bench.py's reference arm to hand the
 * reference's own serial binary the same synthetic inputs the GPU and the
 * oracle get.  The product never links or calls it.
 *
 * or_write_wind_flux writes directional_flux_{r,theta,phi}.dat in the text
 * layout read_sirocco_fluxes parses (Src/LineDriven/line_connect.c:84-165):
 * two header lines, the second holding the angle count as its third token,
 * then one row per active cell, j outer and i inner:
 *     i j 0 r[cm] theta[rad] F_0 .. F_{na-1}
 * with every number printed as %.12e.  The flux is the single-bin synthetic
 * one of oracle.synthetic_flux: L_UV / (4 pi r^2) in the bin
 * floor(theta / (2 pi / 36)) of the radial file, zero elsewhere and in the
 * theta and phi files.  x1, x2 are the cell-centre arrays of the total box
 * (x1 in code units), ngh the ghost zones per side; bit a of `axes` selects
 * the file of axis a (r, theta, phi). */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define OR_PI 3.14159265358979323846

static int write_one(const char *path, int axis, int nr, int nt, const double *x1,
                     const double *x2, int ngh, double l_uv, double unit_length, int na)
{
  FILE *f = fopen(path, "w");
  if (!f) return -1;
  /* a buffer of the call's own: several threads write files at once */
  char *buf = malloc(1 << 20);
  if (buf) setvbuf(f, buf, _IOFBF, 1 << 20);
  fprintf(f, "# synthetic directional UV flux\n# nangles %d\n", na);
  static const char zero[] = " 0.000000000000e+00";
  for (int j = ngh; j < nt + ngh; j++) {
    const int a = (int)floor(x2[j] / (2 * 3.14159265358979 / 36));
    for (int i = ngh; i < nr + ngh; i++) {
      fprintf(f, "%d %d 0 %.12e %.12e", i - ngh, j - ngh, x1[i] * unit_length, x2[j]);
      const double r = x1[i] * unit_length;
      for (int b = 0; b < na; b++) {
        if (axis == 0 && b == a)
          fprintf(f, " %.12e", l_uv / (4 * OR_PI * r * r));
        else
          fputs(zero, f);
      }
      fputc('\n', f);
    }
  }
  const int rc = fclose(f) == 0 ? 0 : -1;
  free(buf);
  return rc;
}

int or_write_wind_flux(const char *dir, int nr, int nt, const double *x1, const double *x2,
                       int ngh, double l_uv, double unit_length, int na, int axes)
{
  static const char *names[3] = {"directional_flux_r.dat", "directional_flux_theta.dat",
                                 "directional_flux_phi.dat"};
  char path[4096];
  for (int ax = 0; ax < 3; ax++) {
    if (!(axes & (1 << ax))) continue;
    if (snprintf(path, sizeof(path), "%s/%s", dir, names[ax]) >= (int)sizeof(path)) return -1;
    if (write_one(path, ax, nr, nt, x1, x2, ngh, l_uv, unit_length, na)) return -1;
  }
  return 0;
}
