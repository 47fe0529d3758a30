/* Initial condition for the reference CPU build of the 3-D blast wave:
   rho = 1*(1 + U(-NOISE, NOISE)) drawn cell by cell in (k, j, i) order over
   the active domain from PLUTO's MT19937-64 generator (PRNG_MT) seeded
   with 1, p = P_AMB, v = 0, and p = P_IN where the distance from
   (0.5, 0.5, 0.5) is below R_IN.  Ghost cells start at the ambient state;
   the first Boundary() call overwrites them.
   Test infrastructure only: compiled by oracle/ref.mk into oracle/_ref. */
#include "pluto.h"

void Init (double *v, double x1, double x2, double x3)
{
  v[RHO] = 1.0;
  v[VX1] = 0.0;
  v[VX2] = 0.0;
  v[VX3] = 0.0;
  v[PRS] = g_inputParam[P_AMB];
}

void InitDomain (Data *d, Grid *grid)
{
  int i, j, k;
  double *x1 = grid->x[IDIR];
  double *x2 = grid->x[JDIR];
  double *x3 = grid->x[KDIR];
  double ax, ay, az, r;

  RandomSeed (1, 0);
  DOM_LOOP(k,j,i){
    d->Vc[RHO][k][j][i] = 1.0*(1.0 + RandomNumber(-g_inputParam[NOISE],
                                                   g_inputParam[NOISE]));
    d->Vc[VX1][k][j][i] = 0.0;
    d->Vc[VX2][k][j][i] = 0.0;
    d->Vc[VX3][k][j][i] = 0.0;
    ax = x1[i] - 0.5;
    ay = x2[j] - 0.5;
    az = x3[k] - 0.5;
    r  = sqrt(ax*ax + ay*ay + az*az);
    d->Vc[PRS][k][j][i] = (r < g_inputParam[R_IN]) ? g_inputParam[P_IN]
                                                    : g_inputParam[P_AMB];
  }
}

void Analysis (const Data *d, Grid *grid)
{
}

void UserDefBoundary (const Data *d, RBox *box, int side, Grid *grid)
{
}
