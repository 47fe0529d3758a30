/* Initial condition, boundaries and body force for the reference CPU
   build of the 2-D line-driven disk wind.
   - Init: isothermal (T_ISO) disk-plane layer
       rho = RHO_0 exp(-G M / (2 cs^2 r tan^2 theta)),  cs^2 = Rgas T / MU,
     above a halo at DFLOOR; Keplerian v_phi = sqrt(G M / r) sin(theta);
     tracer 1 in the layer, 0 in the halo.
   - UserDefBoundary: side 0 applies the density floor (velocities scaled by
     rho/DFLOOR, sound speed kept, temperature floor 500 K) and the pressure
     floor of the SIROCCO disk-wind setup; X1_BEG copies the first active
     cell with v_r limited to inflow.
   - BodyForceVector: point-mass gravity -G M / r^2.
   Test infrastructure only: compiled by oracle/ref.mk into oracle/_ref. */
#include "pluto.h"

void Init (double *v, double x1, double x2, double x3)
{
  double gm_cgs = CONST_G * g_inputParam[CENT_MASS];
  double mu     = g_inputParam[MU];
  double T      = g_inputParam[T_ISO];
  double r      = x1 * UNIT_LENGTH;
  double cs2    = CONST_Rgas * T / mu;
  double tt     = tan(x2);
  double rho_d  = g_inputParam[RHO_0] * exp(-gm_cgs / (2.0 * cs2 * r * tt * tt)) / UNIT_DENSITY;
  double rho_a  = g_inputParam[DFLOOR] / UNIT_DENSITY;

  v[VX1] = 0.0;
  v[VX2] = 0.0;
  if (rho_d > rho_a) {
    v[RHO] = rho_d;
    v[TRC] = 1.0;
  } else {
    v[RHO] = rho_a;
    v[TRC] = 0.0;
  }
  v[VX3] = sqrt(gm_cgs / r) * sin(x2) / UNIT_VELOCITY;
  v[PRS] = v[RHO] * T / (KELVIN * mu);
}

void InitDomain (Data *d, Grid *grid)
{
}

void Analysis (const Data *d, Grid *grid)
{
}

void UserDefBoundary (const Data *d, RBox *box, int side, Grid *grid)
{
  int i, j, k, nv;
  double mu     = g_inputParam[MU];
  double dfloor = g_inputParam[DFLOOR] / UNIT_DENSITY;
  double tfloor = 5.e2;
  double pfloor = dfloor * tfloor / (KELVIN * mu);

  if (side == 0) {
    RBox cell_box;
    TOT_LOOP(k,j,i){
      int convert = 0;
      if (d->Vc[RHO][k][j][i] < dfloor) {
        double cs, dfact, temp;
        if (d->Vc[RHO][k][j][i] < 0.0) d->Vc[RHO][k][j][i] = dfloor;
        cs    = sqrt(g_gamma * d->Vc[PRS][k][j][i] / d->Vc[RHO][k][j][i]);
        dfact = d->Vc[RHO][k][j][i] / dfloor;
        d->Vc[RHO][k][j][i] = dfloor;
        d->Vc[VX1][k][j][i] = dfact * d->Vc[VX1][k][j][i];
        d->Vc[VX2][k][j][i] = dfact * d->Vc[VX2][k][j][i];
        d->Vc[VX3][k][j][i] = dfact * d->Vc[VX3][k][j][i];
        d->Vc[PRS][k][j][i] = cs * cs * d->Vc[RHO][k][j][i] / g_gamma;
        temp = d->Vc[PRS][k][j][i] / d->Vc[RHO][k][j][i] * KELVIN * mu;
        if (temp < tfloor) {
          d->Vc[PRS][k][j][i] = d->Vc[RHO][k][j][i] * tfloor / (KELVIN * mu);
        }
        d->Vc[TRC][k][j][i] = 0.0;
        convert = 1;
      }
      if (d->Vc[PRS][k][j][i] < pfloor) {
        d->Vc[PRS][k][j][i] = pfloor;
        convert = 1;
      }
      if (convert) {
        RBoxDefine (i, i, j, j, k, k, CENTER, &cell_box);
        PrimToCons3D(d->Vc, d->Uc, &cell_box, grid);
      }
    }
  }

  if (side == X1_BEG && box->vpos == CENTER) {
    BOX_LOOP(box,k,j,i){
      for (nv = 0; nv < NVAR; nv++) d->Vc[nv][k][j][i] = d->Vc[nv][k][j][IBEG];
      d->Vc[VX1][k][j][i] = MIN(d->Vc[VX1][k][j][i], 0.0);
    }
  }
}

void BodyForceVector (double *v, double *g, double x1, double x2, double x3)
{
  double gm_cgs  = CONST_G * g_inputParam[CENT_MASS];
  double gm_code = gm_cgs / (UNIT_LENGTH * UNIT_VELOCITY * UNIT_VELOCITY);
  g[IDIR] = -1.0 * gm_code / (x1 * x1);
  g[JDIR] = 0.0;
  g[KDIR] = 0.0;
}

double BodyForcePotential (double x1, double x2, double x3)
{
  return 0.0;
}
