/* ps_pluto_shim.c -- PLUTO's AdvanceStep() and SplitSource() on the GB300
 * path: the drop-in a PLUTO build links in place of
 * Src/Time_Stepping/rk_step.c and Src/split_source.c.  PLUTO's own main loop
 * (Src/main.c: Integrate, NextTimeStep, output) stays as it is and calls
 *
 *   int  AdvanceStep (Data *d, timeStep *Dts, Grid *grid)        Src/prototypes.h:5
 *   void SplitSource (Data *d, double dt, timeStep *Dts, Grid *grid)
 *                                                                Src/prototypes.h:204
 *
 * which run the step on the GPU through the C ABI of include/ps_gb300.h:
 *  - the first call creates the device context from the build's switches
 *    (definitions.h: DIMENSIONS, GEOMETRY, LIMITER, NVAR, COOLING, the
 *    numerics switches), the runtime ([Solver], [Time]) and the grid
 *    (x, xl, xr, dx and the boundary types of every direction); for the
 *    line-driven wind it hands over the [Parameters] block, the units and
 *    the fluxes read_sirocco_fluxes read (flux_r_UV / flux_t_UV / flux_p_UV);
 *  - every call copies Data.Vc to the device, runs the step and copies it
 *    back, so that everything PLUTO does between the calls (output,
 *    analysis, restart dumps) sees the current state;
 *  - AdvanceStep leaves Dts->invDt_hyp as UpdateStage does
 *    (Src/Time_Stepping/update_stage.c:389-394); SplitSource lowers
 *    Dts->dt_cool as CoolingSource does (Src/Cooling/cooling_source.c), both
 *    read by NextTimeStep (Src/main.c:601-644);
 *  - with PS_LEARNED_COOLING set to a network file (ps_sg_save),
 *    SplitSource runs the learned BLONDIN step instead of bracket + Brent;
 *  - a NaN in the state stops the run with QUIT_PLUTO(1), as CheckNaN does
 *    (Src/debug_tools.c:13-38); a host-side error prints ps_last_error()
 *    and stops it the same way.
 *
 * Built against the reference's own headers (it includes pluto.h and the
 * problem's definitions.h) by `make -f oracle/ref.mk CFG=<cfg> shim`,
 * which links PLUTO's objects without rk_step.o and split_source.o, this
 * file, and libps_gb300.so.
 */
#include "pluto.h"
#include "ps_gb300.h"

static ps_ctx *g_ps_ctx = NULL;
static ps_surrogate *g_ps_sg = NULL;

static void ps_shim_fail(const char *who, int rc)
{
  print("! %s failed (%d): %s\n", who, rc, ps_last_error());
  QUIT_PLUTO(1);
}

static int ps_shim_bc(int b)
{
  switch (b) {
    case OUTFLOW: return PS_BC_OUTFLOW;
    case REFLECTIVE: return PS_BC_REFLECTIVE;
    case AXISYMMETRIC: return PS_BC_AXISYM;
    case EQTSYMMETRIC: return PS_BC_EQTSYM;
    case PERIODIC: return PS_BC_PERIODIC;
    case USERDEF: return PS_BC_USERDEF;
    default: return -1;
  }
}

static ps_ctx *ps_shim_context(Data *d, Grid *grid)
{
  if (g_ps_ctx) return g_ps_ctx;
  Runtime *rt = RuntimeGet();
  ps_config c;
  memset(&c, 0, sizeof(c));
  c.dims = DIMENSIONS;
  for (int dir = 0; dir < 3; dir++) c.nx[dir] = dir < DIMENSIONS ? grid->np_int[dir] : 1;
  c.nvar = NVAR;
#if GEOMETRY == SPHERICAL
  c.geometry = PS_SPHERICAL;
#else
  c.geometry = PS_CARTESIAN;
#endif
#if LIMITER == MC_LIM
  c.limiter = PS_LIM_MC;
#elif LIMITER == VANLEER_LIM
  c.limiter = PS_LIM_VL;
#else
  c.limiter = PS_LIM_MM;
#endif
  c.solver = strcmp(rt->solv_type, "hll") == 0 ? PS_HLL : PS_HLLC;
  for (int dir = 0; dir < 3; dir++) {
    c.bc[2 * dir] = dir < DIMENSIONS ? ps_shim_bc(grid->lbound[dir]) : PS_BC_OUTFLOW;
    c.bc[2 * dir + 1] = dir < DIMENSIONS ? ps_shim_bc(grid->rbound[dir]) : PS_BC_OUTFLOW;
  }
  c.gamma = g_gamma;
  c.cfl = rt->cfl;
  c.cfl_max_var = rt->cfl_max_var;
  c.tstop = rt->tstop;
  c.first_dt = rt->first_dt;
#if COOLING == BLONDIN
  c.cooling = 1;
#elif COOLING == TABULATED
  c.cooling = 2;
#endif
  c.char_limiting = CHAR_LIMITING == YES;
  c.shock_flattening = SHOCK_FLATTENING == MULTID;
#if ENTROPY_SWITCH == SELECTIVE
  c.entropy_switch = 1;
#elif ENTROPY_SWITCH == ALWAYS
  c.entropy_switch = 2;
#endif

  int rc = ps_create(&c, &g_ps_ctx);
  if (rc) ps_shim_fail("ps_create", rc);
  for (int dir = 0; dir < DIMENSIONS; dir++) {
    rc = ps_set_grid(g_ps_ctx, dir, grid->x[dir], grid->xl[dir], grid->xr[dir], grid->dx[dir]);
    if (rc) ps_shim_fail("ps_set_grid", rc);
  }
  rc = ps_set_state(g_ps_ctx, d->Vc[0][0][0]);
  if (rc) ps_shim_fail("ps_set_state", rc);
#if LINE_DRIVEN_WIND != NO
  ps_wind w;
  memset(&w, 0, sizeof(w));
  w.unit_density = UNIT_DENSITY;
  w.unit_length = UNIT_LENGTH;
  w.unit_velocity = UNIT_VELOCITY;
  w.mu = g_inputParam[MU];
  w.rho_0 = g_inputParam[RHO_0];
  w.cent_mass = g_inputParam[CENT_MASS];
  w.t_iso = g_inputParam[T_ISO];
  w.l_star = g_inputParam[L_star];
  w.frac_x = g_inputParam[f_x];
  w.frac_uv = g_inputParam[f_uv];
  w.t_x = g_inputParam[T_x];
  w.krad = g_inputParam[KRAD];
  w.alpharad = g_inputParam[ALPHARAD];
  w.dfloor = g_inputParam[DFLOOR];
  w.body_force = (BODY_FORCE & VECTOR) ? 1 : 0;
  w.line_force = 1;
  w.floors = 1;
  w.nangles = NFLUX_ANGLES;
  rc = ps_set_wind(g_ps_ctx, &w, flux_r_UV[0][0][0], flux_t_UV[0][0][0], flux_p_UV[0][0][0]);
  if (rc) ps_shim_fail("ps_set_wind", rc);
#if COOLING == BLONDIN
  {
    /* PS_LEARNED_COOLING=<file>: SplitSource runs the learned BLONDIN step
       with the network saved there by ps_sg_save (the reference method
       stays the fallback for the cells it hands back) */
    const char *net = getenv("PS_LEARNED_COOLING");
    if (net && *net) {
      rc = ps_sg_load(net, &g_ps_sg);
      if (rc) ps_shim_fail("ps_sg_load", rc);
      rc = ps_set_surrogate(g_ps_ctx, g_ps_sg, 1);
      if (rc) ps_shim_fail("ps_set_surrogate", rc);
      print("> learned cooling step, network %s\n", net);
    }
  }
#endif
#endif
  return g_ps_ctx;
}

static void ps_shim_check(const char *who, int rc)
{
  if (rc < 0) ps_shim_fail(who, rc);
  if (rc & PS_F_NAN) {
    print("! %s: NaN found in the state\n", who);
    QUIT_PLUTO(1);
  }
  if (rc & PS_F_COOLING) {
    print("! %s: the cooling integration failed\n", who);
    QUIT_PLUTO(1);
  }
}

int AdvanceStep(Data *d, timeStep *Dts, Grid *grid)
{
  ps_ctx *ctx = ps_shim_context(d, grid);
  int rc = ps_set_state(ctx, d->Vc[0][0][0]);
  if (rc) ps_shim_fail("ps_set_state", rc);
  double inv = Dts->invDt_hyp;
  rc = ps_advance_step(ctx, g_dt, &inv);
  ps_shim_check("AdvanceStep", rc);
  Dts->invDt_hyp = inv;
  int rg = ps_get_state(ctx, d->Vc[0][0][0]);
  if (rg) ps_shim_fail("ps_get_state", rg);
#if FAILSAFE == YES
  if (rc & PS_F_CONS2PRIM) return 1;
#endif
  return 0;
}

void SplitSource(Data *d, double dt, timeStep *Dts, Grid *grid)
{
#if COOLING != NO
  ps_ctx *ctx = ps_shim_context(d, grid);
  int rc = ps_set_state(ctx, d->Vc[0][0][0]);
  if (rc) ps_shim_fail("ps_set_state", rc);
  double dt_cool = 1.e38;
  rc = ps_split_source_dt(ctx, dt, g_time, &dt_cool);
  ps_shim_check("SplitSource", rc);
  Dts->dt_cool = MIN(Dts->dt_cool, dt_cool);
  int rg = ps_get_state(ctx, d->Vc[0][0][0]);
  if (rg) ps_shim_fail("ps_get_state", rg);
#endif
}
