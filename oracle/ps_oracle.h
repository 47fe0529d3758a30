/* ps_oracle.h -- CPU oracle for the PLUTO-sirocco hydro step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the
 * reference algorithm (PLUTO 4.4 + sirocco additions) used as the checker
 * for the CUDA path and as the timed CPU baseline ("port").  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it; the
 * product never links or calls it.
 *
 * Parity pinning: the restatement is compared bit for bit against the
 * reference's own serial build (oracle/ref.mk -> oracle/_ref/<cfg>/pluto)
 * through golden vectors committed under tests/golden/.
 *
 * Array conventions follow the reference: primitive variables V are stored
 * [nv][k][j][i] over the total box including ghost zones
 * (Src/structs.h:526-540, Src/arrays.c:250-300); grid arrays are 1-D per
 * direction over the total box (Src/structs.h:133-187).
 */
#ifndef PS_ORACLE_H
#define PS_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Values mirror Src/pluto.h:163-171 and the limiter/solver names. */
enum { OR_CARTESIAN = 0, OR_SPHERICAL = 3 };
enum { OR_LIM_MC = 0, OR_LIM_VL = 1, OR_LIM_MM = 2 };
enum { OR_HLLC = 0, OR_HLL = 1 };
enum { OR_BC_OUTFLOW = 1, OR_BC_REFLECTIVE = 2, OR_BC_AXISYMMETRIC = 3,
       OR_BC_EQTSYMMETRIC = 4, OR_BC_PERIODIC = 5, OR_BC_USERDEF = 8 };
enum { OR_GRID_UNIFORM = 0, OR_GRID_LOG_INC = 1, OR_GRID_RATIO = 2 };

typedef struct {
  int    dims;          /* 1, 2 or 3 active directions                     */
  int    nx[3];         /* active cells per direction (1 if inactive)      */
  int    nvar;          /* 5 (rho, vx1, vx2, vx3, prs) + passive scalars   */
  int    geometry;      /* OR_CARTESIAN / OR_SPHERICAL                      */
  int    limiter;       /* OR_LIM_*                                        */
  int    solver;        /* OR_HLLC / OR_HLL                                */
  int    bc[6];         /* X1_BEG, X1_END, X2_BEG, X2_END, X3_BEG, X3_END  */
  int    gridtype[3];   /* OR_GRID_*                                       */
  double xbeg[3], xend[3], ratio[3];
  double gamma;
  double cfl, cfl_max_var, tstop, first_dt;
  int    cooling;       /* 0: none; 1: BLONDIN split source (Strang rules);
                           2: the ODE path (COOLING TABULATED with the
                           production problem's CoolingSource/Radiat)     */
  /* line-driven disk wind (all zero for the plain hydro configurations) */
  int    body_force;    /* point-mass gravity (BodyForceVector)            */
  int    line_force;    /* VGradCalc + LineForce                           */
  int    floors;        /* internal-boundary density/pressure floors       */
  double unit_density, unit_length, unit_velocity;
  double mu, rho_0, cent_mass, t_iso, l_star, f_x, f_uv, t_x;
  double krad, alpharad, dfloor;
  /* > 0: BLONDIN at this constant ionisation parameter with t_x (the
   * Cartesian cooling configuration) instead of xi from the state */
  double xi_const;
  /* CHAR_LIMITING YES: PLM limited on the characteristic variables of the
   * primitive HD system (Src/States/plm_states.c:481-746) */
  int    char_limiting;
  /* SHOCK_FLATTENING MULTID: minmod reconstruction in and next to shocked
   * zones (Src/flag_shock.c:81-250, plm_states.c:176-193, 613-625) */
  int    shock_flattening;
  /* ENTROPY_SWITCH: 0 NO, 1 SELECTIVE, 2 ALWAYS.  The entropy s = p/rho^gamma
   * is the last variable; pressure is recovered from rho s in the zones
   * tagged FLAG_ENTROPY (Src/entropy_switch.c, Src/HD/mappers.c:185-221,
   * Src/flag_shock.c:138-148, 251-267) */
  int    entropy_switch;
} or_config;

typedef struct or_sim or_sim;

or_sim *or_create(const or_config *cfg);
void    or_destroy(or_sim *s);

/* Geometry of the total box (ngh ghosts each side of active dirs). */
int     or_ntot(const or_sim *s, int dir);
int     or_nghost(const or_sim *s, int dir);
/* which: 0 = x (centre), 1 = xl, 2 = xr, 3 = dx, 4 = xgc (centroid) */
const double *or_grid(const or_sim *s, int dir, int which);

/* Primitive state [nv][k][j][i] over the total box (read/write). */
double *or_state(or_sim *s);

/* 2-D/3-D blast initial condition: rho = 1*(1 + U(-noise, noise)) from the
 * MT19937-64 sequence seeded with `seed` (PLUTO's PRNG_MT), drawn over the
 * active domain in (k, j, i) order; p = p_in where |x - centre| < r_in
 * else p_amb; v = 0. */
void    or_init_blast(or_sim *s, double p_amb, double p_in, double r_in,
                      double noise, long seed);

/* Line-driven wind: initial condition of the wind problem (Init() called
 * on every cell of the total box at the volume centroids, as Startup does)
 * followed by read_sirocco_heatcool(flag = 0): frozen xi and T_r. */
void    or_init_wind(or_sim *s);
/* The frozen xi / T_r and the entropy of the state the caller put in the
 * context (read_sirocco_heatcool(flag = 0), Startup's ComputeEntropy). */
void    or_wind_reset(or_sim *s);

/* Directional UV fluxes, [angle][k][j][i] over the total box, for the
 * line force (flux_r_UV / flux_t_UV / flux_p_UV, Src/globals.h:191-210). */
/* Tabulated force multiplier (read_sirocco_fluxes with KRAD = ALPHARAD =
 * 999, Src/LineDriven/line_connect.c:182-257): t at npoints and the cells'
 * M, [point][k][j][i] over the total box, as the file holds them (their
 * log10 is kept). */
void    or_set_mfit(or_sim *s, int npoints, const double *t_fit, const double *m_fit);
void    or_set_flux(or_sim *s, int nangles, const double *fr, const double *ft,
                    const double *fp);

/* Run `nsteps` steps of the main loop (Src/main.c:215-337 semantics).
 * Returns 0 on success, 1 if dt became too small (NextTimeStep abort),
 * 2 if a ConsToPrim failure flag was raised, 3 if dv/ds became NaN
 * (the reference exits there). */
int     or_run(or_sim *s, int nsteps);

void    or_time(const or_sim *s, double *t, double *dt, long *step);
void    or_set_time(or_sim *s, double t, double dt, long step);

/* Per-step record of the last or_run: dt used by each step and the
 * invDt_hyp the stage-1 reduction produced.  Returns count copied. */
int     or_history(const or_sim *s, double *dt_used, double *inv_dt, int max);

/* One BLONDIN cooling pass over the active cells with the given dt and
 * simulation time (BlondinCooling, Src/Cooling/BLONDIN/cooling.c:50-165). */
void    or_cooling(or_sim *s, double dt, double t);
double  or_blondin_point(double nH, double T, double xi, double tx, double dt_s, double mu);

/* Frozen ionisation parameter and radiation temperature per cell
 * ([k][j][i], total box). */
const double *or_sirocco_xi(const or_sim *s);
void    or_set_sirocco(or_sim *s, const double *xi, const double *t_r, const double *pre);

#ifdef __cplusplus
}
#endif
#endif
