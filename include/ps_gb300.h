/* ps_gb300.h -- C ABI of the GB300 (sm_103a) implementation of the
 * PLUTO-sirocco per-step hydro path.
 *
 * Plain C types only (ints, doubles, pointers and sizes).  A PLUTO build
 * binds these entry points from its own C host code in place of the
 * functions named beside each declaration (paths inside the reference
 * project); the array arguments are the very arrays PLUTO allocates:
 *   Vc        Data.Vc, primitive variables [nv][k][j][i] over the total box
 *             (ghost zones included), one contiguous block as made by
 *             ARRAY_4D (Src/structs.h:526, Src/arrays.c:250-300)
 *   x/xl/xr/dx Grid.x / Grid.xl / Grid.xr / Grid.dx per direction over the
 *             total box (Src/structs.h:133-187)
 *
 * Return convention: 0 on success; a negative PS_E* code for a host-side
 * error (see ps_last_error()); a positive value is the OR of PS_F* flags
 * raised by the device during the call.
 */
#ifndef PS_GB300_H
#define PS_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* geometry, limiter, solver and boundary codes (Src/pluto.h:163-171) */
#define PS_CARTESIAN      0
#define PS_SPHERICAL      3
#define PS_LIM_MC         0
#define PS_LIM_VL         1
#define PS_LIM_MM         2
#define PS_HLLC           0
#define PS_HLL            1
#define PS_BC_OUTFLOW     1
#define PS_BC_REFLECTIVE  2
#define PS_BC_AXISYM      3
#define PS_BC_EQTSYM      4
#define PS_BC_PERIODIC    5
#define PS_BC_USERDEF     8
#define PS_GRID_UNIFORM   0
#define PS_GRID_LOG_INC   1
#define PS_GRID_RATIO     2

/* host-side error codes */
#define PS_EINVAL   (-1)
#define PS_ECUDA    (-2)
#define PS_ENOMEM   (-3)
#define PS_ESTATE   (-4)

/* device flags (positive return values) */
#define PS_F_NAN          0x01  /* NaN in the state (Src/debug_tools.c:13-38)   */
#define PS_F_CONS2PRIM    0x02  /* FLAG_CONS2PRIM_FAIL (Src/HD/mappers.c:139-200) */
#define PS_F_NEG_DENSITY  0x04  /* FLAG_NEGATIVE_DENSITY                          */
#define PS_F_DT_SMALL     0x08  /* dt too small (Src/main.c:672-683)              */
#define PS_F_TMA_TIMEOUT  0x10  /* a bounded wait on a tile copy ran out          */
#define PS_F_COOLING      0x20  /* the ODE cooling path failed in a cell: NaN
                                   temperature or more than 1000 substeps
                                   (QUIT_PLUTO in Src/Cooling/cooling_ode_solver.c) */

typedef struct ps_config {
  int    dims;         /* DIMENSIONS: 2 or 3                                  */
  int    nx[3];        /* active cells per direction (1 when inactive)        */
  int    nvar;         /* NVAR: 5 (rho, vx1, vx2, vx3, prs) + passive scalars */
  int    geometry;     /* GEOMETRY: PS_CARTESIAN                              */
  int    limiter;      /* LIMITER: PS_LIM_*                                   */
  int    solver;       /* [Solver] Solver: PS_HLLC / PS_HLL                   */
  int    bc[6];        /* [Boundary] X1-beg, X1-end, X2-beg, ... : PS_BC_*    */
  double gamma;        /* g_gamma                                             */
  double cfl;          /* [Time] CFL                                          */
  double cfl_max_var;  /* [Time] CFL_max_var                                  */
  double tstop;        /* [Time] tstop                                        */
  double first_dt;     /* [Time] first_dt                                     */
  int    cooling;      /* COOLING: 0 NO; 1 BLONDIN (split implicit solve);
                           2 the ODE path of the production wind (COOLING
                           TABULATED with its CoolingSource and Radiat:
                           BLONDIN rates integrated by RKF12 / Cash-Karp,
                           sets dt_cool; spherical contexts).  With cooling,
                           dt is recomputed after odd steps only          */
  int    char_limiting; /* CHAR_LIMITING YES: PLM on characteristic variables
                           (Src/States/plm_states.c:481-746; spherical
                           contexts)                                      */
  int    shock_flattening; /* SHOCK_FLATTENING MULTID: minmod reconstruction
                           in and next to shocked zones, HLL next to them
                           with HLLC (Src/flag_shock.c:81-250; spherical
                           contexts).  Such contexts carry 3 ghost zones
                           per side instead of 2 (Src/get_nghost.c)       */
  int    entropy_switch; /* ENTROPY_SWITCH: 0 NO, 1 SELECTIVE, 2 ALWAYS.
                           The entropy s = p / rho^gamma is the last of the
                           nvar variables (nvar = 7 for the wind); pressure
                           is recovered from rho s in the tagged zones
                           (Src/HD/mappers.c:185-221; spherical contexts) */
} ps_config;

/* Ghost zones per side of an active direction: PS_NGHOST(cfg) */
#define PS_NGHOST(cfg) ((cfg)->shock_flattening ? 3 : 2)

typedef struct ps_ctx ps_ctx;

/* Line-driven disk wind terms of a 2-D spherical context: units
 * (definitions.h UNIT_*), the [Parameters] of the sirocco wind problem,
 * and which source terms are on. */
typedef struct ps_wind {
  double unit_density, unit_length, unit_velocity;
  double mu;           /* MU: mean molecular weight                        */
  double rho_0;        /* RHO_0: disk-plane density [g cm^-3]              */
  double cent_mass;    /* CENT_MASS: central point mass [g]                 */
  double t_iso;        /* T_ISO: initial isothermal temperature [K]        */
  double l_star;       /* L_star [erg s^-1]                                 */
  double frac_x, frac_uv; /* X-ray and UV fractions of L_star (the problem's
                          f_x, f_uv parameters)                          */
  double t_x;          /* T_x: X-ray (Compton) temperature [K]              */
  double krad, alpharad; /* force multiplier M = krad * t^alpharad          */
  double dfloor;       /* DFLOOR: density floor [g cm^-3]                   */
  int    body_force;   /* BodyForceVector: point-mass gravity               */
  int    line_force;   /* VGradCalc + LineForce                             */
  int    floors;       /* UserDefBoundary(side 0) density/pressure floors   */
  int    nangles;      /* NFLUX_ANGLES (36 for SIROCCO), at most 64         */
} ps_wind;

const char *ps_last_error(void);

/* ---------------------------------------------------------------- */
/* host helpers (no device needed)                                   */
/* ---------------------------------------------------------------- */

/* One direction of the grid over the total box: n active cells between
 * xbeg and xend plus ngh ghost cells on each side, as SetGrid builds it
 * (Src/set_grid.c:100-140 for ghosts and centres, 405-450 for the
 * uniform, logarithmic "l+" and ratio "r" patches).  Arrays hold n+2*ngh
 * entries. */
int ps_grid_build(int type, int n, int ngh, double xbeg, double xend,
                  double ratio, double *x, double *xl, double *xr, double *dx);

/* Blast-wave initial condition used by the 2-D/3-D Cartesian tests and
 * benchmark: rho = 1*(1 + U(-noise, noise)) from PLUTO's PRNG_MT sequence
 * (RandomSeed(seed, 0) / RandomNumber, Src/Math_Tools/math_random.c:36-183)
 * drawn over the active cells in (k, j, i) order; v = 0; p = p_in where
 * the distance from the box centre (0.5, 0.5[, 0.5]) is below r_in,
 * p_amb elsewhere.  Ghost cells are set to the ambient state.  x1..x3 are
 * the cell-centre arrays of the total box; Vc is [nv][k][j][i]. */
int ps_init_blast(const ps_config *cfg, const double *x1, const double *x2,
                  const double *x3, double p_amb, double p_in, double r_in,
                  double noise, long seed, double *Vc);

/* Initial condition of the line-driven disk wind on a 2-D spherical grid:
 * Init() evaluated on every cell of the total box at the volume centroids
 * (Src/startup.c:70-100, Src/set_geometry.c:81-104): an isothermal
 * (t_iso) disk-plane layer rho_0 exp(-G M / (2 cs^2 r tan^2 theta)) above a
 * halo at dfloor, Keplerian v_phi, tracer 1 in the layer.  Grid arrays are
 * those of ps_grid_build for x1 and x2; Vc is [nv][j][i] with nv = 6. */
int ps_init_wind(const ps_config *cfg, const ps_wind *w, const double *x1,
                 const double *xl1, const double *xr1, const double *dx1,
                 const double *x2, const double *xl2, const double *xr2,
                 double *Vc);

/* Synthetic directional UV flux for the line force: l_star*f_uv/(4 pi r^2)
 * in the angle bin that contains the radial direction of each active cell
 * (bins (a + 1/2) 2 pi / 36 from the polar axis), zero elsewhere, rounded
 * through the 13-significant-digit text of the directional_flux_*.dat
 * files that read_sirocco_fluxes parses (Src/LineDriven/line_connect.c:
 * 84-165).  fr/ft/fp are [angle][j][i] over the total box. */
int ps_wind_synthetic_flux(const ps_config *cfg, const ps_wind *w,
                           const double *x1, const double *x2,
                           double *fr, double *ft, double *fp);

/* The same with flux in every bin, a stand-in for SIROCCO's fluxes (which
 * fill most bins): weight 1 in the radial bin, 0.05/(1 + |d|) d bins away,
 * split into (F_r, F_theta) by the cosine and sine of the bin's angle from
 * the radial one, rounded the same way. */
int ps_wind_synthetic_flux_dense(const ps_config *cfg, const ps_wind *w,
                                 const double *x1, const double *x2,
                                 double *fr, double *ft, double *fp);

/* Readers of the files a SIROCCO run hands to the wind problem
 * (Src/LineDriven/line_connect.c:43-497), host only.  Records are placed on
 * the 2-D spherical grid (x1, x2: cell-centre arrays of the total box, x1 in
 * code units) by their coordinates with the reference's tolerances, found by
 * binary search instead of the reference's scan of every cell; arrays are
 * [j][i] over the total box and cells without a record keep their values.
 *   ps_read_sirocco_fluxes: <dir>/directional_flux_{r,theta,phi}.dat into
 *     fr/ft/fp ([angle][j][i], at most max_angles planes); returns the
 *     number of angle bins (read_sirocco_fluxes).
 *   ps_read_sirocco_heatcool: py_heatcool.dat into xi and t_r with the
 *     reference's floors xi >= 1, t_r >= 1e3 K.
 *   ps_read_sirocco_prefactors: prefactors.dat into six arrays in the
 *     file's order comp_h, comp_c, xray_h, brem_c, line_c, xi_ion.
 *   ps_read_m_uv_fit: M_UV_data.dat, the force-multiplier table read when
 *     KRAD = ALPHARAD = 999 (line_connect.c:182-257), into t_fit (the
 *     table's t values) and m_fit ([point][j][i]), at most max_points
 *     points; returns the number of points.
 * *matched (may be NULL) gets the number of records placed. */
int ps_read_sirocco_fluxes(const ps_config *cfg, double unit_length, const double *x1,
                           const double *x2, const char *dir, int max_angles, double *fr,
                           double *ft, double *fp, long *matched);
int ps_read_sirocco_heatcool(const ps_config *cfg, double unit_length, const double *x1,
                             const double *x2, const char *path, double *xi, double *t_r,
                             long *matched);
int ps_read_sirocco_prefactors(const ps_config *cfg, double unit_length, const double *x1,
                               const double *x2, const char *path, double *pre, long *matched);
int ps_read_m_uv_fit(const ps_config *cfg, double unit_length, const double *x1,
                     const double *x2, const char *path, int max_points, double *t_fit,
                     double *m_fit, long *matched);

/* ---------------------------------------------------------------- */
/* device context                                                    */
/* ---------------------------------------------------------------- */

/* Allocates the device mirrors of Data.Vc and the stage scratch for one
 * grid on the current CUDA device (the device-side counterpart of
 * Initialize(), Src/initialize.c, and of the static scratch of
 * AdvanceStep/UpdateStage, Src/Time_Stepping/rk_step.c:78-101,
 * update_stage.c:85-95). */
int ps_create(const ps_config *cfg, ps_ctx **out);
int ps_destroy(ps_ctx *ctx);

/* Copies one direction of Grid (x, xl, xr, dx over the total box) to the
 * device; replaces the device side of SetGrid/SetGeometry. */
int ps_set_grid(ps_ctx *ctx, int dir, const double *x, const double *xl,
                const double *xr, const double *dx);

/* Host Data.Vc -> device (after Startup / restart / InitDomain), and
 * device -> host Data.Vc (before WriteData / Analysis / restart dumps). */
int ps_set_state(ps_ctx *ctx, const double *Vc);
int ps_get_state(ps_ctx *ctx, double *Vc);

/* Turns a 2-D spherical context into the line-driven disk wind: point-mass
 * gravity (BodyForceVector), the problem's UserDefBoundary (floors on every
 * cell; X1_BEG copies the first active cell with inflow only), VGradCalc +
 * LineForce with the fluxes flux_* ([angle][j][i] over the total box, i.e.
 * flux_r_UV / flux_t_UV / flux_p_UV of Src/globals.h:191-210), and the
 * BLONDIN split source when cfg.cooling is set.  Call after ps_set_grid and
 * ps_set_state: sirocco_xi and sirocco_t_r are initialised from the state
 * as read_sirocco_heatcool(flag = 0) does (line_connect.c:287-306). */
int ps_set_wind(ps_ctx *ctx, const ps_wind *w, const double *flux_r,
                const double *flux_t, const double *flux_p);

/* g_time, g_dt, g_stepNumber of the main loop (Src/globals.h:104-110). */
int ps_set_time(ps_ctx *ctx, double t, double dt, long step);
int ps_get_time(ps_ctx *ctx, double *t, double *dt, long *step,
                double *inv_dt_hyp);

/* AdvanceStep (Src/Time_Stepping/rk_step.c:29-384) for TIME_STEPPING RK2
 * with the given dt: V^n -> V^{n+1} on the device.  On return
 * *inv_dt_hyp holds Dts->invDt_hyp as UpdateStage leaves it
 * (update_stage.c:389-394), ready for PLUTO's own NextTimeStep(). */
int ps_advance_step(ps_ctx *ctx, double dt, double *inv_dt_hyp);

/* SplitSource (Src/split_source.c:28-79) with COOLING == BLONDIN: one
 * BlondinCooling pass (Src/Cooling/BLONDIN/cooling.c:50-165) over the
 * active cells with the given dt at simulation time t.  No-op without
 * cooling. */
int ps_split_source(ps_ctx *ctx, double dt, double t);

/* ps_split_source, and *dt_cool = the smallest cooling time step the cells
 * asked for in this pass (1e38 when none did: BLONDIN sets none; the ODE
 * path of cooling = 2 sets it, Src/Cooling/cooling_source.c), for the host's
 * Dts->dt_cool = MIN(Dts->dt_cool, *dt_cool), which NextTimeStep reads
 * (Src/main.c:644). */
int ps_split_source_dt(ps_ctx *ctx, double dt, double t, double *dt_cool);

/* The main loop of Src/main.c:215-337 (Integrate + NextTimeStep and the
 * tstop clamp) for nsteps steps, entirely on the device and replayed
 * from a captured CUDA graph; no host synchronisation between steps. */
int ps_run(ps_ctx *ctx, int nsteps);

/* Waits for the context's stream and returns the accumulated device
 * flags (PS_F_*), or a negative error. */
int ps_sync(ps_ctx *ctx);

/* Device address of the primitive state (pitched [nv][k][j][px]) and its
 * row pitch in elements, for callers that keep inputs resident. */
double *ps_device_state(ps_ctx *ctx, int *pitch_elems);

/* Number of kernels launched by this context since creation. */
long ps_launch_count(const ps_ctx *ctx);

/* dt used by each of the first `max` steps (indexed by g_stepNumber, up to
 * 4096), as recorded on the device; returns the count copied. */
int ps_get_dt_history(ps_ctx *ctx, double *out, int max);

/* Issue all further work of the context on `stream` (a cudaStream_t owned
 * by the caller; NULL restores the context's own stream).  No reference
 * counterpart: lets a host framework order the path with its own work. */
int ps_set_stream(ps_ctx *ctx, void *stream);

/* Operator-split BLONDIN heating/cooling on a Cartesian context (created
 * with cooling = 1) at a constant ionisation parameter: SplitSource with
 * BlondinCooling (Src/split_source.c:28-79,
 * Src/Cooling/BLONDIN/cooling.c:50-165, prefactors 1) with xi and T_x
 * fixed instead of read from sirocco_xi / sirocco_t_r.  ps_run then
 * alternates the source around the hydro step in PLUTO's Strang order,
 * and ps_split_source() runs it alone. */
typedef struct ps_cooling {
  double unit_density, unit_length, unit_velocity;  /* UNIT_* of definitions.h */
  double mu;      /* MU: mean molecular weight                           */
  double t_x;     /* T_x: X-ray (Compton) temperature [K]                */
  double xi;      /* ionisation parameter L_x / (n_H r^2), constant       */
} ps_cooling;
int ps_set_cooling(ps_ctx *ctx, const ps_cooling *c);

/* ---------------------------------------------------------------- */
/* batches of independent wind models                                */
/* ---------------------------------------------------------------- */

/* read_sirocco_heatcool with flag 1 (line_connect.c:267-497) on the
 * device: per-cell xi and radiation temperature (BLONDIN uses them once
 * g_time > 3) and the prefactors of the rates (six [j][i] arrays in the
 * prefactors.dat order; xi_ion is not used by BLONDIN).  NULL leaves a part
 * as it is; ps_set_wind starts from xi and T_x of the state and prefactors
 * 1.  Call before ps_batch_create for contexts that go into a batch.  The
 * learned cooling step leaves cells whose prefactors are not 1 to the
 * reference method. */
int ps_set_sirocco(ps_ctx *ctx, const double *xi, const double *t_r, const double *pre);

/* The tabulated force multiplier of a wind whose KRAD and ALPHARAD are both
 * 999 (read_sirocco_fluxes, line_connect.c:182-257; LineForce with
 * linterp, 858-887): the table's t values (npoints) and every cell's M
 * ([point][j][i] over the total box), as M_UV_data.dat holds them
 * (ps_read_m_uv_fit).  Such a wind does not step before this is called.
 * Call before ps_batch_create for contexts that go into a batch. */
int ps_set_mfit(ps_ctx *ctx, int npoints, const double *t_fit, const double *m_fit);

/* No reference counterpart (the reference runs one model per process).
 * Advances n independent line-driven wind contexts (each already set up
 * with ps_set_grid, ps_set_state, ps_set_time and ps_set_wind; uneven grid
 * sizes and parameters allowed; same limiter, solver, cooling switch and
 * step number) together: every phase of a step is one launch over all
 * models and each step is one CUDA-graph replay; every model keeps its
 * own dt (its own C_dt reduction and NextTimeStep).  Results are
 * identical to ps_run on each context.  The contexts stay owned by the
 * caller and must outlive the batch. */
typedef struct ps_batch ps_batch;
int  ps_batch_create(ps_ctx **ctxs, int n, ps_batch **out);
int  ps_batch_destroy(ps_batch *b);
int  ps_batch_run(ps_batch *b, int nsteps);
int  ps_batch_sync(ps_batch *b);      /* OR of every model's PS_F_* flags */
/* Every model's Data.Vc to / from host arrays (Vc[m]: model m's
 * [nv][k][j][i] array over its total box), the copies queued together on
 * the batch's stream (get: then one synchronisation); the models' time
 * state is kept.  For hosts that hand the states in and out between steps. */
int  ps_batch_set_states(ps_batch *b, const double *const *Vc);
int  ps_batch_get_states(ps_batch *b, double *const *Vc);
/* The same transfers by the copy engines only, queued without waiting:
 * several batches on their own streams then overlap each batch's transfers
 * with the others' steps (four batches hide them on the benchmark batch,
 * two do not: both compute at once, then both copy).  The host arrays
 * (pinned) are in use until ps_batch_sync returns. */
int  ps_batch_set_states_async(ps_batch *b, const double *const *Vc);
int  ps_batch_get_states_async(ps_batch *b, double *const *Vc);
int  ps_batch_set_stream(ps_batch *b, void *stream);
/* The models are dealt out by size into ngroups groups (default 2, 1 for
 * a single model) whose
 * steps run as parallel branches of the step graph, so that one group's
 * short, latency-bound kernels can overlap the others' stage kernels.
 * Results do not depend on it. */
int  ps_batch_set_groups(ps_batch *b, int ngroups);
long ps_batch_launch_count(const ps_batch *b);
/* Tile shape of the stage kernels per model: 0 = 32x8, 1 = 16x16,
 * 2 = 64x4, 3 = 16x16 with one extra warp sharing the halo work, 4 and 5 =
 * shapes 3 and 0 compiled for three CTAs per multiprocessor instead of two,
 * 6 = 32x16 with two extra warps, one CTA per multiprocessor
 * (model = -1: all models).  ps_batch_autotune times the stage
 * kernel of every distinct grid size with each shape and keeps the fastest
 * (`reps` timed launches each); the state is left unchanged. */
int  ps_batch_set_shape(ps_batch *b, int model, int shape);
int  ps_batch_get_shape(const ps_batch *b, int model, int *tx, int *ty);
int  ps_batch_autotune(ps_batch *b, int reps);
/* One step launched kernel by kernel, timed with CUDA events: ms[0] the
 * stage-1 launches, ms[1] the stage-2 launches, ms[2] everything else. */
int  ps_batch_time_step_kernels(ps_batch *b, float ms[3]);

/* ---------------------------------------------------------------- */
/* learned cooling step (surrogate of BLONDIN)                       */
/* ---------------------------------------------------------------- */

/* No reference counterpart.  A 4 -> 64 -> 64 -> 1 SiLU network maps
 * (log10 n_H [cm^-3], log10 T [K], log10 xi, log10 dt [s]) to
 * log10 T_new of one BLONDIN solve (Src/Cooling/BLONDIN/cooling.c:50-165,
 * prefactors 1, T_x and mu fixed); it runs on the tensor cores (BF16
 * weights, FP32 accumulation).  Per cell, FP64 Newton steps on BLONDIN's
 * implicit energy equation judge and polish the result: a cell whose
 * residual at the old temperature is already within 1e-3 of its thermal
 * energy takes one Newton step from there; a stiff cell iterates from the
 * network's prediction (at most 5 net-rate evaluations in all); when the
 * net rate at the solution has changed sign, the equilibrium temperature
 * between the two is solved for, as the reference does.  A cell is left to
 * the reference method (bracket + Brent) when its inputs leave the box,
 * when the residual does not reach 1e-3, or when the energy equation is
 * not monotone there (thermally unstable cells).
 * Parameter vector (FP32, 4545 values): W1[64][4], b1[64], W2[64][64],
 * b2[64], w3[64], b3. */
typedef struct ps_surrogate ps_surrogate;
typedef struct {
  double lo[4], hi[4];   /* log10 bounds of n_H, T, xi, dt (the training box) */
  double t_x, mu;        /* X-ray temperature [K] and mean molecular weight */
} ps_sg_box;
enum { PS_SG_ACCEPT = 0, PS_SG_OUT_OF_BOX = 1, PS_SG_REJECT = 2, PS_SG_BELOW_MIN = 3 };

int ps_sg_create(const ps_sg_box *box, ps_surrogate **out);
int ps_sg_destroy(ps_surrogate *s);
int ps_sg_set_params(ps_surrogate *s, const float *params);
int ps_sg_get_params(const ps_surrogate *s, float *params);
/* A trained network (its box and parameters) to a file and back, so that a
 * run can use a network trained once (the drop-in reads the file named by
 * PS_LEARNED_COOLING).  Format: "PSSGNET1", lo[4], hi[4], t_x, mu (doubles),
 * the parameter count (int32, 4545), the parameters (float), little-endian.
 * ps_sg_load creates the surrogate; a file of another size or tag is
 * refused. */
int ps_sg_save(const ps_surrogate *s, const char *path);
int ps_sg_load(const char *path, ps_surrogate **out);
/* T_new of the reference method on the GPU for n tuples (row-major
 * n x 4: n_H, T, xi, dt [s]): the training labels.  t_cool (may be NULL)
 * gets the cooling time E / |net rate| at T in seconds. */
int ps_sg_label(ps_surrogate *s, const double *tuples, long n, double *t_new, double *t_cool);
/* Training set (tuples inside the box are used) and Adam training on the
 * GPU: `steps` minibatches of `batch` rows (multiple of 128), learning
 * rate cosine-decayed from lr to lr_end; loss_hist[steps] (may be NULL)
 * gets the mean squared error of (log10 T_new - log10 T) / 4 per step. */
int ps_sg_set_data(ps_surrogate *s, const double *tuples, const double *t_new, long n);
int ps_sg_train(ps_surrogate *s, int steps, int batch, float lr, float lr_end,
                unsigned long long seed, float *loss_hist);
/* Loss and gradient (4545 values, the parameter layout) of the mean
 * squared error over n tuples, without an update. */
int ps_sg_grad(ps_surrogate *s, const double *tuples, const double *t_new, int n,
               float *grad, float *loss);
/* The surrogate cooling step on n tuples: t_out (after the 1e4 K floor),
 * status (PS_SG_*), t_mlp (network prediction, may be NULL).  use_net = 0
 * starts the Newton steps from T instead of the prediction. */
int ps_sg_predict(ps_surrogate *s, const double *tuples, long n, int use_net,
                  double *t_out, int *status, double *t_mlp);
/* Counters since the last reset: cells accepted, out of box, rejected by
 * the judge, below 1e4 K; net-rate evaluations made by the judge; stiff
 * cells (not already within the residual at the old temperature). */
int ps_sg_stats(ps_surrogate *s, long long out[6], int reset);
/* Use the surrogate in the wind context's split-source step (NULL: the
 * reference method).  use_net as in ps_sg_predict. */
int ps_set_surrogate(ps_ctx *ctx, ps_surrogate *s, int use_net);
int ps_batch_set_surrogate(ps_batch *b, ps_surrogate *s, int use_net);
/* (n_H, T, xi, dt [s]) of every cell the next split-source step of the
 * wind context would solve (at most cap rows); *n = rows written. */
int ps_sg_collect(ps_ctx *ctx, double *tuples, long cap, long *n);

/* PLUTO's DBL snapshots of the device state: WriteData in single-file
 * mode (Src/write_data.c:132-220, Src/bin_io.c:216-258) writes
 * <dir>/data.<nfile>.dbl (every variable in Data.Vc order over the active
 * cells, x fastest, little-endian doubles) and the dbl.out line
 * "nfile t dt nstep single_file little <names>" (write_data.c:420-448),
 * keeping the first nfile lines of an existing dbl.out.  names may be NULL
 * (rho vx1 vx2 vx3 prs tr1 ...).  ps_read_dbl loads such a file into the
 * context (the .dbl part of RestartFromFile, Src/restart.c:104-170); the
 * time comes from restart.out on the host side (ps_set_time). */
int ps_write_dbl(ps_ctx *ctx, const char *dir, int nfile, const char *names);
int ps_read_dbl(ps_ctx *ctx, const char *path);

/* Device-side checkpoint / restore of Data.Vc and the main-loop scalars:
 * the backup that FAILSAFE keeps before a step (Src/failsafe.c:5-160),
 * held on the GPU so that a step can be retried or a run replayed. */
int ps_save_state(ps_ctx *ctx);
int ps_restore_state(ps_ctx *ctx);

/* Diagnostic with no reference counterpart: runs one step with a CUDA
 * event around each of its kernels; ms[0..2] = stage 1, stage 2 and the
 * dt kernel.  Advances the state by one step. */
int ps_time_step_kernels(ps_ctx *ctx, double *ms);

/* No counterpart in the reference.  ps_advance_step() for callers that
 * cannot allocate device memory: the caller owns the state (Vc_dev, a
 * device buffer laid out like Data.Vc, [nv][k][j][i] over the total box,
 * 16-byte aligned) and passes the host dx arrays of each direction; the
 * stage scratch comes from a fixed array inside the library (3.3 MB per
 * GPU, held until exit).  Limits: 32768 total-box cells per variable,
 * 6 variables, 2048 cells per direction, even total-box row length;
 * larger grids get PS_EINVAL, as do the characteristic-limiting,
 * shock-flattening and entropy-switch options (spherical wind contexts
 * only).  Calls that overlap on the GPU share the scratch and race.  The
 * first call on each device looks up the scratch address.  Every call
 * copies dx in and waits for its stream before returning, so it cannot be
 * called while that stream is being captured.  stream may be NULL. */
int ps_advance_step_noalloc(const ps_config *cfg, const double *dx1,
                            const double *dx2, const double *dx3,
                            double *Vc_dev, double dt, double *inv_dt_hyp,
                            void *stream);

#ifdef __cplusplus
}
#endif
#endif
