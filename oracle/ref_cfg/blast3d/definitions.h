/* Problem configuration for the reference CPU build of the 2-D Cartesian
   ideal-gas blast wave (PLM + MC limiter, HLLC, RK2, outflow).
   Test infrastructure only: compiled by oracle/Makefile into oracle/_ref. */
#define  PHYSICS                        HD
#define  DIMENSIONS                     3
#define  GEOMETRY                       CARTESIAN
#define  BODY_FORCE                     NO
#define  COOLING                        NO
#define  RECONSTRUCTION                 LINEAR
#define  TIME_STEPPING                  RK2
#define  NTRACER                        0
#define  PARTICLES                      NO
#define  USER_DEF_PARAMETERS            4
#define  LINE_DRIVEN_WIND               NO

/* -- physics dependent declarations -- */

#define  DUST_FLUID                     NO
#define  EOS                            IDEAL
#define  ENTROPY_SWITCH                 NO
#define  INCLUDE_LES                    NO
#define  THERMAL_CONDUCTION             NO
#define  VISCOSITY                      NO
#define  RADIATION                      NO
#define  ROTATING_FRAME                 NO

/* -- user-defined parameters (labels) -- */

#define  P_AMB                          0
#define  P_IN                           1
#define  R_IN                           2
#define  NOISE                          3

/* [Beg] user-defined constants (do not change this line) */

#define  LIMITER                        MC_LIM
#define  WARNING_MESSAGES               NO
#define  SHOW_TIME_STEPS                NO
#define  PRNG                           PRNG_MT

/* [End] user-defined constants (do not change this line) */
