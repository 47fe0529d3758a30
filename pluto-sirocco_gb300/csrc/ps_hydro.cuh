// ps_hydro.cuh -- device data structures shared by the hydro kernels and the
// C-ABI layer.
#pragma once

#include <cuda.h>
#include <cstdint>

namespace ps {

// Scalars of the main loop kept on the device so that a whole run can be
// replayed from a CUDA graph without host round trips
// (g_time, g_dt, g_stepNumber: Src/globals.h:104-110; timeStep:
// Src/structs.h:372-397).
struct Scalars {
  double t;            // g_time
  double dt;           // g_dt (for the step about to run)
  double inv_dt_hyp;   // Dts->invDt_hyp
  double dt_cool;      // Dts->dt_cool
  long long step;      // g_stepNumber
  int last;            // last step reached (tstop clamp)
  int done;            // no further steps run
  unsigned flags;      // accumulated F_* device flags
  int pad;
  unsigned long long cdt_bits;  // max over cells of C_dt (bit pattern, >= 0)
};

constexpr int kHist = 4096;  // per-step dt history kept on the device

struct Params {
  int dims, nvar, limiter, solver, cooling;
  int char_lim;           // PLM on characteristic variables (spherical path)
  int shock;              // MULTID shock flattening (spherical path)
  int entropy;            // ENTROPY_SWITCH: 0 NO, 1 SELECTIVE, 2 ALWAYS (entropy = last var)
  int nx[3], ntot[3], beg[3];
  int px;                 // row pitch of device arrays (elements)
  int xoff;               // column of cell i = 0 within a pitched row: 1 when the
                          // ghost count is odd (3 with MULTID), so that every stage
                          // tile's TMA load starts on a 16-byte boundary; else 0
  long long vstride;      // elements between variables
  int bc[6];
  double gamma, gmm1;
  double igmm1;           // 1 / (gamma - 1): p / (gamma - 1) as a product
  double cfl, cfl_max_var, tstop, first_dt;
};

// FlagShock runs at the start of a step for MULTID shock flattening and
// for ENTROPY_SWITCH SELECTIVE
__host__ __device__ inline bool needs_shock_flags(const Params &p)
{
  return p.shock || p.entropy == 1;
}

struct StageArgs {
  const double *Vn;       // V^n (stage 2 reads it at the own cell)
  double *Vout;           // stage 1: V*, stage 2: V^{n+1} (== Vn buffer)
  double *Us;             // stage-1 conservative state
  const double *dtdx[3];  // dt/dx per direction for the current dt
  const double *inv_dx[3];
  Scalars *sc;
  Params p;
};

struct FinishArgs {
  Scalars *sc;
  double *hist_dt;        // [kHist]
  double *dtdx[3];
  const double *dx[3];
  Params p;
  int mode;               // 0 begin only, 1 finish+begin, 2 finish (no dt update)
};

}  // namespace ps
