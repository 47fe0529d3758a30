// ps_finish.cuh -- end of one step and start of the next for one grid, run
// by one CTA: invDt_hyp from the stage-1 maximum of C_dt, g_time update,
// NextTimeStep (with the COOLING rule that dt is recomputed after odd steps
// only and invDt_hyp carries over the step pair), the tstop clamp, the
// resets of Integrate(), then dt/dx for the new dt.
//
// Reference (paths inside the reference project):
//   main loop / tstop clamp   Src/main.c:215-337
//   Integrate (resets)        Src/main.c:383-497
//   NextTimeStep              Src/main.c:521-697
//   invDt_hyp reduction       Src/Time_Stepping/update_stage.c:389-394
#pragma once

#include "ps_hydro.cuh"
#include "ps_physics.cuh"

namespace ps {

enum { MODE_BEGIN = 0, MODE_STEP = 1, MODE_INV = 2, MODE_PREP = 3 };

__device__ __forceinline__ void finish_block(const FinishArgs &f)
{
  __shared__ double s_dt;
  __shared__ int s_run;
  if (threadIdx.x == 0) {
    Scalars *sc = f.sc;
    const Params &p = f.p;
    if (!sc->done && (f.mode == MODE_STEP || f.mode == MODE_INV)) {
      const double maxc = __longlong_as_double((long long)sc->cdt_bits);
      double inv = dmax(sc->inv_dt_hyp, maxc);
      inv /= (double)(p.dims);
      sc->inv_dt_hyp = inv;
      const long long n = sc->step;
      if (f.hist_dt && n >= 0 && n < kHist) f.hist_dt[n] = sc->dt;
      if (f.mode == MODE_STEP) {
        sc->t += sc->dt;
        if (!p.cooling || n % 2 == 1) {
          double dt_hyp = 1.0 / sc->inv_dt_hyp;
          dt_hyp *= p.cfl;
          double dtnext = dt_hyp;
          if (p.cooling) dtnext = dmin(dtnext, sc->dt_cool);
          dtnext = dmin(dtnext, p.cfl_max_var * sc->dt);
          if (dtnext < p.first_dt * 1.e-9) {
            sc->flags |= F_DT_SMALL;
            sc->done = 1;
          } else if (p.cfl_max_var != 1.0) {
            sc->dt = dtnext;
          }
        }
        sc->step = n + 1;
        if (sc->last) sc->done = 1;
      }
    }
    if (!sc->done && (f.mode == MODE_BEGIN || f.mode == MODE_STEP)) {
      if ((sc->t + sc->dt) >= p.tstop * (1.0 - 1.e-8)) {
        sc->dt = p.tstop - sc->t;
        sc->last = 1;
      }
      const long long n = sc->step;
      if (!p.cooling || (n - 1) % 2 == 1) {
        sc->inv_dt_hyp = 0.0;
        sc->dt_cool = 1.e38;
      }
    }
    if (f.mode != MODE_INV) sc->cdt_bits = 0ull;
    s_dt = sc->dt;
    s_run = !sc->done && f.mode != MODE_INV;
  }
  __syncthreads();
  if (!s_run) return;
  for (int d = 0; d < f.p.dims; d++)
    for (int i = threadIdx.x; i < f.p.ntot[d]; i += blockDim.x)
      f.dtdx[d][i] = s_dt / f.dx[d][i];
}

}  // namespace ps
