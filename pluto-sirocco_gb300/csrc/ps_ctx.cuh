// ps_ctx.cuh -- the device context behind the opaque ps_ctx handle of the
// C ABI (shared by ps_api.cu and ps_wind.cu).
#pragma once

#include "ps_gb300.h"
#include "ps_hydro.cuh"
#include "ps_wind.cuh"

#include <cuda.h>
#include <cuda_runtime.h>

namespace ps {
struct WindDev;
}

struct ps_ctx {
  ps_config cfg;
  ps::Params p;
  int tile[6];
  dim3 grid, block;
  size_t smem;
  const void *k1, *k2;
  double *V, *Vs, *Us;
  double *Vsave;            // device checkpoint of V (ps_save_state)
  ps::Scalars *sc_save;
  double *dx[3], *inv_dx[3], *dtdx[3];
  double *hx[3], *hxl[3], *hxr[3], *hdx[3];  // host copies of the grid
  ps::Scalars *sc;
  double *hist;
  CUtensorMap tmV, tmVs;
  cudaStream_t stream;      // stream the work is issued on
  cudaStream_t own_stream;  // stream created by the context
  cudaGraphExec_t g1, gN;
  cudaGraphExec_t gw[3];    // wind: even step, odd step, step pair
  int nG;
  long launches;
  int grid_mask;
  long long host_step;      // host mirror of g_stepNumber (wind graph parity)
  long long host_step_save; // host_step at ps_save_state
  ps::WindDev *wind;        // line-driven wind terms (NULL for plain hydro)
  int cool_on;              // Cartesian BLONDIN at constant xi (ps_set_cooling)
  ps::WindParams coolw;     // its units and parameters
  struct ps_surrogate *sg;  // learned cooling step (NULL: reference BLONDIN)
  int sg_use_net;           // 0: Newton from the old temperature (no network)
  void *sg_queue;           // cells left to the reference method (int2 each)
  int *sg_qcount;
  void *sg_items;           // (0, block) work items of the surrogate kernel
};
