// ps_wind_kernels.cuh -- the single-model wind stage kernel (one CTA per
// 16x16 tile of one context, tensor map as a kernel parameter) and its table
// over limiter, solver and stage, instantiated per variable count and
// limiting form in ps_wind.cu and ps_wind_k.cu.
#pragma once

#include "ps_wind_dev.cuh"

namespace ps {

// The tile of the single-model wind kernels: 16x16 with a ninth warp for
// the halo work of PLM and Riemann, compiled for two CTAs per
// multiprocessor -- the shape the batch's autotuner keeps for every grid
// size, with the primitive limiter (96 registers) and with characteristic
// limiting (which otherwise takes about 130 registers and one CTA).
using WindTile = Tile2D<16, 16, 32, 2>;

template <int NV, int LIM, int SOLVER, int STAGE, bool CHAR>
__global__ void __launch_bounds__(TileGeom<WindTile>::NT, TileMinBlocks<WindTile>::value)
    k_stage_sph(const __grid_constant__ CUtensorMap tm, const WindStageArgs A)
{
  extern __shared__ __align__(128) unsigned char smem_raw[];
  stage_sph_tile<NV, LIM, SOLVER, STAGE, WindTile, CHAR>(&tm, A, blockIdx.x, blockIdx.y,
                                                         smem_raw);
}

template <int NV, bool CHAR, int LIM, int SOLVER>
const void *pick_sph(int stage)
{
  return stage == 1 ? reinterpret_cast<const void *>(&k_stage_sph<NV, LIM, SOLVER, 1, CHAR>)
                    : reinterpret_cast<const void *>(&k_stage_sph<NV, LIM, SOLVER, 2, CHAR>);
}

// nv 6: rho, v1, v2, v3, p, tracer; 7: and the entropy (ENTROPY_SWITCH);
// CHAR: CHAR_LIMITING YES
template <int NV, bool CHAR>
const void *stage_kernel_sph_nv(int lim, int solver, int stage)
{
  if (solver == HLL) {
    if (lim == LIM_VL) return pick_sph<NV, CHAR, LIM_VL, HLL>(stage);
    if (lim == LIM_MM) return pick_sph<NV, CHAR, LIM_MM, HLL>(stage);
    return pick_sph<NV, CHAR, LIM_MC, HLL>(stage);
  }
  if (lim == LIM_VL) return pick_sph<NV, CHAR, LIM_VL, HLLC>(stage);
  if (lim == LIM_MM) return pick_sph<NV, CHAR, LIM_MM, HLLC>(stage);
  return pick_sph<NV, CHAR, LIM_MC, HLLC>(stage);
}

}  // namespace ps
