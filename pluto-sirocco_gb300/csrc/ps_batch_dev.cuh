// ps_batch_dev.cuh -- device side of the batch of wind models: the
// per-model descriptor table entry, the work items of the stage kernels,
// the stage kernel itself and its tables over the tile shapes the
// autotuner chooses from (instantiated per variable count in ps_batch.cu
// and ps_batch7.cu).
#pragma once

#include "ps_finish.cuh"
#include "ps_wind_dev.cuh"

#include <cudaTypedefs.h>

#include <type_traits>

namespace ps {

struct BatchModel {
  CUtensorMap tm[2];     // V (stage-1 input) and V* (stage-2 input), tile box of the model
  WindStageArgs st[2];   // stage 1 and stage 2 arguments
  FinishArgs fin;        // dt kernel arguments (MODE_STEP)
};

struct TileItem {
  int m, bx, by, pad;
};

__device__ __forceinline__ void tensormap_acquire(const CUtensorMap *tm)
{
  asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(tm) : "memory");
}

template <int NV, int LIM, int SOLVER, int STAGE, class TL, bool CHAR>
__global__ void __launch_bounds__(TileGeom<TL>::NT, TileMinBlocks<TL>::value)
    k_batch_stage(const BatchModel *__restrict__ models, const TileItem *__restrict__ items)
{
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const TileItem it = items[blockIdx.x];
  const BatchModel &M = models[it.m];
  const CUtensorMap *tm = &M.tm[STAGE - 1];
  if (threadIdx.x == 0) tensormap_acquire(tm);
  stage_sph_tile<NV, LIM, SOLVER, STAGE, TL, CHAR>(tm, M.st[STAGE - 1], it.bx, it.by, smem_raw);
}

// ------------------------------------------------------------------
// kernel tables for the tile shapes the autotuner chooses from
// ------------------------------------------------------------------

constexpr int kNumShapes = 7;
const int kShapeX[kNumShapes] = {32, 16, 64, 16, 16, 32, 32};
const int kShapeY[kNumShapes] = {8, 16, 4, 16, 16, 8, 16};
// threads per CTA: one per cell, plus one warp for the halo work of the
// 16x16 tile's PLM (18 x 16 items) in shapes 3 and 4, and two for the 32x16
// tile's (34 x 16 and 32 x 18 items) in shape 6
const int kShapeNT[kNumShapes] = {256, 256, 256, 288, 288, 256, 576};
using Shape3 = Tile2D<16, 16, 32>;
// Shape 6: 32x16, one CTA per multiprocessor; PLM recomputes 6% (x) and
// 12.5% (y) of its cells in the halo and the Riemann solver 3% and 6% of
// its faces, against 12.5% and 6% in both directions for 16x16
using Shape6 = Tile2D<32, 16, 64>;
// Shapes 4 and 5: shapes 3 and 0 compiled for more CTAs per multiprocessor:
// three (at most 72 / 80 registers, with some spilling) instead of two for
// the primitive-PLM 6-variable kernels, two (at most 112 / 128 registers)
// instead of one for the others, whose natural register count (about 130
// with characteristic limiting) leaves one CTA per multiprocessor.
template <int NV, bool CHAR> struct Shape4 {
  using T = typename std::conditional<NV == 6 && !CHAR, Tile2D<16, 16, 32, 3>,
                                      Tile2D<16, 16, 32, 2>>::type;
};
template <int NV, bool CHAR> struct Shape5 {
  using T = typename std::conditional<NV == 6 && !CHAR, Tile2D<32, 8, 0, 3>,
                                      Tile2D<32, 8, 0, 2>>::type;
};

template <int NV, bool CHAR, int LIM, int SOLVER, class TL>
const void *pick_batch(int stage)
{
  return stage == 1
             ? reinterpret_cast<const void *>(&k_batch_stage<NV, LIM, SOLVER, 1, TL, CHAR>)
             : reinterpret_cast<const void *>(&k_batch_stage<NV, LIM, SOLVER, 2, TL, CHAR>);
}

template <int NV, bool CHAR, class TL>
const void *pick_batch_shape(int lim, int solver, int stage)
{
  if (solver == HLL) {
    if (lim == LIM_VL) return pick_batch<NV, CHAR, LIM_VL, HLL, TL>(stage);
    if (lim == LIM_MM) return pick_batch<NV, CHAR, LIM_MM, HLL, TL>(stage);
    return pick_batch<NV, CHAR, LIM_MC, HLL, TL>(stage);
  }
  if (lim == LIM_VL) return pick_batch<NV, CHAR, LIM_VL, HLLC, TL>(stage);
  if (lim == LIM_MM) return pick_batch<NV, CHAR, LIM_MM, HLLC, TL>(stage);
  return pick_batch<NV, CHAR, LIM_MC, HLLC, TL>(stage);
}

// One tile shape's kernels (CHAR: CHAR_LIMITING YES)
template <int NV, bool CHAR, int S>
const void *batch_kernel_s(int lim, int solver, int stage)
{
  if constexpr (S == 1) return pick_batch_shape<NV, CHAR, Tile2D<16, 16>>(lim, solver, stage);
  else if constexpr (S == 2) return pick_batch_shape<NV, CHAR, Tile2D<64, 4>>(lim, solver, stage);
  else if constexpr (S == 3) return pick_batch_shape<NV, CHAR, Shape3>(lim, solver, stage);
  else if constexpr (S == 4)
    return pick_batch_shape<NV, CHAR, typename Shape4<NV, CHAR>::T>(lim, solver, stage);
  else if constexpr (S == 5)
    return pick_batch_shape<NV, CHAR, typename Shape5<NV, CHAR>::T>(lim, solver, stage);
  else if constexpr (S == 6) return pick_batch_shape<NV, CHAR, Shape6>(lim, solver, stage);
  else return pick_batch_shape<NV, CHAR, Tile2D<32, 8>>(lim, solver, stage);
}

template <int NV, bool CHAR>
const void *batch_kernel_nv(int shape, int lim, int solver, int stage)
{
  switch (shape) {
    case 1: return batch_kernel_s<NV, CHAR, 1>(lim, solver, stage);
    case 2: return batch_kernel_s<NV, CHAR, 2>(lim, solver, stage);
    case 3: return batch_kernel_s<NV, CHAR, 3>(lim, solver, stage);
    case 4: return batch_kernel_s<NV, CHAR, 4>(lim, solver, stage);
    case 5: return batch_kernel_s<NV, CHAR, 5>(lim, solver, stage);
    case 6: return batch_kernel_s<NV, CHAR, 6>(lim, solver, stage);
    default: return batch_kernel_s<NV, CHAR, 0>(lim, solver, stage);
  }
}

template <int NV>
size_t batch_smem_nv(int shape)
{
  switch (shape) {
    case 1: return stage_smem_bytes<NV, Tile2D<16, 16>>();
    case 2: return stage_smem_bytes<NV, Tile2D<64, 4>>();
    case 3:
    case 4: return stage_smem_bytes<NV, Shape3>();
    case 6: return stage_smem_bytes<NV, Shape6>();
    default: return stage_smem_bytes<NV, Tile2D<32, 8>>();
  }
}

}  // namespace ps
