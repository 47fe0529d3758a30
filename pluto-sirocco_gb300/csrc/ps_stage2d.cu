// ps_stage2d.cu -- instantiations of the fused stage kernel for
// DIMENSIONS == 2 (one translation unit per dimensionality so that the
// build compiles them in parallel).
#include "ps_stage.cuh"

namespace ps {

template <int NV, int LIM, int SOLVER>
static const void *pick_2d(int stage)
{
  return stage == 1 ? reinterpret_cast<const void *>(&k_stage<2, NV, LIM, SOLVER, 1>)
                    : reinterpret_cast<const void *>(&k_stage<2, NV, LIM, SOLVER, 2>);
}

template <int NV>
static const void *pick_nv_2d(int lim, int solver, int stage)
{
  if (solver == HLL) {
    if (lim == LIM_VL) return pick_2d<NV, LIM_VL, HLL>(stage);
    if (lim == LIM_MM) return pick_2d<NV, LIM_MM, HLL>(stage);
    return pick_2d<NV, LIM_MC, HLL>(stage);
  }
  if (lim == LIM_VL) return pick_2d<NV, LIM_VL, HLLC>(stage);
  if (lim == LIM_MM) return pick_2d<NV, LIM_MM, HLLC>(stage);
  return pick_2d<NV, LIM_MC, HLLC>(stage);
}

const void *stage_kernel_2d(int nv, int lim, int solver, int stage)
{
  if (nv == 5) return pick_nv_2d<5>(lim, solver, stage);
  if (nv == 6) return pick_nv_2d<6>(lim, solver, stage);
  return nullptr;
}

size_t stage_smem_2d(int nv)
{
  return nv == 5 ? stage_smem_bytes<5, TileT<2>>() : stage_smem_bytes<6, TileT<2>>();
}

void stage_tile_2d(int *t)
{
  t[0] = TileT<2>::X; t[1] = TileT<2>::Y; t[2] = TileT<2>::Z;
  t[3] = TileT<2>::HX; t[4] = TileT<2>::HY; t[5] = TileT<2>::HZ;
}

void fill_ghosts_2d(double *V, const Params &p, cudaStream_t s)
{
  const long long n = (long long)p.nx[0] * p.nx[1] * p.nx[2];
  int blocks = (int)((n + 255) / 256);
  if (blocks > 4096) blocks = 4096;
  if (p.nvar == 5)
    k_fill_ghosts<2, 5><<<blocks, 256, 0, s>>>(V, p);
  else
    k_fill_ghosts<2, 6><<<blocks, 256, 0, s>>>(V, p);
}

}  // namespace ps
