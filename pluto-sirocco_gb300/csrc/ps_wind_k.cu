// ps_wind_k.cu -- the single-model wind stage kernels other than the
// primitive-PLM 6-variable set: characteristic limiting, and the 7-variable
// state of ENTROPY_SWITCH contexts (compiled apart so that the sets build in
// parallel).
#include "ps_wind_kernels.cuh"

namespace ps {

const void *stage_kernel_sph_other(int nv, bool ch, int lim, int solver, int stage)
{
  if (nv == 6) return stage_kernel_sph_nv<6, true>(lim, solver, stage);
  if (nv != 7) return nullptr;
  return ch ? stage_kernel_sph_nv<7, true>(lim, solver, stage)
            : stage_kernel_sph_nv<7, false>(lim, solver, stage);
}

}  // namespace ps
