// ps_batch7.cu -- the batch's stage kernels for the 7-variable state of
// ENTROPY_SWITCH contexts (rho, v1, v2, v3, p, tracer, entropy), compiled
// apart from the 6-variable set so that the two build in parallel.
#include "ps_batch_dev.cuh"

namespace ps {

const void *batch_kernel7(int shape, int lim, int solver, int stage)
{
  return batch_kernel_nv<7, false>(shape, lim, solver, stage);
}

size_t batch_smem7(int shape) { return batch_smem_nv<7>(shape); }

}  // namespace ps
