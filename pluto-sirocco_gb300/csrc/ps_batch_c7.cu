// ps_batch_c7.cu -- the batch's stage kernels with characteristic limiting
// for the 7-variable state of ENTROPY_SWITCH contexts (the production
// numerics), compiled apart so that the kernel sets build in parallel.
#include "ps_batch_dev.cuh"

namespace ps {

const void *batch_kernel_c7(int shape, int lim, int solver, int stage)
{
  return batch_kernel_nv<7, true>(shape, lim, solver, stage);
}

}  // namespace ps
