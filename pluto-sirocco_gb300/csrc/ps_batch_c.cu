// ps_batch_c.cu -- the batch's stage kernels with characteristic limiting
// (CHAR_LIMITING YES) for the 6-variable state, compiled apart so that the
// kernel sets build in parallel.
#include "ps_batch_dev.cuh"

namespace ps {

const void *batch_kernel_c6(int shape, int lim, int solver, int stage)
{
  return batch_kernel_nv<6, true>(shape, lim, solver, stage);
}

}  // namespace ps
