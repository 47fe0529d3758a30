// ps_batch6_s1.cu -- the batch's stage kernels of tile shape 1 for the
// 6-variable primitive-PLM state, in a translation unit of their own so that
// the shapes build in parallel.
#include "ps_batch_dev.cuh"

namespace ps {

const void *batch_kernel6_s1(int lim, int solver, int stage)
{
  return batch_kernel_s<6, false, 1>(lim, solver, stage);
}

}  // namespace ps
