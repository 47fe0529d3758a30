// ps_probe.cu -- FP64 issue-rate probe used as the denominator of the FP64
// roofline: independent chains of dependent double-precision FMAs in
// registers, many warps per SM, no memory traffic.
#include "ps_gb300.h"

#include <cuda_runtime.h>

namespace ps {

constexpr int kChains = 8;

__global__ void k_fp64_fma_chains(double *out, int iters, double a, double b)
{
  double x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; c++) x[c] = (double)(threadIdx.x + c) * 1e-3;
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int c = 0; c < kChains; c++) x[c] = fma(x[c], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; c++) s += x[c];
  if (s == 12345.678) out[0] = s;  // keeps the chains live
}

}  // namespace ps

extern "C" void ps_set_error_msg(const char *msg);

// FP64 FLOP/s of the current device (2 flops per FMA), best of `reps`.
extern "C" double ps_probe_fp64_flops(int reps)
{
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1.0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  double *out = nullptr;
  if (cudaMalloc(&out, sizeof(double)) != cudaSuccess) return -1.0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int threads = 256, blocks = sms * 8, iters = 4096;
  ps::k_fp64_fma_chains<<<blocks, threads>>>(out, 64, 0.999999, 1e-9);  // warm-up
  double best = 0.0;
  for (int r = 0; r < (reps > 0 ? reps : 5); r++) {
    cudaEventRecord(e0);
    ps::k_fp64_fma_chains<<<blocks, threads>>>(out, iters, 0.999999, 1e-9);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    const double flops = 2.0 * ps::kChains * (double)iters * threads * blocks;
    const double rate = flops / (ms * 1e-3);
    if (rate > best) best = rate;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (cudaGetLastError() != cudaSuccess) return -1.0;
  return best;
}
