// ps_probe.cu -- measurement helpers kept out of the product library
// (built into libps_probe.so, used by bench.py and the tests only):
//   ps_probe_fp64_flops  FP64 issue-rate probe, the denominator of the FP64
//                        roofline: independent chains of dependent
//                        double-precision FMAs in registers, many warps per
//                        SM, no memory traffic;
//   ps_probe_fastmath    the table-driven exp / log of the stage kernels
//                        (csrc/ps_fastmath.cuh) next to CUDA's on the same
//                        arguments, for the accuracy test;
//   ps_probe_fp64_lanes  the time of dependent FP64 FMAs in warps with only
//                        some lanes active (how the cost of a double-
//                        precision instruction depends on the active lanes,
//                        for the kernels that run few cells per warp);
//   ps_probe_wait_timeout
//                        the bounded mbarrier wait of the stage and learned-
//                        step kernels (ps_tma.cuh) on a barrier that nothing
//                        completes: it must give up after its poll limit and
//                        report, leaving the context usable (the failure test
//                        of a wait, without a GPU fault).
#include "ps_fastmath.cuh"
#include "ps_tma.cuh"

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

// `chains` (1..8) dependent FMA chains per active lane; lanes >= active
// of every warp return at once
__global__ void k_fp64_lanes(double *out, int active, int chains, int iters, double a, double b)
{
  if ((int)(threadIdx.x & 31) >= active) return;
  double x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; c++) x[c] = (double)(threadIdx.x + c) * 1e-3;
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int c = 0; c < kChains; c++)
      if (c < chains) x[c] = fma(x[c], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; c++) s += x[c];
  if (s == 12345.678) out[0] = s;
}

// One CTA: an mbarrier for one arrival; with `arrive` the barrier's phase
// is completed first (arrival with no transaction bytes), otherwise nothing
// completes it.  out[0] = 1 if every thread's bounded wait saw the phase
// complete, 0 if they gave up after `limit` polls.
__global__ void k_wait_timeout(int limit, int arrive, int *out)
{
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    if (arrive) mbar_expect_tx(&bar, 0);
  }
  __syncthreads();
  const bool ok = mbar_wait_bounded(&bar, 0, (uint32_t)limit);
  const int all = __syncthreads_and(ok);
  if (threadIdx.x == 0) out[0] = all ? 1 : 0;
}

__global__ void k_fastmath(int op, const double *x, double *fast, double *ref, long n)
{
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x) {
    const double v = x[i];
    fast[i] = op == 0 ? fm::exp(v) : fm::log(v);
    ref[i] = op == 0 ? ::exp(v) : ::log(v);
  }
}

}  // namespace ps

// op 0: exp, 1: log.  x, fast and ref are host arrays of n doubles; returns
// 0 or -1 on a CUDA error.
extern "C" int ps_probe_fastmath(int op, const double *x, double *fast, double *ref, long n)
{
  if (n <= 0 || (op != 0 && op != 1)) return -1;
  double *d = nullptr;
  const size_t bytes = (size_t)n * sizeof(double);
  if (cudaMalloc(&d, 3 * bytes) != cudaSuccess) return -1;
  cudaError_t e = cudaMemcpy(d, x, bytes, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    ps::k_fastmath<<<1024, 256>>>(op, d, d + n, d + 2 * n, n);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(fast, d + n, bytes, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(ref, d + 2 * n, bytes, cudaMemcpyDeviceToHost);
  cudaFree(d);
  return e == cudaSuccess ? 0 : -1;
}

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

// Milliseconds of `iters` steps of `chains` dependent FMA chains on `blocks`
// CTAs of `warps` warps with `active` lanes of each warp running (best of
// 3 after one warm-up); -1 on a bad argument or a CUDA error.
extern "C" double ps_probe_fp64_lanes(int active, int chains, int blocks, int warps, int iters)
{
  if (active < 1 || active > 32 || chains < 1 || chains > ps::kChains || blocks < 1 ||
      blocks > 65535 || warps < 1 || warps > 32 || iters < 1)
    return -1.0;
  double *out = nullptr;
  if (cudaMalloc(&out, sizeof(double)) != cudaSuccess) return -1.0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  ps::k_fp64_lanes<<<blocks, 32 * warps>>>(out, active, chains, 16, 0.999999, 1e-9);
  float best = -1.f;
  for (int r = 0; r < 3; r++) {
    cudaEventRecord(e0);
    ps::k_fp64_lanes<<<blocks, 32 * warps>>>(out, active, chains, iters, 0.999999, 1e-9);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (best < 0.f || ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (cudaGetLastError() != cudaSuccess) return -1.0;
  return best;
}

// The bounded wait (see k_wait_timeout) with a poll limit of `limit`
// (1..65536): *completed = 1 if the wait saw the barrier complete, 0 if it
// gave up.  Returns 0, or -1 on a bad argument or a CUDA error.
extern "C" int ps_probe_wait_timeout(int limit, int arrive, int *completed)
{
  if (limit < 1 || limit > 65536 || !completed) return -1;
  int *d = nullptr;
  if (cudaMalloc(&d, sizeof(int)) != cudaSuccess) return -1;
  cudaError_t e = cudaMemset(d, 0xFF, sizeof(int));
  if (e == cudaSuccess) {
    ps::k_wait_timeout<<<1, 128>>>(limit, arrive, d);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(completed, d, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(d);
  return e == cudaSuccess ? 0 : -1;
}
