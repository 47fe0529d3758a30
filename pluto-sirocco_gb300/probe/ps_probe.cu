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
//   ps_probe_dmul_rate   throughput of binary64 products on the FP64 unit,
//                        on the integer pipes (csrc/ps_dmul.cuh) and in
//                        mixes of the two;
//   ps_probe_dmul_check  the integer product against the hardware multiply,
//                        bit for bit, on the GPU or (the same code compiled
//                        for the host) against the host's multiply;
//   ps_probe_wait_timeout
//                        the bounded mbarrier wait of the stage and learned-
//                        step kernels (ps_tma.cuh) on a barrier that nothing
//                        completes: it must give up after its poll limit and
//                        report, leaving the context usable (the failure test
//                        of a wait, without a GPU fault).
#include "ps_dmul.cuh"
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

// `emul` of every 8 chains take the integer product, the others the FP64
// unit's; the multipliers alternate between m0 and m1 so that the chains
// stay near 1
template <int EMUL>
__global__ void k_dmul_rate(double *out, int iters, double m0, double m1)
{
  double x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; c++) x[c] = 1.0 + (double)(threadIdx.x + c) * 1e-6;
  bool bad = false;
  for (int it = 0; it < iters; it++) {
    const double m = (it & 1) ? m0 : m1;
#pragma unroll
    for (int c = 0; c < kChains; c++) x[c] = c < EMUL ? dmul_int(x[c], m, bad) : __dmul_rn(x[c], m);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; c++) s += x[c];
  if (s == 12345.678 || bad) out[0] = s;
}

// Operand pairs for the check, five kinds by i % 5: exponents near the
// middle of the range; short significands (exact products and exact ties);
// any bit pattern; products near either end of the normal range; zeros,
// powers of two and sign mixes.
__host__ __device__ __forceinline__ uint64_t dm_mix(uint64_t z)
{
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

__host__ __device__ __forceinline__ void dm_pair(uint64_t seed, long long i, uint64_t &A,
                                                 uint64_t &B)
{
  const uint64_t k0 = seed + 4ull * (uint64_t)i;
  A = dm_mix(k0);
  B = dm_mix(k0 + 1);
  const uint64_t r0 = dm_mix(k0 + 2), r1 = dm_mix(k0 + 3);
  const uint64_t SG = 0x8000000000000000ull, MT = 0x000fffffffffffffull;
  switch ((int)(i % 5)) {
    case 0:
      A = (A & (SG | MT)) | ((uint64_t)(923 + r0 % 200) << 52);
      B = (B & (SG | MT)) | ((uint64_t)(923 + r1 % 200) << 52);
      break;
    case 1: {
      const int ka = 1 + (int)(r0 % 53), kb = 1 + (int)((r0 >> 8) % 53);
      const uint64_t ma = ka == 1 ? 0 : (A & MT) >> (53 - ka) << (53 - ka);
      const uint64_t mb = kb == 1 ? 0 : (B & MT) >> (53 - kb) << (53 - kb);
      A = (A & SG) | ma | ((uint64_t)(993 + r1 % 60) << 52);
      B = (B & SG) | mb | ((uint64_t)(993 + (r1 >> 8) % 60) << 52);
      break;
    }
    case 2:
      break;
    case 3: {
      const int ea = (int)(r0 % 2048);
      const int target = (r1 & 1) ? 2042 + (int)((r1 >> 1) % 8) : -3 + (int)((r1 >> 1) % 8);
      int eb = target - ea + 1023;
      eb = eb < 0 ? 0 : (eb > 2047 ? 2047 : eb);
      A = (A & (SG | MT)) | ((uint64_t)ea << 52);
      B = (B & (SG | MT)) | ((uint64_t)eb << 52);
      break;
    }
    default: {
      const int k = (int)(r0 % 4);
      if (k == 0) A &= SG;
      else if (k == 1) B &= SG;
      else if (k == 2) A &= 0xfff0000000000000ull;
      break;
    }
  }
}

// cnt[0]: pairs whose integer product differs from the hardware's,
// cnt[1]: pairs handed back (bad); first[0..1]: the first differing pair
__global__ void k_dmul_check(uint64_t seed, long long n, unsigned long long *cnt,
                             unsigned long long *first)
{
  unsigned long long mism = 0, nbad = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    uint64_t A, B;
    dm_pair(seed, i, A, B);
    const double a = dm_double(A), b = dm_double(B);
    bool bad = false, bh = false, bq = false, bt = false, b4 = false, bp = false;
    const double r = dmul_int(a, b, bad);
    const double h = dpow2m_int<1>(a, bh), qt = dpow2m_int<2>(a, bq);
    const double tw = dtwice_int(a, bt), x4 = dquad_int(a, b4);
    const bool pos = dposprod_int(a, b, bp);
    const double pr = __dmul_rn(a, b);
    const bool off = (!bad && dm_bits(r) != dm_bits(pr)) ||
                     (!bh && dm_bits(h) != dm_bits(__dmul_rn(a, 0.5))) ||
                     (!bq && dm_bits(qt) != dm_bits(__dmul_rn(a, 0.25))) ||
                     (!bt && dm_bits(tw) != dm_bits(__dmul_rn(a, 2.0))) ||
                     (!b4 && dm_bits(x4) != dm_bits(__dmul_rn(a, 4.0))) ||
                     (!bp && pos != (pr > 0.0));
    if (bad) nbad++;
    if (off) {
      if (atomicCAS(first + 2, 0ull, 1ull) == 0ull) {
        first[0] = A;
        first[1] = B;
      }
      mism++;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    mism += __shfl_down_sync(0xffffffffu, mism, o);
    nbad += __shfl_down_sync(0xffffffffu, nbad, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(cnt, mism);
    atomicAdd(cnt + 1, nbad);
  }
}

}  // namespace ps

// Milliseconds of `iters` steps of 8 product chains per thread, `emul`
// (0..8) of them on the integer pipes, on `blocks` CTAs of `warps` warps
// (best of 3 after a warm-up); -1 on a bad argument or a CUDA error.
extern "C" double ps_probe_dmul_rate(int emul, int blocks, int warps, int iters)
{
  if (emul < 0 || emul > 8 || blocks < 1 || blocks > 65535 || warps < 1 || warps > 32 ||
      iters < 1)
    return -1.0;
  using K = void (*)(double *, int, double, double);
  const K ks[9] = {ps::k_dmul_rate<0>, ps::k_dmul_rate<1>, ps::k_dmul_rate<2>,
                   ps::k_dmul_rate<3>, ps::k_dmul_rate<4>, ps::k_dmul_rate<5>,
                   ps::k_dmul_rate<6>, ps::k_dmul_rate<7>, ps::k_dmul_rate<8>};
  const double m0 = 1.0 + 0x1p-20, m1 = 1.0 / m0;
  double *out = nullptr;
  if (cudaMalloc(&out, sizeof(double)) != cudaSuccess) return -1.0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  ks[emul]<<<blocks, 32 * warps>>>(out, 16, m0, m1);
  float best = -1.f;
  for (int r = 0; r < 3; r++) {
    cudaEventRecord(e0);
    ks[emul]<<<blocks, 32 * warps>>>(out, iters, m0, m1);
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

// n operand pairs (dm_pair) through the integer product and the product's
// sign test (dposprod_int), and the first operand through the exact
// halving, quartering, doubling and quadrupling, compared bit for bit with
// the GPU's multiply (on_gpu 1) or the host's (on_gpu 0).  out[0]:
// pairs with a differing result, out[1]: products handed back (bad),
// out[2..3]: the first differing pair's bit patterns.  Returns 0, or -1 on a bad argument or a
// CUDA error.
extern "C" int ps_probe_dmul_check(int on_gpu, unsigned long long seed, long long n,
                                   unsigned long long *out)
{
  if (n < 0 || !out) return -1;
  out[0] = out[1] = out[2] = out[3] = 0;
  if (!on_gpu) {
    bool seen = false;
    for (long long i = 0; i < n; i++) {
      uint64_t A, B;
      ps::dm_pair(seed, i, A, B);
      const double a = ps::dm_double(A), b = ps::dm_double(B);
      bool bad = false, bh = false, bq = false, bt = false, b4 = false, bp = false;
      const double r = ps::dmul_int(a, b, bad);
      const double h = ps::dpow2m_int<1>(a, bh), qt = ps::dpow2m_int<2>(a, bq);
      const double tw = ps::dtwice_int(a, bt), x4 = ps::dquad_int(a, b4);
      const bool pos = ps::dposprod_int(a, b, bp);
      const volatile double ref = a * b, rh = a * 0.5, rq = a * 0.25, rt = a * 2.0,
                            r4 = a * 4.0;
      const bool off = (!bad && ps::dm_bits(r) != ps::dm_bits(ref)) ||
                       (!bh && ps::dm_bits(h) != ps::dm_bits(rh)) ||
                       (!bq && ps::dm_bits(qt) != ps::dm_bits(rq)) ||
                       (!bt && ps::dm_bits(tw) != ps::dm_bits(rt)) ||
                       (!b4 && ps::dm_bits(x4) != ps::dm_bits(r4)) ||
                       (!bp && pos != (ref > 0.0));
      if (bad) out[1]++;
      if (off) {
        if (!seen) {
          out[2] = A;
          out[3] = B;
          seen = true;
        }
        out[0]++;
      }
    }
    return 0;
  }
  unsigned long long *d = nullptr;
  if (cudaMalloc(&d, 5 * sizeof(unsigned long long)) != cudaSuccess) return -1;
  cudaError_t e = cudaMemset(d, 0, 5 * sizeof(unsigned long long));
  if (e == cudaSuccess) {
    ps::k_dmul_check<<<4096, 256>>>(seed, n, d, d + 2);
    e = cudaGetLastError();
  }
  unsigned long long h[5] = {0, 0, 0, 0, 0};
  if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost);
  cudaFree(d);
  out[0] = h[0];
  out[1] = h[1];
  out[2] = h[2];
  out[3] = h[3];
  return e == cudaSuccess ? 0 : -1;
}

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
