// ps_surrogate_cool.cuh -- the surrogate inside the wind's split-source
// step (BLONDIN, Src/split_source.c:52-53), shared by the single-grid and
// the batched kernels: one 128-cell block per CTA, the network on the
// tensor cores, the Newton judge per cell, and a queue of the cells left to
// the reference method (bracket + Brent).
#pragma once

#include "ps_surrogate.cuh"
#include "ps_wind_dev.cuh"

namespace ps {

// Dynamic shared memory of an inference CTA: the forward pass needs about
// 31 KB; asking for 48 KB keeps at most 4 CTAs (64 tensor-memory columns
// each) on an SM, so tcgen05.alloc never has to wait.
constexpr int kInfBytes = 48 * 1024;

// Tensor-memory allocation and the network in shared memory for a
// 128-thread inference CTA; returns the tensor-memory address.
__device__ __forceinline__ uint32_t sg_inf_setup(const SgNet &net, unsigned char *smem)
{
  uint32_t *slot = reinterpret_cast<uint32_t *>(smem + kSgOffSlot);
  if ((threadIdx.x >> 5) == 0) tmem_alloc(slot, 64);
  if (threadIdx.x == 0) mbar_init(reinterpret_cast<uint64_t *>(smem + kSgOffBar), 1);
  sg_load_net(net, smem);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  return *slot;
}

__device__ __forceinline__ void sg_inf_teardown(uint32_t tmem)
{
  tc_fence_before();
  __syncthreads();
  if ((threadIdx.x >> 5) == 0) tmem_dealloc(tmem, 64);
}

// Prediction + judge for one prepared cell; status and (if accepted) T_f.
__device__ __forceinline__ int sg_decide(BlCtx &b, double T, bool inbox, float y, int use_net,
                                         double &T_f, double &T0, int &evals, bool &stiff)
{
  evals = 0;
  stiff = false;
  if (!inbox) return SG_OUT_OF_BOX;
  b.sqxi = sqrt(b.xi);
  b.sqsqxi = pow(b.xi, 0.25);
  T0 = T * exp10(4.0 * (double)y);
  return sg_judge(b, T, T0, use_net != 0, T_f, evals, stiff);
}

// stats: [0] accepted, [1] out of box, [2] rejected by the judge,
// [3] below 1e4 K, [4] net-rate evaluations of the judge, [5] stiff cells
// (not converged at the old temperature)
__device__ __forceinline__ void sg_count(int st, bool active, int evals, bool stiff,
                                         unsigned long long *stats)
{
  const int a = __syncthreads_count(active && st == SG_ACCEPT);
  const int o = __syncthreads_count(active && st == SG_OUT_OF_BOX);
  const int j = __syncthreads_count(active && st == SG_REJECT);
  const int m = __syncthreads_count(active && st == SG_BELOW_MIN);
  const int f = __syncthreads_count(active && stiff);
  const unsigned e = __reduce_add_sync(0xffffffffu, active ? (unsigned)evals : 0u);
  if ((threadIdx.x & 31) == 0 && e) atomicAdd(&stats[4], (unsigned long long)e);
  if (threadIdx.x == 0) {
    if (a) atomicAdd(&stats[0], (unsigned long long)a);
    if (o) atomicAdd(&stats[1], (unsigned long long)o);
    if (j) atomicAdd(&stats[2], (unsigned long long)j);
    if (m) atomicAdd(&stats[3], (unsigned long long)m);
    if (f) atomicAdd(&stats[5], (unsigned long long)f);
  }
}

struct SgCoolArgs {
  double *V;
  const double *xi, *tr, *x1;
  Params p;
  WindParams w;
  Scalars *sc;
};

// One 128-cell block of one grid: surrogate + judge; rejected cells are
// queued (model, cell) for the reference method.
__device__ __forceinline__ void sg_cool_block(const SgNet &net, const SgBox &bx, const SgCoolArgs &A,
                                              int model, int blk, int use_net, unsigned char *smem,
                                              int2 *queue, int *qcount, unsigned long long *stats)
{
  if (A.sc->done) return;  // uniform over the CTA
  const uint32_t tmem = sg_inf_setup(net, smem);
  const int ncell = A.p.nx[0] * A.p.nx[1];
  const int q = blk * kSgRows + threadIdx.x;
  const bool active = q < ncell;
  const double dt = A.sc->dt, t = A.sc->t;
  BlCtx b;
  double T = 0.0;
  long long c = 0;
  float x[4] = {0.f, 0.f, 0.f, 0.f};
  bool inbox = false, solve = false;
  if (active) {
    solve = blondin_ctx(A.V, A.xi, A.tr, A.p, A.w, A.x1, dt, t, q, b, T, c);
    if (solve && b.tx == bx.t_x) {
      inbox = sg_features(bx, b.nH, T, b.xi, b.dt_share, x);
      if (!inbox) x[0] = x[1] = x[2] = x[3] = 0.f;
    }
  }
  uint32_t phase = 0;
  float y = 0.f;
  const bool ok = sg_forward(smem, tmem, phase, x, 0, 0, y);
  if (!ok && threadIdx.x == 0) atomicOr(&A.sc->flags, F_TMA_TIMEOUT);
  int st = SG_BELOW_MIN, evals = 0;
  bool stiff = false;
  if (solve) {
    double T_f = 0.0, T0;
    st = ok ? sg_decide(b, T, inbox, y, use_net, T_f, T0, evals, stiff) : SG_REJECT;
    if (st == SG_ACCEPT) {
      blondin_store(A.V, A.p, A.w, b, c, T_f);
    } else {
      const int k = atomicAdd(qcount, 1);
      queue[k] = make_int2(model, q);
    }
  }
  sg_count(st, active, evals, stiff, stats);
  sg_inf_teardown(tmem);
}

}  // namespace ps
