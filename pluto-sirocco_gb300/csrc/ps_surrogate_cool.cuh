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
constexpr int kInfCtasPerSm = 4;

// (model, block of cells) work item
struct BlockItem {
  int m, b;
};

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

// Prediction + judge for one cell; status and (if accepted) T_f.  The
// context needs nH, n, E, xi, tx and dt.
__device__ __forceinline__ int sg_decide(SgCtx &b, double T, bool inbox, float y, int use_net,
                                         double &T_f, double &T0, int &evals, bool &stiff)
{
  evals = 0;
  stiff = false;
  if (!inbox) return SG_OUT_OF_BOX;
  // xi^-1/2 and xi^1/4 = (xi^-1/2)^-1/2 by two reciprocal square roots
  b.isqxi = rsqrt(b.xi);
  b.sqsqxi = rsqrt(b.isqxi);
  T0 = T * (double)exp10f(4.0f * y);
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
  const double *pre;  // per-cell prefactors (5 arrays) or NULL
  Params p;
  WindParams w;
  Scalars *sc;
};

// Unit conversions of the learned step (set_sg_units, with the
// parameters): E = p e_of_p, n_H = rho nh_of_rho, n = rho n_of_rho,
// T = (p / rho) t_of_pr, p_new = T_new n p_of_tn.
struct SgUnits {
  double e_of_p, nh_of_rho, n_of_rho, t_of_pr, p_of_tn;
};

__device__ __forceinline__ SgUnits sg_units(const SgCoolArgs &A)
{
  return SgUnits{A.w.sg_e_of_p, A.w.sg_nh_of_rho, A.w.sg_n_of_rho, A.w.sg_t_of_pr,
                 A.w.sg_p_of_tn};
}

// The cell's quantities for the learned step.  Returns 0 (below 1e4 K:
// left alone, as the reference does), 1 (to solve) or 2 (within 1e-12 of
// 1e4 K: the exact path decides).
__device__ __forceinline__ int sg_cell_ctx(const SgCoolArgs &A, const SgUnits &u, double dt,
                                           double t, long long q, SgCtx &b, double &T, long long &c)
{
  const Params &p = A.p;
  int gi, gj, gk;
  cell_of(p, q, gi, gj, gk);
  c = vcell3(p, gk, gj, gi);
  const double rho = A.V[RHO * p.vstride + c], pr = A.V[PRS * p.vstride + c];
  T = pr / rho * u.t_of_pr;
  if (T < 1.e4 * (1.0 - 1e-12)) return 0;
  b.dt = dt * A.w.unit_time;
  b.E = pr * u.e_of_p;
  b.nH = rho * u.nh_of_rho;
  b.n = rho * u.n_of_rho;
  if (A.w.xi_const > 0.0) {
    b.xi = A.w.xi_const;
    b.tx = A.w.t_x;
  } else if (t <= 3.0) {
    const double r = A.x1[gi] * A.w.unit_length;
    b.xi = A.w.lx / (b.nH * r * r);
    b.tx = A.w.t_x;
  } else {
    b.xi = A.xi[c];
    b.tx = A.tr[c];
  }
  if (A.pre) {  // the network knows prefactors 1 only
    for (int k = 0; k < 5; k++)
      if (A.pre[k * p.vstride + c] != 1.0) return 2;
  }
  return T < 1.e4 * (1.0 + 1e-12) ? 2 : 1;
}

// One CTA over 128-cell blocks of grids: the network on the tensor cores,
// the judge per cell; cells the judge rejects are queued (model, cell)
// for the reference method.  `blocks` gives (model, block) per item;
// args(m) the model's arguments.  Set-up (tensor memory, network in shared
// memory) once per CTA.
template <class ArgsOf>
__device__ __forceinline__ void sg_cool_items(const SgNet &net, const SgBox &bx, ArgsOf args_of,
                                              const BlockItem *blocks, int nitems, int use_net,
                                              unsigned char *smem, int2 *queue, int *qcount,
                                              unsigned long long *stats)
{
  const uint32_t tmem = sg_inf_setup(net, smem);
  uint32_t phase = 0;
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const BlockItem bi = blocks[it];
    const SgCoolArgs A = args_of(bi.m);
    if (A.sc->done) continue;  // uniform over the CTA
    const SgUnits u = sg_units(A);
    const long long ncell = (long long)A.p.nx[0] * A.p.nx[1] * A.p.nx[2];
    const long long q = (long long)bi.b * kSgRows + threadIdx.x;
    const bool active = q < ncell;
    const double dt = A.sc->dt, t = A.sc->t;
    SgCtx b;
    double T = 0.0;
    long long c = 0;
    float x[4] = {0.f, 0.f, 0.f, 0.f};
    bool inbox = false;
    int kind = 0;
    if (active) {
      kind = sg_cell_ctx(A, u, dt, t, q, b, T, c);
      if (kind == 1 && b.tx == bx.t_x) {
        inbox = sg_features(bx, b.nH, T, b.xi, b.dt, x);
        if (!inbox) x[0] = x[1] = x[2] = x[3] = 0.f;
      }
    }
    // the judge's first rate evaluation settles the non-stiff cells, which
    // do not read the network's prediction; the network runs only for a
    // block that holds a stiff cell (CTA-uniform), to start its iterations
    int st = SG_BELOW_MIN, evals = 0;
    bool stiff = false;
    double T_f = 0.0, z = 0.0, dz = 0.0;
    if (kind == 1 && inbox) {
      // xi^-1/2 and xi^1/4 = (xi^-1/2)^-1/2 by two reciprocal square roots
      b.isqxi = rsqrt(b.xi);
      b.sqsqxi = rsqrt(b.isqxi);
      evals = 1;
      bool bad = false;
      st = sg_judge_first_t<true>(b, T, z, dz, T_f, bad);
      if (bad) st = sg_judge_first_t<false>(b, T, z, dz, T_f, bad);
      stiff = st == SG_PENDING;
    } else if (kind == 1) {
      st = SG_OUT_OF_BOX;
    } else if (kind == 2) {
      st = SG_REJECT;
    }
    bool ok = true;
    float y = 0.f;
    if (__syncthreads_or(stiff && use_net)) {
      ok = sg_forward(smem, tmem, phase, x, 0, 0, y);
      if (!ok && threadIdx.x == 0) atomicOr(&A.sc->flags, F_TMA_TIMEOUT);
    }
    if (stiff) {
      const double T0 = T * (double)exp10f(4.0f * y);
      st = ok ? sg_judge_rest(b, T, T0, use_net != 0, z, dz, T_f, evals) : SG_REJECT;
    }
    if (kind) {
      if (st == SG_ACCEPT) {
        A.V[PRS * A.p.vstride + c] = dmax(T_f, 1.e4) * b.n * u.p_of_tn;
      } else {
        const int k = atomicAdd(qcount, 1);
        queue[k] = make_int2(bi.m, q);
      }
    }
    sg_count(st, active, evals, stiff, stats);
    if (!ok) break;
  }
  sg_inf_teardown(tmem);
}

}  // namespace ps
