// ps_surrogate.cuh -- the learned cooling step: a 4 -> 64 -> 64 -> 1 SiLU
// MLP mapping (log n_H, log T, log xi, log dt) to log T_new of one BLONDIN
// solve, run on the tensor cores (BF16 operands, FP32 accumulation in tensor
// memory), followed by FP64 Newton steps on BLONDIN's implicit energy
// equation that both polish the prediction and judge it (sg_judge).  A
// cell whose inputs leave the training box, or whose residual does not
// reach 1e-3 of its thermal energy, is solved by the reference method
// (bracket + Brent) instead.
//
// Network (all per row b of a 128-row tile, one thread per row):
//   x   = features, 4 values in [-1, 1] (bf16), padded with zeros to K = 16
//   z1  = W1 x + b1          (tensor cores, FP32)   h1 = silu(z1)   -> bf16
//   z2  = W2 h1 + b2         (tensor cores, FP32)   h2 = silu(z2)   (FP32)
//   y   = w3 . h2 + b3       (CUDA cores, FP32; w3 rounded to bf16)
//   log10 T_new = log10 T + 4 y
// Parameter vector (FP32 master copy, kSgParams values):
//   W1[64][4], b1[64], W2[64][64], b2[64], w3[64], b3.
#pragma once

#include <cuda_bf16.h>

#include "ps_blondin.cuh"
#include "ps_fastmath.cuh"
#include "ps_physics.cuh"
#include "ps_tc.cuh"

namespace ps {

constexpr int kSgH = 64, kSgIn = 4, kSgK1 = 16, kSgRows = 128;
constexpr int kSgW1 = 0, kSgB1 = 256, kSgW2 = 320, kSgB2 = 4416, kSgW3 = 4480, kSgB3 = 4544;
constexpr int kSgParams = 4545;
constexpr int kSgSmall = 3 * kSgH + 1;  // b1, b2, w3 (bf16-rounded), b3 as FP32

// Training box and scales: u = (log10 v - lo) * scale - 1.
struct SgBox {
  double lo[4], hi[4], scale[4];
  double t_x, mu;
};

// Device copies of the network the kernels read.
struct SgNet {
  const __nv_bfloat16 *w1b;   // [64][16] W1 in bf16, inputs 4..15 zero
  const __nv_bfloat16 *w2b;   // [64][64] W2 (row j = output unit)
  const __nv_bfloat16 *w2tb;  // [64][64] W2 transposed
  const float *small;         // b1[64], b2[64], w3r[64], b3
};

// Acceptance rule of the Newton judge: |z| / thermal energy, and the
// most net-rate evaluations per cell (the one at the old T included).
constexpr double kSgResidual = 1e-3;
constexpr int kSgMaxNewton = 5;
// A stiff cell starts from the prediction when that moves T by more than
// this fraction; below it the first Newton step from T is as good a start.
constexpr double kSgJump = 0.1;

enum { SG_ACCEPT = 0, SG_OUT_OF_BOX = 1, SG_REJECT = 2, SG_BELOW_MIN = 3 };

// ------------------------------------------------------------------
// shared-memory layout of the forward pass
// ------------------------------------------------------------------

constexpr int kSgOffX = 0;                                   // 128 x 16 bf16
constexpr int kSgOffW1 = kSgOffX + kSgRows * kSgK1 * 2;      // 64 x 16 bf16
constexpr int kSgOffH1 = kSgOffW1 + kSgH * kSgK1 * 2;        // 128 x 64 bf16
constexpr int kSgOffW2 = kSgOffH1 + kSgRows * kSgH * 2;      // 64 x 64 bf16
constexpr int kSgOffSmall = kSgOffW2 + kSgH * kSgH * 2;      // 193 floats
constexpr int kSgOffBar = kSgOffSmall + 1024;                // mbarrier
constexpr int kSgOffSlot = kSgOffBar + 8;                    // tensor-memory address
constexpr int kSgFwdBytes = kSgOffSlot + 8;

__device__ __forceinline__ float sg_silu(float z) { return z / (1.0f + __expf(-z)); }

__device__ __forceinline__ uint32_t pack_bf16(float a, float b)
{
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<const uint32_t *>(&h);
}

// Copies the network into shared memory (all threads of the CTA).
__device__ __forceinline__ void sg_load_net(const SgNet &net, unsigned char *smem)
{
  const int tid = threadIdx.x, nt = blockDim.x;
  // W1: 64 rows x 2 chunks of 8 bf16
  for (int c = tid; c < kSgH * 2; c += nt) {
    const int j = c >> 1, kb = c & 1;
    *reinterpret_cast<uint4 *>(smem + kSgOffW1 + kmaj_off(j, kb * 8, kSgK1)) =
        *reinterpret_cast<const uint4 *>(net.w1b + j * kSgK1 + kb * 8);
  }
  // W2: 64 rows x 8 chunks
  for (int c = tid; c < kSgH * 8; c += nt) {
    const int j = c >> 3, kb = c & 7;
    *reinterpret_cast<uint4 *>(smem + kSgOffW2 + kmaj_off(j, kb * 8, kSgH)) =
        *reinterpret_cast<const uint4 *>(net.w2b + j * kSgH + kb * 8);
  }
  float *sm = reinterpret_cast<float *>(smem + kSgOffSmall);
  for (int c = tid; c < kSgSmall; c += nt) sm[c] = net.small[c];
}

// Writes one row of bf16 values (16 at a time) into a K-major operand.
__device__ __forceinline__ void sg_store_row16(unsigned char *base, int r, int k0, int K,
                                               const float (&v)[16])
{
  uint4 a, b;
  a.x = pack_bf16(v[0], v[1]);
  a.y = pack_bf16(v[2], v[3]);
  a.z = pack_bf16(v[4], v[5]);
  a.w = pack_bf16(v[6], v[7]);
  b.x = pack_bf16(v[8], v[9]);
  b.y = pack_bf16(v[10], v[11]);
  b.z = pack_bf16(v[12], v[13]);
  b.w = pack_bf16(v[14], v[15]);
  *reinterpret_cast<uint4 *>(base + kmaj_off(r, k0, K)) = a;
  *reinterpret_cast<uint4 *>(base + kmaj_off(r, k0 + 8, K)) = b;
}

// Bounded wait for the MMA group committed to `bar`; CTA-uniform result.
__device__ __forceinline__ bool sg_wait(uint64_t *bar, uint32_t &phase)
{
  const bool ok = mbar_wait_bounded(bar, phase, 1u << 22);
  phase ^= 1u;
  tc_fence_after();
  return __syncthreads_and(ok) != 0;
}

// Forward pass of a 128-row tile; thread tid owns row tid (tensor-memory
// lane tid).  Tensor memory: z1 in columns [c1, c1 + 64), z2 in
// [c2, c2 + 64) (c1 == c2 is allowed: z1 is consumed before the second
// MMA is issued).  The network and the tensor-memory address must already
// be in shared memory.  Returns false (CTA-uniform) if an MMA did not
// complete in time.
__device__ __forceinline__ bool sg_forward(unsigned char *smem, uint32_t tmem, uint32_t &phase,
                                           const float (&x)[4], int c1, int c2, float &y)
{
  const int r = threadIdx.x, warp = r >> 5;
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem + kSgOffBar);
  const float *sm = reinterpret_cast<const float *>(smem + kSgOffSmall);
  const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
  {
    uint4 a, z = make_uint4(0u, 0u, 0u, 0u);
    a.x = pack_bf16(x[0], x[1]);
    a.y = pack_bf16(x[2], x[3]);
    a.z = 0u;
    a.w = 0u;
    *reinterpret_cast<uint4 *>(smem + kSgOffX + kmaj_off(r, 0, kSgK1)) = a;
    *reinterpret_cast<uint4 *>(smem + kSgOffX + kmaj_off(r, 8, kSgK1)) = z;
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  if (r == 0) {
    tc_fence_after();
    umma_bf16(tmem + c1, umma_slice_desc(smem + kSgOffX, kSgK1, 0),
              umma_slice_desc(smem + kSgOffW1, kSgK1, 0), umma_idesc_bf16(128, kSgH), false);
    umma_commit(bar);
  }
  if (!sg_wait(bar, phase)) return false;
#pragma unroll
  for (int c = 0; c < 4; c++) {
    float v[16];
    tmem_ld16(lane_addr + c1 + 16 * c, v);
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = sg_silu(v[i] + sm[16 * c + i]);
    sg_store_row16(smem + kSgOffH1, r, 16 * c, kSgH, v);
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  if (r == 0) {
    tc_fence_after();
#pragma unroll
    for (int s = 0; s < 4; s++)
      umma_bf16(tmem + c2, umma_slice_desc(smem + kSgOffH1, kSgH, s),
                umma_slice_desc(smem + kSgOffW2, kSgH, s), umma_idesc_bf16(128, kSgH), s > 0);
    umma_commit(bar);
  }
  if (!sg_wait(bar, phase)) return false;
  float acc = 0.0f;
#pragma unroll
  for (int c = 0; c < 4; c++) {
    float v[16];
    tmem_ld16(lane_addr + c2 + 16 * c, v);
#pragma unroll
    for (int i = 0; i < 16; i++) {
      const float h = sg_silu(v[i] + sm[kSgH + 16 * c + i]);
      acc += sm[2 * kSgH + 16 * c + i] * h;
    }
  }
  y = acc + sm[3 * kSgH];
  return true;
}

// Features of a tuple (FP32 logarithms: the network sees them as bf16);
// false when the tuple lies outside the training box.
__device__ __forceinline__ bool sg_features(const SgBox &bx, double nH, double T, double xi,
                                            double dt, float (&x)[4])
{
  const float l[4] = {log10f((float)nH), log10f((float)T), log10f((float)xi), log10f((float)dt)};
  bool in = true;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    in = in && (l[i] >= (float)bx.lo[i]) && (l[i] <= (float)bx.hi[i]);
    x[i] = (l[i] - (float)bx.lo[i]) * (float)bx.scale[i] - 1.0f;
  }
  return in;
}

// One cell's BLONDIN quantities for the learned step: n_H, n, thermal
// energy E, xi with sqrt(xi)^-1 and xi^1/4, T_x, dt [s] and the net rate at
// the old temperature.
struct SgCtx {
  double nH, n, E, xi, isqxi, sqsqxi, tx, dt, hc_init;
};

// heatcool (Src/Cooling/BLONDIN/cooling.c:173-222, prefactors 1) and its
// T-derivative, term by term:
//   ne = nH r(T), r = 1e-2 + 10^(a + b log10 T) -> r' = b 10^(a + b log10 T) / T
//   (the middle branch without the 1e-2), 0 above 3.3e4 K;
//   comp_cool' = 8.9e-36 xi 4; xray' = -xray / (2T);
//   line term 1e-16 e^(-1.3e5/T) / (sqrt(xi) T): ' = term (1.3e5/T - 1) / T;
//   the min() term: 0, 2.5e-27/sqrt(T) or -1.5e-17/T^2 by the active branch;
//   brem' = brem / (2T).
template <bool INT>
__device__ __forceinline__ double sg_heatcool_d_t(const SgCtx &b, double T, double &dhc,
                                                  bool &bad)
{
  // products no add absorbs by dmul_t<INT> (on the integer pipes with INT,
  // ps_dmul.cuh; the same bits either way)
  // 1/T and sqrt(T) from one reciprocal square root (the judge's own
  // arithmetic: it only has to find the root the network points at)
  const double rT = rsqrt(T), sqT = dmul_t<INT>(T, rT, bad), iT = dmul_t<INT>(rT, rT, bad);
  double r, dr;
  if (T < 1.5e4) {
    const double q = fm::exp(2.302585092994046 * (-51.59417133) + 12.27740153 * fm::log(T));
    r = 1e-2 + q;
    dr = dmul_t<INT>(dmul_t<INT>(12.27740153, q, bad), iT, bad);
  } else if (T < 3.3e4) {
    const double q = fm::exp(2.302585092994046 * (-3.80749689) + 0.86092628 * fm::log(T));
    r = q;
    dr = dmul_t<INT>(dmul_t<INT>(0.86092628, q, bad), iT, bad);
  } else {
    r = 1.21;
    dr = 0.0;
  }
  const double ne = dmul_t<INT>(b.nH, r, bad), dne = dmul_t<INT>(b.nH, dr, bad);
  const double cxi = dmul_t<INT>(8.9e-36, b.xi, bad);
  const double comp_heat = dmul_t<INT>(cxi, b.tx, bad);
  const double comp_cool = dmul_t<INT>(cxi, dquad_t<INT>(T, bad), bad);
  const double dcomp_cool = dquad_t<INT>(cxi, bad);
  const double xray_heat = dmul_t<INT>(dmul_t<INT>(1.5e-21, b.sqsqxi, bad), rT, bad);
  const double dxray_heat = dmul_t<INT>(-dhalf_t<INT>(xray_heat, bad), iT, bad);
  const double l1 = dmul_t<INT>(
      dmul_t<INT>(dmul_t<INT>(1e-16, fm::exp(dmul_t<INT>(-1.3e5, iT, bad)), bad), b.isqxi, bad),
      iT, bad);
  const double dl1 = dmul_t<INT>(dmul_t<INT>(l1, fma(1.3e5, iT, -1.0), bad), iT, bad);
  const double m1 = dmul_t<INT>(5e-27, sqT, bad), m2 = dmul_t<INT>(1.5e-17, iT, bad);
  double l2, dl2;
  if (1e-24 <= m1 && 1e-24 <= m2) {
    l2 = 1e-24;
    dl2 = 0.0;
  } else if (m1 <= m2) {
    l2 = m1;
    dl2 = dmul_t<INT>(dhalf_t<INT>(m1, bad), iT, bad);
  } else {
    l2 = m2;
    dl2 = -dmul_t<INT>(m2, iT, bad);
  }
  const double brem_cool = dmul_t<INT>(3.3e-27, sqT, bad);
  const double dbrem_cool = dmul_t<INT>(dhalf_t<INT>(brem_cool, bad), iT, bad);
  const double net = comp_heat - comp_cool - (l1 + l2) - brem_cool;
  const double dnet = -dcomp_cool - (dl1 + dl2) - dbrem_cool;
  dhc = dmul_t<INT>(b.nH, fma(b.nH, dxray_heat, fma(ne, dnet, dmul_t<INT>(dne, net, bad))), bad);
  return dmul_t<INT>(b.nH, fma(b.nH, xray_heat, dmul_t<INT>(ne, net, bad)), bad);
}
__device__ __forceinline__ double sg_heatcool_d(const SgCtx &b, double T, double &dhc)
{
  bool bad = false;
  return sg_heatcool_d_t<false>(b, T, dhc, bad);
}

// z(T) = T n kB / (2/3) - E - dt (hc(T_old) + hc(T)) / 2 (cooling.c:233-237)
// and dz/dT.
__device__ __forceinline__ double sg_z(const SgCtx &b, double T, double &dz, double &hc)
{
  double dhc;
  hc = sg_heatcool_d(b, T, dhc);
  const double cth = b.n * kKB * 1.5;
  dz = cth - b.dt * dhc * 0.5;
  return T * cth - b.E - b.dt * (b.hc_init + hc) * 0.5;
}

// The judge.  The net rate and its derivative at the old temperature T give
// z(T) = -dt hc(T).  If |z(T)| is already within kSgResidual of the
// thermal energy, one Newton step from T is the answer (non-stiff cell: one
// rate evaluation in all).  Otherwise (stiff cell) damped Newton iterations
// (each step kept within a factor 2) run until the residual is within
// kSgResidual, at most kSgMaxNewton evaluations, starting from the
// network's prediction T0 when it moves T by more than kSgJump (from T when
// from_net is false or the predicted change is small); a final Newton step
// polishes the converged point.  When the net rate at the converged point
// has the opposite sign of the initial one, the answer is instead the
// equilibrium temperature between T and that point (the reference's second
// Brent solve, cooling.c:150-157), found by a bracketed Newton iteration
// on the net rate (sg_judge_equilibrium).  Rejected: no convergence,
// z' <= 0, or a root more than 1e-8 T on the wrong side of T.  Sets
// hc_init.
//
// In three parts, so that a kernel can settle the non-stiff cells before
// it knows whether it needs the network at all (sg_cool_items):
// sg_judge_first evaluates the rate at T and settles a non-stiff cell
// (SG_PENDING for a stiff one, with z and dz at T), sg_judge_rest iterates
// a stiff cell from there, and sg_judge_final is the polishing step and
// the checks of both.
constexpr int SG_PENDING = 4;

constexpr int kSgMaxEquil = 8;   // net-rate evaluations of the equilibrium iteration

// The equilibrium temperature, the root of the net rate hc between T (rate
// hc_init) and Tk (rate hc_k, of the opposite sign): Newton steps on hc,
// each kept inside the bracket, which shrinks to the side whose rate has
// the sign of the lower end's (a step that would leave it bisects
// instead); converged when a step moves T by at most 1e-10 T.  dhc_k is
// dhc/dT at Tk.
__device__ __forceinline__ int sg_judge_equilibrium(const SgCtx &b, double T, double Tk,
                                                    double hc_k, double dhc_k, double &T_f,
                                                    int &evals)
{
  double lo = fmin(T, Tk), hi = fmax(T, Tk);
  double flo = T <= Tk ? b.hc_init : hc_k;
  double x = Tk, fx = hc_k, dfx = dhc_k;
  for (int it = 0; it < kSgMaxEquil; it++) {
    double xn = x - fx / dfx;
    if (!(xn > lo && xn < hi)) xn = 0.5 * (lo + hi);   // outside, or not a number
    double dfn;
    const double fn = sg_heatcool_d(b, xn, dfn);
    evals++;
    if (lt0(fn * flo)) {
      hi = xn;
    } else {
      lo = xn;
      flo = fn;
    }
    const double step = fabs(xn - x);
    x = xn;
    fx = fn;
    dfx = dfn;
    if (step <= 1e-10 * x || fn == 0.0) {
      if (!gt0(x) || !isfinite(x)) return SG_REJECT;
      T_f = x;
      return SG_ACCEPT;
    }
  }
  return SG_REJECT;
}

__device__ __forceinline__ int sg_judge_final(const SgCtx &b, double T, double Tk, double z,
                                              double dz, double hc, double &T_f, int &evals)
{
  if (!gt0(dz)) return SG_REJECT;
  if (lt0(hc * b.hc_init)) {
    // dhc/dT at Tk from z' = n kB 3/2 - dt dhc/dT / 2
    const double dhc = (b.n * kKB * 1.5 - dz) * 2.0 / b.dt;
    return sg_judge_equilibrium(b, T, Tk, hc, dhc, T_f, evals);
  }
  const double Tn = Tk - z / dz;
  // a root on the wrong side of T (against the initial net rate) is refused
  // unless the move is below 1e-8 T: at thermal equilibrium dt hc is below
  // the rounding of T n kB 3/2 - E and the step's sign is noise (the
  // reference's Brent solve stops within 1 K)
  if (!gt0(Tn) || !isfinite(Tn) || (lt0((Tn - T) * b.hc_init) && fabs(Tn - T) > 1e-8 * T))
    return SG_REJECT;
  T_f = Tn;
  return SG_ACCEPT;
}

// (the first rate evaluation with its products by dmul_t<INT>: on the
// integer pipes with INT, the same bits either way)
template <bool INT>
__device__ __forceinline__ int sg_judge_first_t(SgCtx &b, double T, double &z, double &dz,
                                                double &T_f, bool &bad)
{
  const double cth = b.n * kKB * 1.5;
  double dhc;
  b.hc_init = sg_heatcool_d_t<INT>(b, T, dhc, bad);
  z = T * cth - b.E - b.dt * b.hc_init;
  dz = cth - b.dt * dhc * 0.5;
  if (!(fabs(z) <= kSgResidual * T * cth)) return SG_PENDING;
  int evals = 1;   // hc at T is hc_init: no sign change, no further evaluation
  return sg_judge_final(b, T, T, z, dz, b.hc_init, T_f, evals);
}
__device__ __forceinline__ int sg_judge_first(SgCtx &b, double T, double &z, double &dz,
                                              double &T_f)
{
  bool bad = false;
  return sg_judge_first_t<false>(b, T, z, dz, T_f, bad);
}

// evals counts the evaluation of sg_judge_first
__device__ __forceinline__ int sg_judge_rest(const SgCtx &b, double T, double T0, bool from_net,
                                             double z, double dz, double &T_f, int &evals)
{
  const double cth = b.n * kKB * 1.5;
  double Tk = T, hc = b.hc_init;
  bool conv = false;
  if (from_net && gt0(T0) && isfinite(T0) && fabs(T0 - T) > kSgJump * T) {
    Tk = T0;
    z = sg_z(b, Tk, dz, hc);
    evals++;
    conv = fabs(z) <= kSgResidual * Tk * cth;
  }
  for (int it = 0; !conv; it++) {
    if (evals >= kSgMaxNewton || !gt0(dz)) return SG_REJECT;
    Tk = fmin(fmax(Tk - z / dz, 0.5 * Tk), 2.0 * Tk);
    z = sg_z(b, Tk, dz, hc);
    evals++;
    conv = fabs(z) <= kSgResidual * Tk * cth;
  }
  return sg_judge_final(b, T, Tk, z, dz, hc, T_f, evals);
}

__device__ __forceinline__ int sg_judge(SgCtx &b, double T, double T0, bool from_net, double &T_f,
                                        int &evals, bool &stiff)
{
  double z, dz;
  evals = 1;
  const int st = sg_judge_first(b, T, z, dz, T_f);
  stiff = st == SG_PENDING;
  if (!stiff) return st;
  return sg_judge_rest(b, T, T0, from_net, z, dz, T_f, evals);
}

}  // namespace ps
