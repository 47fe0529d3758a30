// ps_surrogate.cu -- the learned BLONDIN cooling step: training-pair
// labelling with the reference method, training on the tensor cores with
// the project's own forward/backward kernels and Adam, inference on tuples
// and inside the wind's split-source step (with the Newton judge and the
// bracket + Brent fallback).
//
// Training, per 128-row tile of a minibatch (one CTA, one thread per row;
// tensor memory: z1 in columns 0-63, z2 then dL/dh1 in 64-127, the dW2
// partial in 128-255):
//   forward as in ps_surrogate.cuh, loss = mean (y - y*)^2,
//   dy   = 2 (y - y*) / B
//   g_w3 = sum dy h2,  g_b3 = sum dy
//   dz2  = dy w3 silu'(z2),  g_b2 = sum dz2
//   g_W2 = dz2^T h1          (tensor cores: bf16 dz2, bf16 h1; the two
//                             64-row halves of the tile are the two diagonal
//                             64 x 64 blocks of one M = N = 128 product)
//   dh1  = dz2 W2            (tensor cores: bf16 dz2, bf16 W2)
//   dz1  = dh1 silu'(z1),    g_b1 = sum dz1,  g_W1 = dz1^T x
// Per-tile partial gradients are reduced in a fixed order by the Adam
// kernel, so training is deterministic.
#include "ps_ctx.cuh"
#include "ps_surrogate_cool.cuh"

#include <algorithm>
#include <cstdint>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

extern "C" void ps_set_error_msg(const char *msg);

namespace ps {

constexpr int kTrOffW2T = (kSgFwdBytes + 127) / 128 * 128;
constexpr int kTrOffDZ2 = kTrOffW2T + kSgH * kSgH * 2;
constexpr int kTrOffAp = kTrOffDZ2 + kSgRows * kSgH * 2;
constexpr int kTrOffBp = kTrOffAp + kSgRows * kSgH * 2;
constexpr int kTrOffR = kTrOffBp + kSgRows * kSgH * 2;
constexpr int kTrRS = 65;  // row stride of the reduction scratch (floats)
constexpr int kTrOffXf = kTrOffR + kSgRows * kTrRS * 4;
constexpr int kTrOffDy = kTrOffXf + kSgRows * 4 * 4;
constexpr int kTrBytes = kTrOffDy + kSgRows * 4;

__device__ __forceinline__ float bf16r(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

__device__ __forceinline__ void sg_store_bf16(unsigned char *base, int r, int k, int K, float v)
{
  *reinterpret_cast<__nv_bfloat16 *>(base + kmaj_off(r, k, K)) = __float2bfloat16_rn(v);
}

// ------------------------------------------------------------------
// training: forward + backward of one tile
// ------------------------------------------------------------------

__global__ void __launch_bounds__(128) k_sg_train_tile(SgNet net, const float4 *__restrict__ feat,
                                                       const float *__restrict__ target,
                                                       const int *__restrict__ idx, int nrows,
                                                       float inv_batch, float *__restrict__ gpart,
                                                       float *__restrict__ lpart,
                                                       unsigned *flags)
{
  extern __shared__ __align__(1024) unsigned char smem[];
  const int tid = threadIdx.x, warp = tid >> 5;
  uint32_t *slot = reinterpret_cast<uint32_t *>(smem + kSgOffSlot);
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem + kSgOffBar);
  if (warp == 0) tmem_alloc(slot, 256);
  if (tid == 0) mbar_init(bar, 1);
  sg_load_net(net, smem);
  for (int c = tid; c < kSgH * 8; c += 128) {
    const int j = c >> 3, kb = c & 7;
    *reinterpret_cast<uint4 *>(smem + kTrOffW2T + kmaj_off(j, kb * 8, kSgH)) =
        *reinterpret_cast<const uint4 *>(net.w2tb + j * kSgH + kb * 8);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *slot;
  const uint32_t lane_addr = tmem + ((uint32_t)(warp * 32) << 16);
  const float *sm = reinterpret_cast<const float *>(smem + kSgOffSmall);
  float *R = reinterpret_cast<float *>(smem + kTrOffR);
  float *Xf = reinterpret_cast<float *>(smem + kTrOffXf);
  float *Dy = reinterpret_cast<float *>(smem + kTrOffDy);
  float *gp = gpart + (size_t)blockIdx.x * kSgParams;

  const int row = blockIdx.x * kSgRows + tid;
  const bool valid = row < nrows;
  float x[4] = {0.f, 0.f, 0.f, 0.f}, tgt = 0.f;
  if (valid) {
    const float4 f = feat[idx[row]];
    x[0] = f.x;
    x[1] = f.y;
    x[2] = f.z;
    x[3] = f.w;
    tgt = target[idx[row]];
  }
#pragma unroll
  for (int i = 0; i < 4; i++) Xf[tid * 4 + i] = bf16r(x[i]);
  uint32_t phase = 0;
  float y = 0.f;
  bool ok = sg_forward(smem, tmem, phase, x, 0, 64, y);
  if (ok) {
    const float e = valid ? (y - tgt) : 0.f;
    const float dy = 2.f * e * inv_batch;
    Dy[tid] = dy;
    // h1^T into the B operand of the dW2 product: (n = half*64 + i, k = row in half)
    {
      const int h = tid >> 6, bq = tid & 63;
#pragma unroll
      for (int c = 0; c < 8; c++) {
        const uint4 v = *reinterpret_cast<const uint4 *>(smem + kSgOffH1 + kmaj_off(tid, 8 * c, kSgH));
        const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int q = 0; q < 4; q++) {
          *reinterpret_cast<uint16_t *>(smem + kTrOffBp + kmaj_off(h * 64 + 8 * c + 2 * q, bq, 64)) =
              (uint16_t)(w[q] & 0xFFFFu);
          *reinterpret_cast<uint16_t *>(smem + kTrOffBp + kmaj_off(h * 64 + 8 * c + 2 * q + 1, bq, 64)) =
              (uint16_t)(w[q] >> 16);
        }
      }
    }
    // pass 1 over z2: dy * h2 for g_w3
#pragma unroll
    for (int c = 0; c < 4; c++) {
      float v[16];
      tmem_ld16(lane_addr + 64 + 16 * c, v);
#pragma unroll
      for (int i = 0; i < 16; i++) R[tid * kTrRS + 16 * c + i] = dy * sg_silu(v[i] + sm[kSgH + 16 * c + i]);
    }
    // loss partial: warp sums, then the block's in Dy-free scratch (Xf is kept)
    float l = e * e;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    __syncthreads();
    if (tid < kSgH) {
      float s = 0.f;
      for (int b = 0; b < kSgRows; b++) s += R[b * kTrRS + tid];
      gp[kSgW3 + tid] = s;
    } else if (tid == kSgH) {
      float s = 0.f;
      for (int b = 0; b < kSgRows; b++) s += Dy[b];
      gp[kSgB3] = s;
    }
    if ((tid & 31) == 0) atomicAdd(&lpart[blockIdx.x], l);
    __syncthreads();
    // pass 2 over z2: dz2 (FP32 for g_b2, bf16 for the two products)
    {
      const int h = tid >> 6, bq = tid & 63;
#pragma unroll
      for (int c = 0; c < 4; c++) {
        float v[16], d[16];
        tmem_ld16(lane_addr + 64 + 16 * c, v);
#pragma unroll
        for (int i = 0; i < 16; i++) {
          const int j = 16 * c + i;
          const float z = v[i] + sm[kSgH + j];
          const float s = 1.0f / (1.0f + __expf(-z));
          d[i] = dy * sm[2 * kSgH + j] * (s * (1.0f + z * (1.0f - s)));
          R[tid * kTrRS + j] = d[i];
          sg_store_bf16(smem + kTrOffAp, h * 64 + j, bq, 64, d[i]);
        }
        sg_store_row16(smem + kTrOffDZ2, tid, 16 * c, kSgH, d);
      }
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
      // dL/dh1 = dz2 W2 -> columns 64..127
#pragma unroll
      for (int s = 0; s < 4; s++)
        umma_bf16(tmem + 64, umma_slice_desc(smem + kTrOffDZ2, kSgH, s),
                  umma_slice_desc(smem + kTrOffW2T, kSgH, s), umma_idesc_bf16(128, kSgH), s > 0);
      // dW2 partials (diagonal blocks of A' B'^T) -> columns 128..255
#pragma unroll
      for (int s = 0; s < 4; s++)
        umma_bf16(tmem + 128, umma_slice_desc(smem + kTrOffAp, 64, s),
                  umma_slice_desc(smem + kTrOffBp, 64, s), umma_idesc_bf16(128, 128), s > 0);
      umma_commit(bar);
    }
    if (tid < kSgH) {
      float s = 0.f;
      for (int b = 0; b < kSgRows; b++) s += R[b * kTrRS + tid];
      gp[kSgB2 + tid] = s;
    }
    ok = sg_wait(bar, phase);
  }
  if (ok) {
    // dz1 = dh1 silu'(z1)
#pragma unroll
    for (int c = 0; c < 4; c++) {
      float dh[16], z[16];
      tmem_ld16(lane_addr + 64 + 16 * c, dh);
      tmem_ld16(lane_addr + 16 * c, z);
#pragma unroll
      for (int i = 0; i < 16; i++) {
        const float zz = z[i] + sm[16 * c + i];
        const float s = 1.0f / (1.0f + __expf(-zz));
        R[tid * kTrRS + 16 * c + i] = dh[i] * (s * (1.0f + zz * (1.0f - s)));
      }
    }
    // this thread's lane of the dW2 product: row j of the half it belongs to
    float p[64];
    {
      const int off = tid < 64 ? 128 : 192;
#pragma unroll
      for (int c = 0; c < 4; c++) {
        float v[16];
        tmem_ld16(lane_addr + off + 16 * c, v);
#pragma unroll
        for (int i = 0; i < 16; i++) p[16 * c + i] = v[i];
      }
    }
    __syncthreads();
    if (tid < kSgH) {
      float s = 0.f;
      for (int b = 0; b < kSgRows; b++) s += R[b * kTrRS + tid];
      gp[kSgB1 + tid] = s;
    }
    for (int o = tid; o < kSgH * kSgIn; o += 128) {
      const int j = o >> 2, i = o & 3;
      float s = 0.f;
      for (int b = 0; b < kSgRows; b++) s += R[b * kTrRS + j] * Xf[b * 4 + i];
      gp[kSgW1 + o] = s;
    }
    __syncthreads();
    // the two halves' dW2 partials through the scratch, summed in a fixed order
#pragma unroll
    for (int i = 0; i < 64; i++) R[tid * 64 + i] = p[i];
    __syncthreads();
    for (int o = tid; o < kSgH * kSgH; o += 128) gp[kSgW2 + o] = R[o] + R[4096 + o];
  }
  if (!ok && tid == 0) atomicOr(flags, F_TMA_TIMEOUT);
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, 256);
}

// Adam on the master parameters from the per-tile partials (fixed-order
// sum), then the bf16 / FP32 copies the kernels read.  `apply` = 0 only
// reduces the gradient into `grad`.
__global__ void k_sg_adam(float *__restrict__ prm, float *__restrict__ m1, float *__restrict__ m2,
                          const float *__restrict__ gpart, int nblk, float lr, float bc1,
                          float bc2, int apply, float *__restrict__ grad, __nv_bfloat16 *w1b,
                          __nv_bfloat16 *w2b, __nv_bfloat16 *w2tb, float *small)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kSgParams) return;
  float g = 0.f;
  for (int b = 0; b < nblk; b++) g += gpart[(size_t)b * kSgParams + i];
  if (grad) grad[i] = g;
  float w = prm[i];
  if (apply) {
    const float a = 0.9f * m1[i] + 0.1f * g;
    const float v = 0.999f * m2[i] + 0.001f * g * g;
    m1[i] = a;
    m2[i] = v;
    w -= lr * (a / bc1) / (sqrtf(v / bc2) + 1e-8f);
    prm[i] = w;
  }
  if (i < kSgB1) {
    w1b[(i >> 2) * kSgK1 + (i & 3)] = __float2bfloat16_rn(w);
  } else if (i < kSgW2) {
    small[i - kSgB1] = w;
  } else if (i < kSgB2) {
    const int j = (i - kSgW2) >> 6, k = (i - kSgW2) & 63;
    w2b[j * kSgH + k] = __float2bfloat16_rn(w);
    w2tb[k * kSgH + j] = __float2bfloat16_rn(w);
  } else if (i < kSgW3) {
    small[kSgH + i - kSgB2] = w;
  } else if (i < kSgB3) {
    small[2 * kSgH + i - kSgW3] = bf16r(w);
  } else {
    small[3 * kSgH] = w;
  }
}

__global__ void k_sg_loss(const float *__restrict__ lpart, int nblk, float inv_batch, float *out)
{
  float s = 0.f;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) s += lpart[b];
  __shared__ float red[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (int w = 0; w < (int)(blockDim.x + 31) / 32; w++) t += red[w];
    *out = t * inv_batch;
  }
}

// ------------------------------------------------------------------
// tuples: labels (reference method), features, prediction
// ------------------------------------------------------------------

// BLONDIN context of a tuple (n_H, T, xi, dt_s): n = n_H 1.43 / mu,
// E = T n kB / (2/3).
__device__ __forceinline__ void sg_tuple_ctx(const SgBox &bx, double nH, double T, double xi,
                                             double dt, BlCtx &b)
{
  b.dt_share = dt;
  b.nH = nH;
  b.n = nH * 1.43 / bx.mu;
  b.E = T * b.n * kKB / (2.0 / 3.0);
  b.xi = xi;
  b.tx = bx.t_x;
}

__device__ __forceinline__ double sg_tuple_solve(const SgBox &bx, const double *tup, long r, long n,
                                                 unsigned *flags)
{
  const double T = tup[n + r];
  if (T < 1.e4) return T;
  BlCtx b;
  sg_tuple_ctx(bx, tup[r], T, tup[2 * n + r], tup[3 * n + r], b);
  bl_prepare(b, T);
  bool overflow;
  const double T_f = bl_solve(b, T, overflow);
  if (overflow) atomicOr(flags, F_NAN);
  return dmax(T_f, 1.e4);
}

// tuples are SoA: nH[n], T[n], xi[n], dt[n]; tcool (optional) gets the
// cooling time E / |net rate| at the old temperature
__global__ void k_sg_label(SgBox bx, const double *__restrict__ tup, long n, double *__restrict__ out,
                           double *__restrict__ tcool, unsigned *flags)
{
  for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x) {
    out[r] = sg_tuple_solve(bx, tup, r, n, flags);
    if (tcool) {
      BlCtx b;
      const double T = tup[n + r];
      sg_tuple_ctx(bx, tup[r], T, tup[2 * n + r], tup[3 * n + r], b);
      bl_prepare(b, T);
      tcool[r] = b.E / fabs(b.hc_init);
    }
  }
}

__global__ void k_sg_prep(SgBox bx, const double *__restrict__ tup, const double *__restrict__ tnew,
                          long n, float4 *__restrict__ feat, float *__restrict__ target,
                          int *__restrict__ inbox)
{
  for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < n; r += (long)gridDim.x * blockDim.x) {
    float x[4];
    const double T = tup[n + r];
    const bool in = sg_features(bx, tup[r], T, tup[2 * n + r], tup[3 * n + r], x);
    feat[r] = make_float4(x[0], x[1], x[2], x[3]);
    target[r] = (float)((log10(tnew[r]) - log10(T)) * 0.25);
    inbox[r] = in && T >= 1.e4;
  }
}

__global__ void __launch_bounds__(128) k_sg_predict(SgNet net, SgBox bx, const double *__restrict__ tup,
                                                    long n, int use_net, double *__restrict__ tout,
                                                    int *__restrict__ status, double *__restrict__ t0out,
                                                    int *queue, int *qcount,
                                                    unsigned long long *stats, unsigned *flags)
{
  extern __shared__ __align__(1024) unsigned char smem[];
  const uint32_t tmem = sg_inf_setup(net, smem);
  const long r = blockIdx.x * (long)kSgRows + threadIdx.x;
  const bool active = r < n;
  SgCtx b;
  double T = 0.0;
  float x[4] = {0.f, 0.f, 0.f, 0.f};
  bool inbox = false;
  int st = SG_BELOW_MIN;
  if (active) {
    T = tup[n + r];
    b.nH = tup[r];
    b.n = b.nH * 1.43 / bx.mu;
    b.E = T * b.n * kKB * 1.5;
    b.xi = tup[2 * n + r];
    b.tx = bx.t_x;
    b.dt = tup[3 * n + r];
    if (T >= 1.e4) {
      st = SG_OUT_OF_BOX;
      inbox = sg_features(bx, tup[r], T, tup[2 * n + r], tup[3 * n + r], x);
      if (!inbox) x[0] = x[1] = x[2] = x[3] = 0.f;
    }
  }
  uint32_t phase = 0;
  float y = 0.f;
  const bool ok = sg_forward(smem, tmem, phase, x, 0, 0, y);
  if (!ok && threadIdx.x == 0) atomicOr(flags, F_TMA_TIMEOUT);
  double T0 = 0.0;
  int evals = 0;
  bool stiff = false;
  if (active) {
    if (st != SG_BELOW_MIN) {
      double T_f = 0.0;
      st = ok ? sg_decide(b, T, inbox, y, use_net, T_f, T0, evals, stiff) : SG_REJECT;
      if (st == SG_ACCEPT) {
        tout[r] = dmax(T_f, 1.e4);
      } else {
        const int k = atomicAdd(qcount, 1);
        queue[k] = (int)r;
      }
    } else {
      tout[r] = T;
    }
    status[r] = st;
    if (t0out) t0out[r] = T0;
  }
  sg_count(st, active, evals, stiff, stats);
  sg_inf_teardown(tmem);
}

__global__ void k_sg_fallback_tuples(SgBox bx, const double *__restrict__ tup, long n,
                                     const int *__restrict__ queue, const int *__restrict__ qcount,
                                     double *__restrict__ tout, unsigned *flags)
{
  const int cnt = *qcount;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < cnt; k += gridDim.x * blockDim.x) {
    const long r = queue[k];
    tout[r] = sg_tuple_solve(bx, tup, r, n, flags);
  }
}

// ------------------------------------------------------------------
// the wind's split-source step with the surrogate
// ------------------------------------------------------------------

__global__ void __launch_bounds__(128) k_sg_cool(SgNet net, SgBox bx, SgCoolArgs A,
                                                 const BlockItem *__restrict__ items, int nitems,
                                                 int use_net, int2 *queue, int *qcount,
                                                 unsigned long long *stats)
{
  extern __shared__ __align__(1024) unsigned char smem[];
  if (A.sc->done) return;
  auto args_of = [&](int) { return A; };
  sg_cool_items(net, bx, args_of, items, nitems, use_net, smem, queue, qcount, stats);
}

__global__ void k_sg_cool_fallback(SgCoolArgs A, const int2 *__restrict__ queue,
                                   const int *__restrict__ qcount)
{
  if (A.sc->done) return;
  const int cnt = *qcount;
  const double dt = A.sc->dt, t = A.sc->t;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < cnt; k += gridDim.x * blockDim.x)
    blondin_cell(A.V, A.xi, A.tr, A.p, A.w, A.x1, A.sc, dt, t, queue[k].y, A.pre);
}

// (n_H, T, xi, dt_s) of every cell BLONDIN would solve now.
__global__ void k_sg_collect(SgCoolArgs A, double *__restrict__ out, long cap, int *count)
{
  const long long ncell = (long long)A.p.nx[0] * A.p.nx[1] * A.p.nx[2];
  const double dt = A.sc->dt, t = A.sc->t;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < ncell;
       q += (long long)gridDim.x * blockDim.x) {
    BlCtx b;
    double T;
    long long c;
    if (!blondin_ctx(A.V, A.xi, A.tr, A.p, A.w, A.x1, dt, t, q, b, T, c, A.pre)) continue;
    const int k = atomicAdd(count, 1);
    if (k < cap) {
      out[4 * k] = b.nH;
      out[4 * k + 1] = T;
      out[4 * k + 2] = b.xi;
      out[4 * k + 3] = b.dt_share;
    }
  }
}

}  // namespace ps

// ------------------------------------------------------------------
// host side
// ------------------------------------------------------------------

struct ps_surrogate {
  ps::SgBox box;
  float *prm = nullptr, *m1 = nullptr, *m2 = nullptr;  // master parameters and Adam moments
  __nv_bfloat16 *w1b = nullptr, *w2b = nullptr, *w2tb = nullptr;
  float *small = nullptr;
  float *grad = nullptr;
  // training set
  float4 *feat = nullptr;
  float *target = nullptr;
  int *inbox = nullptr;
  int *idx = nullptr;
  long ndata = 0;
  std::vector<int> train_rows;  // rows inside the box
  float *gpart = nullptr, *lpart = nullptr, *loss = nullptr;
  int gpart_blocks = 0;
  long long adam_t = 0;
  unsigned long long *stats = nullptr;
  unsigned *flags = nullptr;
  cudaStream_t stream = nullptr;
  ps::SgNet net() const { return ps::SgNet{w1b, w2b, w2tb, small}; }
};

// accessors for the batched kernels
ps::SgNet ps_sg_net(const ps_surrogate *s) { return s->net(); }
ps::SgBox ps_sg_boxv(const ps_surrogate *s) { return s->box; }
unsigned long long *ps_sg_stats_dev(ps_surrogate *s) { return s->stats; }

static int sg_fail(const char *msg)
{
  ps_set_error_msg(msg);
  return PS_EINVAL;
}

static int sg_cuda(cudaError_t e, const char *where)
{
  char buf[512];
  std::snprintf(buf, sizeof(buf), "%s: %s", where, cudaGetErrorString(e));
  ps_set_error_msg(buf);
  return PS_ECUDA;
}

#define SCK(call)                                        \
  do {                                                   \
    cudaError_t e_ = (call);                             \
    if (e_ != cudaSuccess) return sg_cuda(e_, #call);    \
  } while (0)

static int sg_attrs()
{
  static bool done = false;
  if (done) return 0;
  SCK(cudaFuncSetAttribute(ps::k_sg_train_tile, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           ps::kTrBytes));
  SCK(cudaFuncSetAttribute(ps::k_sg_predict, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           ps::kInfBytes));
  SCK(cudaFuncSetAttribute(ps::k_sg_cool, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           ps::kInfBytes));
  done = true;
  return 0;
}

static void sg_free(ps_surrogate *s)
{
  if (!s) return;
  cudaFree(s->prm);
  cudaFree(s->m1);
  cudaFree(s->m2);
  cudaFree(s->w1b);
  cudaFree(s->w2b);
  cudaFree(s->w2tb);
  cudaFree(s->small);
  cudaFree(s->grad);
  cudaFree(s->feat);
  cudaFree(s->target);
  cudaFree(s->inbox);
  cudaFree(s->idx);
  cudaFree(s->gpart);
  cudaFree(s->lpart);
  cudaFree(s->loss);
  cudaFree(s->stats);
  cudaFree(s->flags);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
}

// the bf16/FP32 copies from the master parameters (no update)
static int sg_refresh(ps_surrogate *s)
{
  ps::k_sg_adam<<<(ps::kSgParams + 255) / 256, 256, 0, s->stream>>>(
      s->prm, s->m1, s->m2, s->gpart, 0, 0.f, 1.f, 1.f, 0, nullptr, s->w1b, s->w2b, s->w2tb, s->small);
  SCK(cudaGetLastError());
  return 0;
}

extern "C" int ps_sg_create(const ps_sg_box *box, ps_surrogate **out)
{
  if (!box || !out) return sg_fail("ps_sg_create: null argument");
  *out = nullptr;
  for (int i = 0; i < 4; i++)
    if (!(box->hi[i] > box->lo[i])) return sg_fail("ps_sg_create: empty box");
  if (!(box->t_x > 0) || !(box->mu > 0)) return sg_fail("ps_sg_create: bad t_x / mu");
  int r = sg_attrs();
  if (r) return r;
  ps_surrogate *s = new ps_surrogate();
  for (int i = 0; i < 4; i++) {
    s->box.lo[i] = box->lo[i];
    s->box.hi[i] = box->hi[i];
    s->box.scale[i] = 2.0 / (box->hi[i] - box->lo[i]);
  }
  s->box.t_x = box->t_x;
  s->box.mu = box->mu;
  cudaError_t e;
  const size_t P = sizeof(float) * ps::kSgParams;
  if ((e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaMalloc(&s->prm, P)) != cudaSuccess || (e = cudaMalloc(&s->m1, P)) != cudaSuccess ||
      (e = cudaMalloc(&s->m2, P)) != cudaSuccess || (e = cudaMalloc(&s->grad, P)) != cudaSuccess ||
      (e = cudaMalloc(&s->w1b, 2 * ps::kSgH * ps::kSgK1)) != cudaSuccess ||
      (e = cudaMalloc(&s->w2b, 2 * ps::kSgH * ps::kSgH)) != cudaSuccess ||
      (e = cudaMalloc(&s->w2tb, 2 * ps::kSgH * ps::kSgH)) != cudaSuccess ||
      (e = cudaMalloc(&s->small, sizeof(float) * ps::kSgSmall)) != cudaSuccess ||
      (e = cudaMalloc(&s->loss, sizeof(float) * 2)) != cudaSuccess ||
      (e = cudaMalloc(&s->stats, sizeof(unsigned long long) * 6)) != cudaSuccess ||
      (e = cudaMalloc(&s->flags, sizeof(unsigned))) != cudaSuccess) {
    sg_free(s);
    return sg_cuda(e, "ps_sg_create");
  }
  cudaMemset(s->w1b, 0, 2 * ps::kSgH * ps::kSgK1);
  cudaMemset(s->m1, 0, P);
  cudaMemset(s->m2, 0, P);
  cudaMemset(s->stats, 0, sizeof(unsigned long long) * 6);
  cudaMemset(s->flags, 0, sizeof(unsigned));
  // default initialisation: uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)), seed 3
  std::vector<float> p(ps::kSgParams, 0.f);
  std::mt19937_64 rng(3);
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  for (int i = 0; i < 256; i++) p[ps::kSgW1 + i] = (float)(U(rng) / std::sqrt(4.0));
  for (int i = 0; i < 64; i++) p[ps::kSgB1 + i] = (float)(U(rng) / std::sqrt(4.0));
  for (int i = 0; i < 4096; i++) p[ps::kSgW2 + i] = (float)(U(rng) / 8.0);
  for (int i = 0; i < 64; i++) p[ps::kSgB2 + i] = (float)(U(rng) / 8.0);
  for (int i = 0; i < 64; i++) p[ps::kSgW3 + i] = (float)(U(rng) / 8.0);
  p[ps::kSgB3] = 0.f;
  cudaMemcpy(s->prm, p.data(), P, cudaMemcpyHostToDevice);
  if ((r = sg_refresh(s)) != 0 || (e = cudaStreamSynchronize(s->stream)) != cudaSuccess) {
    sg_free(s);
    return r ? r : sg_cuda(e, "ps_sg_create");
  }
  *out = s;
  return 0;
}

extern "C" int ps_sg_destroy(ps_surrogate *s)
{
  if (!s) return PS_EINVAL;
  cudaStreamSynchronize(s->stream);
  sg_free(s);
  return 0;
}

extern "C" int ps_sg_set_params(ps_surrogate *s, const float *p)
{
  if (!s || !p) return sg_fail("ps_sg_set_params: null argument");
  SCK(cudaMemcpyAsync(s->prm, p, sizeof(float) * ps::kSgParams, cudaMemcpyHostToDevice, s->stream));
  SCK(cudaMemsetAsync(s->m1, 0, sizeof(float) * ps::kSgParams, s->stream));
  SCK(cudaMemsetAsync(s->m2, 0, sizeof(float) * ps::kSgParams, s->stream));
  s->adam_t = 0;
  int r = sg_refresh(s);
  if (r) return r;
  SCK(cudaStreamSynchronize(s->stream));
  return 0;
}

extern "C" int ps_sg_get_params(const ps_surrogate *s, float *p)
{
  if (!s || !p) return sg_fail("ps_sg_get_params: null argument");
  SCK(cudaStreamSynchronize(s->stream));
  SCK(cudaMemcpy(p, s->prm, sizeof(float) * ps::kSgParams, cudaMemcpyDeviceToHost));
  return 0;
}

// A trained network on disk: the tag "PSSGNET1", the box (lo[4], hi[4],
// t_x, mu: ten doubles), the parameter count (a 32-bit integer, 4545) and
// the parameters (FP32, the layout of ps_sg_set_params), little-endian.
static const char kSgTag[8] = {'P', 'S', 'S', 'G', 'N', 'E', 'T', '1'};

static bool sg_little_endian()
{
  const uint32_t one = 1;
  unsigned char b;
  std::memcpy(&b, &one, 1);
  return b == 1;
}

extern "C" int ps_sg_save(const ps_surrogate *s, const char *path)
{
  if (!s || !path) return sg_fail("ps_sg_save: null argument");
  if (!sg_little_endian()) return sg_fail("ps_sg_save: big-endian host not supported");
  std::vector<float> prm(ps::kSgParams);
  if (int r = ps_sg_get_params(s, prm.data())) return r;
  double hdr[10];
  for (int i = 0; i < 4; i++) {
    hdr[i] = s->box.lo[i];
    hdr[4 + i] = s->box.hi[i];
  }
  hdr[8] = s->box.t_x;
  hdr[9] = s->box.mu;
  const int32_t n = ps::kSgParams;
  FILE *f = std::fopen(path, "wb");
  if (!f) return sg_fail("ps_sg_save: cannot open the file");
  bool ok = std::fwrite(kSgTag, 1, 8, f) == 8 && std::fwrite(hdr, sizeof(double), 10, f) == 10 &&
            std::fwrite(&n, sizeof(n), 1, f) == 1 &&
            std::fwrite(prm.data(), sizeof(float), (size_t)n, f) == (size_t)n;
  ok = std::fclose(f) == 0 && ok;
  return ok ? 0 : sg_fail("ps_sg_save: write failed");
}

extern "C" int ps_sg_load(const char *path, ps_surrogate **out)
{
  if (!path || !out) return sg_fail("ps_sg_load: null argument");
  *out = nullptr;
  if (!sg_little_endian()) return sg_fail("ps_sg_load: big-endian host not supported");
  FILE *f = std::fopen(path, "rb");
  if (!f) return sg_fail("ps_sg_load: cannot open the file");
  char tag[8];
  double hdr[10];
  int32_t n = 0;
  std::vector<float> prm(ps::kSgParams);
  bool ok = std::fread(tag, 1, 8, f) == 8 && std::memcmp(tag, kSgTag, 8) == 0 &&
            std::fread(hdr, sizeof(double), 10, f) == 10 && std::fread(&n, sizeof(n), 1, f) == 1 &&
            n == ps::kSgParams &&
            std::fread(prm.data(), sizeof(float), (size_t)n, f) == (size_t)n &&
            std::fgetc(f) == EOF;
  std::fclose(f);
  if (!ok) return sg_fail("ps_sg_load: not a network file of this library (tag, size)");
  ps_sg_box box;
  for (int i = 0; i < 4; i++) {
    box.lo[i] = hdr[i];
    box.hi[i] = hdr[4 + i];
  }
  box.t_x = hdr[8];
  box.mu = hdr[9];
  ps_surrogate *s = nullptr;
  if (int r = ps_sg_create(&box, &s)) return r;
  if (int r = ps_sg_set_params(s, prm.data())) {
    ps_sg_destroy(s);
    return r;
  }
  *out = s;
  return 0;
}

// device copy of host tuples (row-major n x 4) as SoA
static int sg_upload_tuples(ps_surrogate *s, const double *tuples, long n, double **d)
{
  std::vector<double> soa((size_t)4 * n);
  for (long r = 0; r < n; r++)
    for (int k = 0; k < 4; k++) soa[(size_t)k * n + r] = tuples[4 * r + k];
  SCK(cudaMalloc(d, sizeof(double) * 4 * n));
  SCK(cudaMemcpyAsync(*d, soa.data(), sizeof(double) * 4 * n, cudaMemcpyHostToDevice, s->stream));
  SCK(cudaStreamSynchronize(s->stream));
  return 0;
}

extern "C" int ps_sg_label(ps_surrogate *s, const double *tuples, long n, double *t_new,
                           double *t_cool)
{
  if (!s || !tuples || !t_new || n <= 0) return sg_fail("ps_sg_label: bad arguments");
  double *d = nullptr, *o = nullptr, *tc = nullptr;
  int r = sg_upload_tuples(s, tuples, n, &d);
  if (r) return r;
  cudaError_t e = cudaMalloc(&o, sizeof(double) * n);
  if (e == cudaSuccess && t_cool) e = cudaMalloc(&tc, sizeof(double) * n);
  if (e == cudaSuccess) {
    ps::k_sg_label<<<1216, 128, 0, s->stream>>>(s->box, d, n, o, tc, s->flags);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(t_new, o, sizeof(double) * n, cudaMemcpyDeviceToHost, s->stream);
  if (e == cudaSuccess && t_cool)
    e = cudaMemcpyAsync(t_cool, tc, sizeof(double) * n, cudaMemcpyDeviceToHost, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  cudaFree(d);
  cudaFree(o);
  cudaFree(tc);
  if (e != cudaSuccess) return sg_cuda(e, "ps_sg_label");
  return 0;
}

extern "C" int ps_sg_set_data(ps_surrogate *s, const double *tuples, const double *t_new, long n)
{
  if (!s || !tuples || !t_new || n <= 0) return sg_fail("ps_sg_set_data: bad arguments");
  cudaStreamSynchronize(s->stream);
  cudaFree(s->feat);
  cudaFree(s->target);
  cudaFree(s->inbox);
  cudaFree(s->idx);
  s->feat = nullptr;
  s->target = nullptr;
  s->inbox = nullptr;
  s->idx = nullptr;
  s->ndata = 0;
  double *d = nullptr, *tn = nullptr;
  int r = sg_upload_tuples(s, tuples, n, &d);
  if (r) return r;
  SCK(cudaMalloc(&tn, sizeof(double) * n));
  SCK(cudaMalloc(&s->feat, sizeof(float4) * n));
  SCK(cudaMalloc(&s->target, sizeof(float) * n));
  SCK(cudaMalloc(&s->inbox, sizeof(int) * n));
  SCK(cudaMalloc(&s->idx, sizeof(int) * n));
  SCK(cudaMemcpyAsync(tn, t_new, sizeof(double) * n, cudaMemcpyHostToDevice, s->stream));
  ps::k_sg_prep<<<1216, 128, 0, s->stream>>>(s->box, d, tn, n, s->feat, s->target, s->inbox);
  SCK(cudaGetLastError());
  std::vector<int> inb(n);
  SCK(cudaMemcpyAsync(inb.data(), s->inbox, sizeof(int) * n, cudaMemcpyDeviceToHost, s->stream));
  SCK(cudaStreamSynchronize(s->stream));
  cudaFree(d);
  cudaFree(tn);
  s->train_rows.clear();
  for (long i = 0; i < n; i++)
    if (inb[i]) s->train_rows.push_back((int)i);
  s->ndata = n;
  if (s->train_rows.empty()) return sg_fail("ps_sg_set_data: no tuple inside the box");
  return 0;
}

static int sg_ensure_gpart(ps_surrogate *s, int nblk)
{
  if (nblk <= s->gpart_blocks) return 0;
  cudaFree(s->gpart);
  cudaFree(s->lpart);
  s->gpart = nullptr;
  s->lpart = nullptr;
  SCK(cudaMalloc(&s->gpart, sizeof(float) * ps::kSgParams * (size_t)nblk));
  SCK(cudaMalloc(&s->lpart, sizeof(float) * (size_t)nblk));
  s->gpart_blocks = nblk;
  return 0;
}

// One forward/backward over rows idx[0..nrows) of the data set.
static int sg_fwd_bwd(ps_surrogate *s, const int *d_idx, int nrows)
{
  const int nblk = (nrows + ps::kSgRows - 1) / ps::kSgRows;
  int r = sg_ensure_gpart(s, nblk);
  if (r) return r;
  SCK(cudaMemsetAsync(s->lpart, 0, sizeof(float) * nblk, s->stream));
  ps::k_sg_train_tile<<<nblk, 128, ps::kTrBytes, s->stream>>>(
      s->net(), s->feat, s->target, d_idx, nrows, 1.0f / (float)nrows, s->gpart, s->lpart, s->flags);
  SCK(cudaGetLastError());
  ps::k_sg_loss<<<1, 256, 0, s->stream>>>(s->lpart, nblk, 1.0f / (float)nrows, s->loss);
  SCK(cudaGetLastError());
  return 0;
}

extern "C" int ps_sg_train(ps_surrogate *s, int steps, int batch, float lr, float lr_end,
                           unsigned long long seed, float *loss_hist)
{
  if (!s || steps <= 0 || batch < 128 || batch % 128) return sg_fail("ps_sg_train: bad arguments");
  if (s->train_rows.empty()) return sg_fail("ps_sg_train: no data (ps_sg_set_data)");
  const long nt = (long)s->train_rows.size();
  if (batch > nt) batch = (int)(nt / 128 * 128);
  if (batch < 128) return sg_fail("ps_sg_train: fewer than 128 rows inside the box");
  const int nblk = batch / ps::kSgRows;
  int r = sg_ensure_gpart(s, nblk);
  if (r) return r;
  std::mt19937_64 rng(seed);
  std::vector<int> perm(s->train_rows);
  long pos = nt;  // reshuffle at the first step
  float *d_hist = nullptr;
  SCK(cudaMalloc(&d_hist, sizeof(float) * steps));
  for (int it = 0; it < steps; it++) {
    if (pos + batch > nt) {
      std::shuffle(perm.begin(), perm.end(), rng);
      SCK(cudaMemcpyAsync(s->idx, perm.data(), sizeof(int) * nt, cudaMemcpyHostToDevice, s->stream));
      // the copy must land before the host vector changes again
      SCK(cudaStreamSynchronize(s->stream));
      pos = 0;
    }
    r = sg_fwd_bwd(s, s->idx + pos, batch);
    if (r) {
      cudaFree(d_hist);
      return r;
    }
    pos += batch;
    s->adam_t++;
    const double frac = steps > 1 ? (double)it / (steps - 1) : 0.0;
    const float lr_t = (float)(lr_end + 0.5 * (lr - lr_end) * (1.0 + std::cos(M_PI * frac)));
    const float bc1 = (float)(1.0 - std::pow(0.9, (double)s->adam_t));
    const float bc2 = (float)(1.0 - std::pow(0.999, (double)s->adam_t));
    ps::k_sg_adam<<<(ps::kSgParams + 255) / 256, 256, 0, s->stream>>>(
        s->prm, s->m1, s->m2, s->gpart, nblk, lr_t, bc1, bc2, 1, nullptr, s->w1b, s->w2b, s->w2tb,
        s->small);
    SCK(cudaGetLastError());
    SCK(cudaMemcpyAsync(d_hist + it, s->loss, sizeof(float), cudaMemcpyDeviceToDevice, s->stream));
  }
  if (loss_hist)
    SCK(cudaMemcpyAsync(loss_hist, d_hist, sizeof(float) * steps, cudaMemcpyDeviceToHost, s->stream));
  SCK(cudaStreamSynchronize(s->stream));
  cudaFree(d_hist);
  unsigned f = 0;
  SCK(cudaMemcpy(&f, s->flags, sizeof(unsigned), cudaMemcpyDeviceToHost));
  return (int)f;
}

extern "C" int ps_sg_grad(ps_surrogate *s, const double *tuples, const double *t_new, int n,
                          float *grad, float *loss)
{
  if (!s || !tuples || !t_new || n <= 0 || !grad) return sg_fail("ps_sg_grad: bad arguments");
  int r = ps_sg_set_data(s, tuples, t_new, n);
  if (r) return r;
  std::vector<int> id(n);
  for (int i = 0; i < n; i++) id[i] = i;
  SCK(cudaMemcpyAsync(s->idx, id.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s->stream));
  r = sg_fwd_bwd(s, s->idx, n);
  if (r) return r;
  const int nblk = (n + ps::kSgRows - 1) / ps::kSgRows;
  ps::k_sg_adam<<<(ps::kSgParams + 255) / 256, 256, 0, s->stream>>>(
      s->prm, s->m1, s->m2, s->gpart, nblk, 0.f, 1.f, 1.f, 0, s->grad, s->w1b, s->w2b, s->w2tb,
      s->small);
  SCK(cudaGetLastError());
  SCK(cudaMemcpyAsync(grad, s->grad, sizeof(float) * ps::kSgParams, cudaMemcpyDeviceToHost, s->stream));
  if (loss) SCK(cudaMemcpyAsync(loss, s->loss, sizeof(float), cudaMemcpyDeviceToHost, s->stream));
  SCK(cudaStreamSynchronize(s->stream));
  unsigned f = 0;
  SCK(cudaMemcpy(&f, s->flags, sizeof(unsigned), cudaMemcpyDeviceToHost));
  return (int)f;
}

extern "C" int ps_sg_predict(ps_surrogate *s, const double *tuples, long n, int use_net,
                             double *t_out, int *status, double *t_mlp)
{
  if (!s || !tuples || n <= 0 || !t_out || !status) return sg_fail("ps_sg_predict: bad arguments");
  if (n > 0x7fffffffL) return sg_fail("ps_sg_predict: too many tuples");
  double *d = nullptr, *o = nullptr, *t0 = nullptr;
  int *st = nullptr, *queue = nullptr, *qc = nullptr;
  int r = sg_upload_tuples(s, tuples, n, &d);
  if (r) return r;
  cudaError_t e;
  if ((e = cudaMalloc(&o, sizeof(double) * n)) != cudaSuccess ||
      (e = cudaMalloc(&t0, sizeof(double) * n)) != cudaSuccess ||
      (e = cudaMalloc(&st, sizeof(int) * n)) != cudaSuccess ||
      (e = cudaMalloc(&queue, sizeof(int) * n)) != cudaSuccess ||
      (e = cudaMalloc(&qc, sizeof(int))) != cudaSuccess) {
    cudaFree(d);
    cudaFree(o);
    cudaFree(t0);
    cudaFree(st);
    cudaFree(queue);
    return sg_cuda(e, "ps_sg_predict");
  }
  cudaMemsetAsync(qc, 0, sizeof(int), s->stream);
  const unsigned nblk = (unsigned)((n + ps::kSgRows - 1) / ps::kSgRows);
  ps::k_sg_predict<<<nblk, 128, ps::kInfBytes, s->stream>>>(s->net(), s->box, d, n, use_net, o, st,
                                                            t0, queue, qc, s->stats, s->flags);
  e = cudaGetLastError();
  if (e == cudaSuccess) {
    ps::k_sg_fallback_tuples<<<1216, 128, 0, s->stream>>>(s->box, d, n, queue, qc, o, s->flags);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(t_out, o, sizeof(double) * n, cudaMemcpyDeviceToHost, s->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(status, st, sizeof(int) * n, cudaMemcpyDeviceToHost, s->stream);
  if (e == cudaSuccess && t_mlp)
    e = cudaMemcpyAsync(t_mlp, t0, sizeof(double) * n, cudaMemcpyDeviceToHost, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  cudaFree(d);
  cudaFree(o);
  cudaFree(t0);
  cudaFree(st);
  cudaFree(queue);
  cudaFree(qc);
  if (e != cudaSuccess) return sg_cuda(e, "ps_sg_predict");
  unsigned f = 0;
  SCK(cudaMemcpy(&f, s->flags, sizeof(unsigned), cudaMemcpyDeviceToHost));
  return (int)f;
}

extern "C" int ps_sg_stats(ps_surrogate *s, long long *out, int reset)
{
  if (!s || !out) return sg_fail("ps_sg_stats: null argument");
  SCK(cudaDeviceSynchronize());
  unsigned long long h[6];
  SCK(cudaMemcpy(h, s->stats, sizeof(h), cudaMemcpyDeviceToHost));
  for (int i = 0; i < 6; i++) out[i] = (long long)h[i];
  if (reset) SCK(cudaMemset(s->stats, 0, sizeof(h)));
  return 0;
}

// ------------------------------------------------------------------
// wind contexts
// ------------------------------------------------------------------

static ps::SgCoolArgs sg_cool_args(ps_ctx *c)
{
  ps::SgCoolArgs A;
  A.V = c->V;
  A.p = c->p;
  A.sc = c->sc;
  if (c->wind) {
    A.xi = c->wind->xi;
    A.tr = c->wind->tr;
    A.x1 = c->wind->a.g.x1;
    A.pre = c->wind->pre;
    A.w = c->wind->a.w;
  } else {  // Cartesian cooling at constant xi
    A.xi = A.tr = A.x1 = A.pre = nullptr;
    A.w = c->coolw;
  }
  return A;
}

static long long ctx_cells(const ps_ctx *c)
{
  return (long long)c->p.nx[0] * c->p.nx[1] * c->p.nx[2];
}

void ps_ctx_invalidate_graphs(ps_ctx *c);

extern "C" int ps_set_surrogate(ps_ctx *c, ps_surrogate *s, int use_net)
{
  if (!c) return sg_fail("ps_set_surrogate: null context");
  if (s && !c->wind && !c->cool_on)
    return sg_fail("ps_set_surrogate: needs ps_set_wind or ps_set_cooling first");
  if (s && c->p.cooling == 2)
    return sg_fail("ps_set_surrogate: the learned step replaces BLONDIN's implicit solve, not "
                   "the ODE cooling path");
  SCK(cudaStreamSynchronize(c->stream));
  if (s) SCK(cudaStreamSynchronize(s->stream));
  if (s && !c->sg_queue) {
    const size_t ncell = (size_t)ctx_cells(c);
    const int nblk = (int)((ncell + ps::kSgRows - 1) / ps::kSgRows);
    std::vector<ps::BlockItem> items(nblk);
    for (int k = 0; k < nblk; k++) items[k] = ps::BlockItem{0, k};
    SCK(cudaMalloc(&c->sg_queue, sizeof(int2) * ncell));
    SCK(cudaMalloc(&c->sg_qcount, sizeof(int)));
    SCK(cudaMalloc(&c->sg_items, sizeof(ps::BlockItem) * nblk));
    SCK(cudaMemcpy(c->sg_items, items.data(), sizeof(ps::BlockItem) * nblk, cudaMemcpyHostToDevice));
  }
  c->sg = s;
  c->sg_use_net = use_net;
  ps_ctx_invalidate_graphs(c);
  return 0;
}

// The split-source launches of a context with a surrogate.
int ps_sg_cool_launch(ps_ctx *c)
{
  ps_surrogate *s = c->sg;
  const ps::SgCoolArgs A = sg_cool_args(c);
  const long long ncell = ctx_cells(c);
  SCK(cudaMemsetAsync(c->sg_qcount, 0, sizeof(int), c->stream));
  const int nblk = (int)((ncell + ps::kSgRows - 1) / ps::kSgRows);
  int dev = 0, nsm = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  ps::k_sg_cool<<<std::min(nblk, nsm * ps::kInfCtasPerSm), 128, ps::kInfBytes, c->stream>>>(
      s->net(), s->box, A, reinterpret_cast<const ps::BlockItem *>(c->sg_items), nblk,
      c->sg_use_net, reinterpret_cast<int2 *>(c->sg_queue), c->sg_qcount, s->stats);
  // one warp per CTA: the few queued cells spread over every SM
  ps::k_sg_cool_fallback<<<2432, 32, 0, c->stream>>>(A, reinterpret_cast<int2 *>(c->sg_queue),
                                                     c->sg_qcount);
  c->launches += 2;
  SCK(cudaGetLastError());
  return 0;
}

void ps_sg_free_ctx(ps_ctx *c)
{
  cudaFree(c->sg_queue);
  cudaFree(c->sg_qcount);
  cudaFree(c->sg_items);
  c->sg_queue = nullptr;
  c->sg_qcount = nullptr;
  c->sg_items = nullptr;
}

extern "C" int ps_sg_collect(ps_ctx *c, double *tuples, long cap, long *n)
{
  if (!c || !(c->wind || c->cool_on) || !tuples || !n || cap <= 0)
    return sg_fail("ps_sg_collect: bad arguments");
  SCK(cudaStreamSynchronize(c->stream));
  double *d = nullptr;
  int *cnt = nullptr;
  SCK(cudaMalloc(&d, sizeof(double) * 4 * cap));
  SCK(cudaMalloc(&cnt, sizeof(int)));
  cudaMemsetAsync(cnt, 0, sizeof(int), c->stream);
  ps::k_sg_collect<<<1216, 128, 0, c->stream>>>(sg_cool_args(c), d, cap, cnt);
  c->launches++;
  int h = 0;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, cnt, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  const long k = std::min<long>(h, cap);
  if (e == cudaSuccess && k > 0) e = cudaMemcpy(tuples, d, sizeof(double) * 4 * k, cudaMemcpyDeviceToHost);
  cudaFree(d);
  cudaFree(cnt);
  if (e != cudaSuccess) return sg_cuda(e, "ps_sg_collect");
  *n = k;
  return 0;
}
