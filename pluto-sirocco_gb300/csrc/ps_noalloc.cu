// ps_noalloc.cu -- ps_advance_step_noalloc(): one RK2 step of the hydro path
// for callers that cannot allocate device memory.
//
// Who needs it: host codes whose device memory is owned by someone else
// (a framework's caching allocator or a fixed memory pool that must not be
// fragmented), callers that run where cudaMalloc is not allowed (inside a
// region that must not synchronise the device, which cudaMalloc/cudaFree
// may do), and plugin hosts that forbid a library from holding private
// allocations.  They pass the state in their own device buffer; the
// stage scratch (V*, U*, dt/dx, 1/dx and the step scalars) lives in the
// file-scope array below, which every GPU that loads this library holds
// until the process exits.
//
// Limits: at most kNaMaxCells total-box cells per variable (ghost zones
// included), at most kNaMaxVars variables, at most kNaMaxDir cells per
// direction, and an even total-box row length (the tile copies need
// 16-byte row strides).  Larger requests are rejected with PS_EINVAL.
//
// Sharing: every call on a device uses the same array and leaves the last
// call's contents in it; each call rewrites everything it reads before
// reading it (the scalars, the C_dt maximum, dt/dx, 1/dx), so no state
// leaks between calls.  Calls whose work overlaps on the GPU (concurrent
// streams, or several host threads) race on the array and must be
// serialised by the caller.
//
// Set-up: the first call on a device looks up the device address of the
// array with cudaGetSymbolAddress (with that device current) and keeps it.
//
// Streams: every call copies the dx arrays in from pageable host memory and
// waits for its stream before it returns (the flags and invDt_hyp are read
// back), so it cannot be called while that stream is being captured.
#include "ps_gb300.h"
#include "ps_hydro.cuh"
#include "ps_physics.cuh"

#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cstdio>
#include <cstring>
#include <mutex>

namespace ps {
const void *stage_kernel_2d(int nv, int lim, int solver, int stage);
const void *stage_kernel_3d(int nv, int lim, int solver, int stage);
size_t stage_smem_2d(int nv);
size_t stage_smem_3d(int nv);
void stage_tile_2d(int *t);
void stage_tile_3d(int *t);
void fill_ghosts_2d(double *V, const Params &p, cudaStream_t s);
void fill_ghosts_3d(double *V, const Params &p, cudaStream_t s);
__global__ void k_finish(FinishArgs f);
}  // namespace ps

extern "C" void ps_set_error_msg(const char *msg);

namespace {

constexpr long long kNaMaxCells = 32768;  // total-box cells per variable
constexpr int kNaMaxVars = 6;
constexpr int kNaMaxDir = 2048;           // total-box cells per direction
constexpr int kNaMaxDevices = 64;

// Layout of the scratch array (in doubles):
//   [0, V)        V*  (stage-1 primitive state)       kNaMaxVars * kNaMaxCells
//   [V, 2V)       U*  (stage-1 conservative state)    kNaMaxVars * kNaMaxCells
//   then dx, 1/dx, dt/dx for 3 directions             9 * kNaMaxDir
//   then the step scalars                             32 (room for ps::Scalars)
constexpr long long kNaStateDoubles = (long long)kNaMaxVars * kNaMaxCells;
constexpr long long kNaGridOffset = 2 * kNaStateDoubles;
constexpr long long kNaScalarOffset = kNaGridOffset + 9LL * kNaMaxDir;
constexpr long long kNaTotalDoubles = kNaScalarOffset + 32;
static_assert(sizeof(ps::Scalars) <= 32 * sizeof(double), "scalars do not fit");
static_assert((kNaGridOffset * sizeof(double)) % 256 == 0, "grid region alignment");
static_assert((kNaStateDoubles * sizeof(double)) % 256 == 0, "state region alignment");

// 3.3 MB of device memory per GPU that loads the library.
static __device__ __align__(256) double g_noalloc_scratch[kNaTotalDoubles];

struct NaDevice {
  bool ready;
  double *base;  // device address of g_noalloc_scratch on this device
};
NaDevice g_na_dev[kNaMaxDevices];
std::mutex g_na_mutex;

int na_error(const char *msg)
{
  ps_set_error_msg(msg);
  return PS_EINVAL;
}

int na_cuda(cudaError_t e, const char *where)
{
  char buf[512];
  std::snprintf(buf, sizeof(buf), "ps_advance_step_noalloc: %s: %s", where,
                cudaGetErrorString(e));
  ps_set_error_msg(buf);
  return PS_ECUDA;
}

// Scalars of the step and the per-direction dt/dx and 1/dx, recomputed on
// every call from the dx arrays copied in by the host.
__global__ void k_na_prepare(double *base, ps::Params p, double dt, double inv_in)
{
  ps::Scalars *sc = reinterpret_cast<ps::Scalars *>(base + kNaScalarOffset);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    sc->t = 0.0;
    sc->dt = dt;
    sc->inv_dt_hyp = inv_in;
    sc->dt_cool = 1.e38;
    sc->step = -1;  // no per-step history in this entry point
    sc->last = 0;
    sc->done = 0;
    sc->flags = 0;
    sc->cdt_bits = 0ull;
  }
  for (int d = 0; d < p.dims; d++) {
    const double *dx = base + kNaGridOffset + (long long)d * kNaMaxDir;
    double *inv = base + kNaGridOffset + (3LL + d) * kNaMaxDir;
    double *dtdx = base + kNaGridOffset + (6LL + d) * kNaMaxDir;
    for (int i = threadIdx.x; i < p.ntot[d]; i += blockDim.x) {
      inv[i] = 1.0 / (dx[i]);
      dtdx[i] = dt / dx[i];
    }
  }
}

// The driver's tensor-map encoder, looked up once per process under the
// lock (two host threads making their first calls together would race on
// an unguarded static).
PFN_cuTensorMapEncodeTiled_v12000 g_na_encode = nullptr;

int na_encode(const ps::Params &p, const int *tile, double *base, CUtensorMap *tm)
{
  PFN_cuTensorMapEncodeTiled_v12000 encode;
  {
    std::lock_guard<std::mutex> lk(g_na_mutex);
    if (!g_na_encode) {
      cudaDriverEntryPointQueryResult q;
      void *fn = nullptr;
      cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                                       cudaEnableDefault, &q);
      if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn)
        return na_cuda(e == cudaSuccess ? cudaErrorNotSupported : e, "cuTensorMapEncodeTiled");
      g_na_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
    encode = g_na_encode;
  }
  cuuint64_t dims[4] = {(cuuint64_t)p.ntot[0], (cuuint64_t)p.ntot[1], (cuuint64_t)p.ntot[2],
                        (cuuint64_t)p.nvar};
  cuuint64_t strides[3] = {(cuuint64_t)p.px * 8, (cuuint64_t)p.px * p.ntot[1] * 8,
                           (cuuint64_t)p.vstride * 8};
  cuuint32_t box[4] = {(cuuint32_t)(tile[0] + 2 * tile[3]), (cuuint32_t)(tile[1] + 2 * tile[4]),
                       (cuuint32_t)(tile[2] + 2 * tile[5]), (cuuint32_t)p.nvar};
  cuuint32_t estr[4] = {1, 1, 1, 1};
  CUresult r = encode(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 4, base, dims, strides, box, estr,
                      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                      CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return na_error("ps_advance_step_noalloc: tensor map rejected");
  return 0;
}

}  // namespace

extern "C" int ps_advance_step_noalloc(const ps_config *cfg, const double *dx1, const double *dx2,
                                       const double *dx3, double *Vc_dev, double dt,
                                       double *inv_dt_hyp, void *stream)
{
  if (!cfg || !Vc_dev || !dx1 || !dx2 || (cfg->dims == 3 && !dx3))
    return na_error("ps_advance_step_noalloc: null argument");
  if ((cfg->dims != 2 && cfg->dims != 3) || cfg->nvar < 5 || cfg->nvar > kNaMaxVars ||
      cfg->geometry != PS_CARTESIAN || cfg->limiter < 0 || cfg->limiter > 2 ||
      (cfg->solver != PS_HLLC && cfg->solver != PS_HLL) || cfg->gamma <= 1.0)
    return na_error("ps_advance_step_noalloc: unsupported configuration");
  // as ps_create on a Cartesian context: these switches belong to the
  // spherical wind path (SHOCK_FLATTENING MULTID would also mean 3 ghost
  // zones per side, which this entry point does not lay out)
  if (cfg->char_limiting || cfg->shock_flattening || cfg->entropy_switch)
    return na_error("ps_advance_step_noalloc: characteristic limiting, shock flattening and "
                    "the entropy switch need a spherical wind context");
  ps::Params p;
  std::memset(&p, 0, sizeof(p));
  p.dims = cfg->dims;
  p.nvar = cfg->nvar;
  p.limiter = cfg->limiter;
  p.solver = cfg->solver;
  p.cooling = cfg->cooling;
  for (int d = 0; d < 3; d++) {
    if (d < cfg->dims && cfg->nx[d] < 4)
      return na_error("ps_advance_step_noalloc: at least 4 active cells per active direction");
    if (d >= cfg->dims && cfg->nx[d] != 1)
      return na_error("ps_advance_step_noalloc: inactive directions must have nx = 1");
    p.nx[d] = cfg->nx[d];
    p.beg[d] = d < cfg->dims ? 2 : 0;
    p.ntot[d] = cfg->nx[d] + 2 * p.beg[d];
    if (p.ntot[d] > kNaMaxDir)
      return na_error("ps_advance_step_noalloc: more than 2048 cells in one direction");
  }
  for (int s = 0; s < 2 * cfg->dims; s++) {
    const int b = cfg->bc[s];
    if (b != PS_BC_OUTFLOW && b != PS_BC_PERIODIC && b != PS_BC_REFLECTIVE &&
        b != PS_BC_AXISYM && b != PS_BC_EQTSYM)
      return na_error("ps_advance_step_noalloc: boundary type not supported on this path");
    if ((b == PS_BC_PERIODIC) != (cfg->bc[s ^ 1] == PS_BC_PERIODIC))
      return na_error("ps_advance_step_noalloc: periodic boundaries must be paired");
  }
  const long long cells = (long long)p.ntot[0] * p.ntot[1] * p.ntot[2];
  if (cells > kNaMaxCells)
    return na_error("ps_advance_step_noalloc: grid exceeds the 32768-cell scratch "
                    "(total box, ghost zones included)");
  if (p.ntot[0] % 2 != 0)
    return na_error("ps_advance_step_noalloc: total-box row length must be even");
  if (reinterpret_cast<uintptr_t>(Vc_dev) % 16 != 0)
    return na_error("ps_advance_step_noalloc: state buffer must be 16-byte aligned");
  for (int s = 0; s < 6; s++) p.bc[s] = cfg->bc[s];
  p.px = p.ntot[0];
  p.vstride = cells;
  p.gamma = cfg->gamma;
  p.gmm1 = cfg->gamma - 1.0;
  p.igmm1 = 1.0 / p.gmm1;
  p.cfl = cfg->cfl;
  p.cfl_max_var = cfg->cfl_max_var;
  p.tstop = cfg->tstop;
  p.first_dt = cfg->first_dt;

  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return na_cuda(e, "cudaGetDevice");
  if (dev < 0 || dev >= kNaMaxDevices) return na_error("ps_advance_step_noalloc: device index");
  double *base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_na_mutex);
    if (!g_na_dev[dev].ready) {
      void *ptr = nullptr;
      e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
      if (e != cudaSuccess) return na_cuda(e, "cudaGetSymbolAddress");
      g_na_dev[dev].base = static_cast<double *>(ptr);
      g_na_dev[dev].ready = true;
    }
    base = g_na_dev[dev].base;
  }

  int tile[6];
  size_t smem;
  const void *k1, *k2;
  if (p.dims == 2) {
    ps::stage_tile_2d(tile);
    smem = ps::stage_smem_2d(p.nvar);
    k1 = ps::stage_kernel_2d(p.nvar, p.limiter, p.solver, 1);
    k2 = ps::stage_kernel_2d(p.nvar, p.limiter, p.solver, 2);
  } else {
    ps::stage_tile_3d(tile);
    smem = ps::stage_smem_3d(p.nvar);
    k1 = ps::stage_kernel_3d(p.nvar, p.limiter, p.solver, 1);
    k2 = ps::stage_kernel_3d(p.nvar, p.limiter, p.solver, 2);
  }
  if (!k1 || !k2) return na_error("ps_advance_step_noalloc: no kernel for this configuration");
  if ((e = cudaFuncSetAttribute(k1, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
          cudaSuccess ||
      (e = cudaFuncSetAttribute(k2, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
          cudaSuccess)
    return na_cuda(e, "cudaFuncSetAttribute");

  double *Vs = base;
  double *Us = base + kNaStateDoubles;
  double *grid = base + kNaGridOffset;
  ps::Scalars *sc = reinterpret_cast<ps::Scalars *>(base + kNaScalarOffset);
  cudaStream_t st = static_cast<cudaStream_t>(stream);

  CUtensorMap tmV, tmVs;
  int r = na_encode(p, tile, Vc_dev, &tmV);
  if (!r) r = na_encode(p, tile, Vs, &tmVs);
  if (r) return r;

  const double *dxs[3] = {dx1, dx2, dx3};
  for (int d = 0; d < p.dims; d++) {
    e = cudaMemcpyAsync(grid + (long long)d * kNaMaxDir, dxs[d], p.ntot[d] * sizeof(double),
                        cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return na_cuda(e, "copy of dx");
  }
  k_na_prepare<<<1, 256, 0, st>>>(base, p, dt, inv_dt_hyp ? *inv_dt_hyp : 0.0);
  if (p.dims == 2)
    ps::fill_ghosts_2d(Vc_dev, p, st);
  else
    ps::fill_ghosts_3d(Vc_dev, p, st);

  const dim3 block(tile[0] * tile[1] * tile[2]);
  const dim3 grid3((p.nx[0] + tile[0] - 1) / tile[0], (p.nx[1] + tile[1] - 1) / tile[1],
                   (p.nx[2] + tile[2] - 1) / tile[2]);
  for (int stage = 1; stage <= 2; stage++) {
    ps::StageArgs a;
    a.Vn = Vc_dev;
    a.Vout = stage == 1 ? Vs : Vc_dev;
    a.Us = Us;
    for (int d = 0; d < 3; d++) {
      a.dtdx[d] = grid + (6LL + d) * kNaMaxDir;
      a.inv_dx[d] = grid + (3LL + d) * kNaMaxDir;
    }
    a.sc = sc;
    a.p = p;
    void *args[2] = {stage == 1 ? &tmV : &tmVs, &a};
    e = cudaLaunchKernel(stage == 1 ? k1 : k2, grid3, block, args, smem, st);
    if (e != cudaSuccess) return na_cuda(e, "stage launch");
  }
  ps::FinishArgs f;
  std::memset(&f, 0, sizeof(f));
  f.sc = sc;
  f.p = p;
  f.mode = 2;  // invDt_hyp = MAX(in, max C_dt) / DIMENSIONS, nothing else
  ps::k_finish<<<1, 256, 0, st>>>(f);
  e = cudaGetLastError();
  if (e != cudaSuccess) return na_cuda(e, "launch");

  ps::Scalars out;
  e = cudaMemcpyAsync(&out, sc, sizeof(out), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return na_cuda(e, "read-back");
  if (inv_dt_hyp) *inv_dt_hyp = out.inv_dt_hyp;
  return (int)out.flags;
}
