// ps_api.cu -- C ABI of the GB300 hydro path: device context, TMA tensor
// maps, the device-side main-loop scalars (dt selection) and CUDA-graph
// replay of whole runs.
//
// Reference (paths inside the reference project):
//   main loop / tstop clamp   Src/main.c:215-337
//   Integrate (resets)        Src/main.c:383-497
//   NextTimeStep              Src/main.c:521-697
//   invDt_hyp reduction       Src/Time_Stepping/update_stage.c:389-394
#include "ps_gb300.h"
#include "ps_hydro.cuh"
#include "ps_physics.cuh"
#include "ps_finish.cuh"

#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>

namespace ps {
const void *stage_kernel_2d(int nv, int lim, int solver, int stage);
const void *stage_kernel_3d(int nv, int lim, int solver, int stage);
size_t stage_smem_2d(int nv);
size_t stage_smem_3d(int nv);
void stage_tile_2d(int *t);
void wind_tile_2d(int *t, int *threads);
void stage_tile_3d(int *t);

// One CTA: see finish_block().
__global__ void k_finish(FinishArgs f) { finish_block(f); }

void fill_ghosts_2d(double *V, const Params &p, cudaStream_t s);
void fill_ghosts_3d(double *V, const Params &p, cudaStream_t s);

}  // namespace ps

// ------------------------------------------------------------------
// error reporting
// ------------------------------------------------------------------

static thread_local char g_errmsg[512] = "";

extern "C" void ps_set_error_msg(const char *msg)
{
  std::snprintf(g_errmsg, sizeof(g_errmsg), "%s", msg ? msg : "");
}

extern "C" const char *ps_last_error(void) { return g_errmsg; }

static int cuda_fail(cudaError_t e, const char *where)
{
  char buf[512];
  std::snprintf(buf, sizeof(buf), "%s: %s", where, cudaGetErrorString(e));
  ps_set_error_msg(buf);
  return PS_ECUDA;
}

#define CK(call)                                   \
  do {                                             \
    cudaError_t e_ = (call);                       \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

// ------------------------------------------------------------------
// context
// ------------------------------------------------------------------

#include "ps_ctx.cuh"

namespace ps {
static void launch_fill_ghosts(const ps_ctx *c, double *V, cudaStream_t s)
{
  if (c->p.dims == 2)
    fill_ghosts_2d(V, c->p, s);
  else
    fill_ghosts_3d(V, c->p, s);
}
}  // namespace ps

static int encode_map(ps_ctx *c, double *base, CUtensorMap *tm)
{
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if (!encode) {
    cudaDriverEntryPointQueryResult q;
    void *fn = nullptr;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                                     cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn) {
      ps_set_error_msg("cuTensorMapEncodeTiled entry point not available");
      return PS_ECUDA;
    }
    encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  const ps::Params &p = c->p;
  // x runs over the memory columns of a row (cell i at column i + xoff)
  cuuint64_t dims[4] = {(cuuint64_t)(p.ntot[0] + p.xoff), (cuuint64_t)p.ntot[1],
                        (cuuint64_t)p.ntot[2], (cuuint64_t)p.nvar};
  cuuint64_t strides[3] = {(cuuint64_t)p.px * 8, (cuuint64_t)p.px * p.ntot[1] * 8,
                           (cuuint64_t)p.vstride * 8};
  cuuint32_t box[4] = {(cuuint32_t)(c->tile[0] + 2 * c->tile[3]),
                       (cuuint32_t)(c->tile[1] + 2 * c->tile[4]),
                       (cuuint32_t)(c->tile[2] + 2 * c->tile[5]), (cuuint32_t)p.nvar};
  cuuint32_t estr[4] = {1, 1, 1, 1};
  CUresult r = encode(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 4, base, dims, strides, box, estr,
                      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                      CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    char buf[128];
    std::snprintf(buf, sizeof(buf), "cuTensorMapEncodeTiled failed (%d)", (int)r);
    ps_set_error_msg(buf);
    return PS_ECUDA;
  }
  return 0;
}

void ps_wind_free(ps::WindDev *w);
int ps_wind_step_launches(ps_ctx *c, int odd, int (*finish)(ps_ctx *, int));
int ps_wind_hydro_launches(ps_ctx *c);
int ps_wind_check(const ps_ctx *c, const char *who);
int ps_wind_cool_launch(ps_ctx *c);
int ps_wind_bnd_launch(ps_ctx *c, int stage);
int ps_wind_stage_launch(ps_ctx *c, int stage);

void ps_sg_free_ctx(ps_ctx *c);

// Drops the captured step graphs (they are rebuilt at the next ps_run).
void ps_ctx_invalidate_graphs(ps_ctx *c)
{
  for (int k = 0; k < 3; k++)
    if (c->gw[k]) {
      cudaGraphExecDestroy(c->gw[k]);
      c->gw[k] = nullptr;
    }
  if (c->g1) {
    cudaGraphExecDestroy(c->g1);
    c->g1 = nullptr;
  }
  if (c->gN) {
    cudaGraphExecDestroy(c->gN);
    c->gN = nullptr;
  }
}

static void free_ctx(ps_ctx *c)
{
  if (!c) return;
  ps_sg_free_ctx(c);
  if (c->wind) ps_wind_free(c->wind);
  for (int k = 0; k < 3; k++)
    if (c->gw[k]) cudaGraphExecDestroy(c->gw[k]);
  for (int d = 0; d < 3; d++) {
    std::free(c->hx[d]);
    std::free(c->hxl[d]);
    std::free(c->hxr[d]);
    std::free(c->hdx[d]);
  }
  if (c->g1) cudaGraphExecDestroy(c->g1);
  if (c->gN) cudaGraphExecDestroy(c->gN);
  cudaFree(c->V);
  cudaFree(c->Vs);
  cudaFree(c->Us);
  for (int d = 0; d < 3; d++) {
    cudaFree(c->dx[d]);
    cudaFree(c->inv_dx[d]);
    cudaFree(c->dtdx[d]);
  }
  cudaFree(c->sc);
  cudaFree(c->hist);
  cudaFree(c->Vsave);
  cudaFree(c->sc_save);
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  delete c;
}

extern "C" int ps_create(const ps_config *cfg, ps_ctx **out)
{
  if (!cfg || !out) {
    ps_set_error_msg("ps_create: null argument");
    return PS_EINVAL;
  }
  *out = nullptr;
  const bool sph = cfg->geometry == PS_SPHERICAL;
  const int sph_nvar = cfg->entropy_switch ? 7 : 6;
  if ((cfg->dims != 2 && cfg->dims != 3) || (cfg->nvar < 5 || cfg->nvar > 7) ||
      (!sph && cfg->nvar == 7) || (cfg->geometry != PS_CARTESIAN && !sph) ||
      (sph && (cfg->dims != 2 || cfg->nvar != sph_nvar)) ||
      cfg->entropy_switch < 0 || cfg->entropy_switch > 2 || cfg->cooling < 0 ||
      cfg->cooling > 2 || (cfg->cooling == 2 && !sph) ||
      cfg->limiter < 0 || cfg->limiter > 2 ||
      (cfg->solver != PS_HLLC && cfg->solver != PS_HLL) || cfg->gamma <= 1.0) {
    ps_set_error_msg("ps_create: unsupported configuration (Cartesian: dims 2/3, nvar 5/6; "
                     "spherical: dims 2, nvar 6, or 7 with the entropy switch; MC/VL/MM "
                     "limiter, HLLC/HLL)");
    return PS_EINVAL;
  }
  for (int d = 0; d < 3; d++) {
    if (d < cfg->dims && cfg->nx[d] < 4) {
      ps_set_error_msg("ps_create: at least 4 active cells per active direction");
      return PS_EINVAL;
    }
    if (d >= cfg->dims && cfg->nx[d] != 1) {
      ps_set_error_msg("ps_create: inactive directions must have nx = 1");
      return PS_EINVAL;
    }
  }
  if ((cfg->char_limiting || cfg->shock_flattening || cfg->entropy_switch) && !sph) {
    ps_set_error_msg("ps_create: characteristic limiting, shock flattening and the entropy "
                     "switch are built for the spherical wind path");
    return PS_EINVAL;
  }
  for (int s = 0; s < 2 * cfg->dims; s++) {
    int b = cfg->bc[s];
    // user sides of the spherical wind: X1_BEG, X1_END and X2_BEG, with the
    // production problem's hooks (csrc/ps_userdef.cuh)
    const bool userdef_ok = sph && s <= 2 && b == PS_BC_USERDEF;
    if (b != PS_BC_OUTFLOW && b != PS_BC_PERIODIC && b != PS_BC_REFLECTIVE &&
        b != PS_BC_AXISYM && b != PS_BC_EQTSYM && !userdef_ok) {
      ps_set_error_msg("ps_create: boundary type not supported on this path");
      return PS_EINVAL;
    }
    if ((b == PS_BC_PERIODIC) != (cfg->bc[s ^ 1] == PS_BC_PERIODIC)) {
      ps_set_error_msg("ps_create: periodic boundaries must be paired");
      return PS_EINVAL;
    }
  }

  ps_ctx *c = new ps_ctx();
  std::memset(&c->p, 0, sizeof(c->p));
  c->cfg = *cfg;
  ps::Params &p = c->p;
  p.dims = cfg->dims;
  p.nvar = cfg->nvar;
  p.limiter = cfg->limiter;
  p.solver = cfg->solver;
  p.cooling = cfg->cooling;
  p.char_lim = cfg->char_limiting ? 1 : 0;
  p.shock = cfg->shock_flattening ? 1 : 0;
  p.entropy = cfg->entropy_switch;
  for (int d = 0; d < 3; d++) {
    p.nx[d] = cfg->nx[d];
    // GetNghost (Src/get_nghost.c:15-60): 2 ghost zones for PLM, 3 with
    // SHOCK_FLATTENING MULTID
    p.beg[d] = d < cfg->dims ? (cfg->shock_flattening ? 3 : 2) : 0;
    p.ntot[d] = cfg->nx[d] + 2 * p.beg[d];
  }
  for (int s = 0; s < 6; s++) p.bc[s] = cfg->bc[s];
  p.xoff = (p.beg[0] & 1) ? 1 : 0;
  p.px = (p.ntot[0] + p.xoff + 3) & ~3;
  p.vstride = (long long)p.px * p.ntot[1] * p.ntot[2];
  p.gamma = cfg->gamma;
  p.gmm1 = cfg->gamma - 1.0;
  p.igmm1 = 1.0 / p.gmm1;
  p.cfl = cfg->cfl;
  p.cfl_max_var = cfg->cfl_max_var;
  p.tstop = cfg->tstop;
  p.first_dt = cfg->first_dt;

  int threads = 0;  // one per tile cell unless the tile says otherwise
  if (cfg->dims == 2) {
    if (sph)
      ps::wind_tile_2d(c->tile, &threads);
    else
      ps::stage_tile_2d(c->tile);
    c->smem = ps::stage_smem_2d(p.nvar);
    c->k1 = sph ? nullptr : ps::stage_kernel_2d(p.nvar, p.limiter, p.solver, 1);
    c->k2 = sph ? nullptr : ps::stage_kernel_2d(p.nvar, p.limiter, p.solver, 2);
  } else {
    ps::stage_tile_3d(c->tile);
    c->smem = ps::stage_smem_3d(p.nvar);
    c->k1 = ps::stage_kernel_3d(p.nvar, p.limiter, p.solver, 1);
    c->k2 = ps::stage_kernel_3d(p.nvar, p.limiter, p.solver, 2);
  }
  c->block = dim3(threads ? threads : c->tile[0] * c->tile[1] * c->tile[2]);
  c->grid = dim3((p.nx[0] + c->tile[0] - 1) / c->tile[0], (p.nx[1] + c->tile[1] - 1) / c->tile[1],
                 (p.nx[2] + c->tile[2] - 1) / c->tile[2]);

  cudaError_t e;
  const size_t nbytes = (size_t)p.vstride * p.nvar * sizeof(double);
#define TRY(call)                                  \
  do {                                             \
    e = (call);                                    \
    if (e != cudaSuccess) {                        \
      int r_ = cuda_fail(e, #call);                \
      free_ctx(c);                                 \
      return r_;                                   \
    }                                              \
  } while (0)
  TRY(cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking));
  c->stream = c->own_stream;
  TRY(cudaMalloc(&c->V, nbytes));
  TRY(cudaMalloc(&c->Vs, nbytes));
  TRY(cudaMalloc(&c->Us, nbytes));
  TRY(cudaMemset(c->V, 0, nbytes));
  TRY(cudaMemset(c->Vs, 0, nbytes));
  TRY(cudaMemset(c->Us, 0, nbytes));
  for (int d = 0; d < 3; d++) {
    TRY(cudaMalloc(&c->dx[d], p.ntot[d] * sizeof(double)));
    TRY(cudaMalloc(&c->inv_dx[d], p.ntot[d] * sizeof(double)));
    TRY(cudaMalloc(&c->dtdx[d], p.ntot[d] * sizeof(double)));
    TRY(cudaMemset(c->dx[d], 0, p.ntot[d] * sizeof(double)));
    TRY(cudaMemset(c->inv_dx[d], 0, p.ntot[d] * sizeof(double)));
    TRY(cudaMemset(c->dtdx[d], 0, p.ntot[d] * sizeof(double)));
  }
  TRY(cudaMalloc(&c->sc, sizeof(ps::Scalars)));
  TRY(cudaMalloc(&c->hist, ps::kHist * sizeof(double)));
  TRY(cudaMemset(c->hist, 0, ps::kHist * sizeof(double)));
  if (c->k1) {
    TRY(cudaFuncSetAttribute(c->k1, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c->smem));
    TRY(cudaFuncSetAttribute(c->k2, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c->smem));
  }
#undef TRY
  ps::Scalars s0;
  std::memset(&s0, 0, sizeof(s0));
  s0.dt = cfg->first_dt;
  s0.dt_cool = 1.e38;
  if (cudaMemcpy(c->sc, &s0, sizeof(s0), cudaMemcpyHostToDevice) != cudaSuccess) {
    free_ctx(c);
    return cuda_fail(cudaGetLastError(), "ps_create: scalars");
  }
  int r = encode_map(c, c->V, &c->tmV);
  if (!r) r = encode_map(c, c->Vs, &c->tmVs);
  if (r) {
    free_ctx(c);
    return r;
  }
  *out = c;
  return 0;
}

extern "C" int ps_destroy(ps_ctx *c)
{
  if (!c) return PS_EINVAL;
  cudaStreamSynchronize(c->stream);
  free_ctx(c);
  return 0;
}

extern "C" int ps_set_grid(ps_ctx *c, int dir, const double *x, const double *xl,
                           const double *xr, const double *dx)
{
  if (!c || dir < 0 || dir >= c->p.dims || !dx) {
    ps_set_error_msg("ps_set_grid: bad arguments");
    return PS_EINVAL;
  }
  const int n = c->p.ntot[dir];
  if (c->cfg.geometry == PS_SPHERICAL && (!x || !xl || !xr)) {
    ps_set_error_msg("ps_set_grid: spherical geometry needs x, xl, xr and dx");
    return PS_EINVAL;
  }
  double *inv = (double *)std::malloc(n * sizeof(double));
  if (!inv) return PS_ENOMEM;
  const double *src[4] = {x, xl, xr, dx};
  double **dst[4] = {&c->hx[dir], &c->hxl[dir], &c->hxr[dir], &c->hdx[dir]};
  for (int k = 0; k < 4; k++) {
    std::free(*dst[k]);
    *dst[k] = nullptr;
    if (!src[k]) continue;
    *dst[k] = (double *)std::malloc(n * sizeof(double));
    if (!*dst[k]) {
      std::free(inv);
      return PS_ENOMEM;
    }
    std::memcpy(*dst[k], src[k], n * sizeof(double));
  }
  for (int i = 0; i < n; i++) inv[i] = 1.0 / (dx[i]);  // Src/set_geometry.c:243-245
  cudaError_t e = cudaMemcpy(c->dx[dir], dx, n * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(c->inv_dx[dir], inv, n * sizeof(double), cudaMemcpyHostToDevice);
  std::free(inv);
  if (e != cudaSuccess) return cuda_fail(e, "ps_set_grid");
  c->grid_mask |= 1 << dir;
  return 0;
}

static int launch_finish(ps_ctx *c, int mode)
{
  ps::FinishArgs f;
  f.sc = c->sc;
  f.hist_dt = c->hist;
  for (int d = 0; d < 3; d++) {
    f.dtdx[d] = c->dtdx[d];
    f.dx[d] = c->dx[d];
  }
  f.p = c->p;
  f.mode = mode;
  ps::k_finish<<<1, 256, 0, c->stream>>>(f);
  c->launches++;
  return 0;
}

static ps::StageArgs stage_args(ps_ctx *c, int stage)
{
  ps::StageArgs a;
  a.Vn = c->V;
  a.Vout = stage == 1 ? c->Vs : c->V;
  a.Us = c->Us;
  for (int d = 0; d < 3; d++) {
    a.dtdx[d] = c->dtdx[d];
    a.inv_dx[d] = c->inv_dx[d];
  }
  a.sc = c->sc;
  a.p = c->p;
  return a;
}

static cudaError_t launch_stage(ps_ctx *c, int stage)
{
  ps::StageArgs a = stage_args(c, stage);
  CUtensorMap *tm = stage == 1 ? &c->tmV : &c->tmVs;
  void *args[2] = {tm, &a};
  cudaError_t e = cudaLaunchKernel(stage == 1 ? c->k1 : c->k2, c->grid, c->block, args, c->smem,
                                   c->stream);
  c->launches++;
  return e;
}

static int check_ready(ps_ctx *c, const char *who)
{
  if (!c) {
    ps_set_error_msg("null context");
    return PS_EINVAL;
  }
  if (c->grid_mask != (1 << c->p.dims) - 1) {
    char buf[128];
    std::snprintf(buf, sizeof(buf), "%s: ps_set_grid not called for every direction", who);
    ps_set_error_msg(buf);
    return PS_ESTATE;
  }
  return 0;
}

extern "C" int ps_set_state(ps_ctx *c, const double *Vc)
{
  int r = check_ready(c, "ps_set_state");
  if (r) return r;
  if (!Vc) return PS_EINVAL;
  const ps::Params &p = c->p;
  const size_t rows = (size_t)p.ntot[1] * p.ntot[2] * p.nvar;
  if (p.px == p.ntot[0] && p.xoff == 0)   // rows back to back: one linear copy (faster)
    CK(cudaMemcpyAsync(c->V, Vc, rows * p.ntot[0] * 8, cudaMemcpyHostToDevice, c->stream));
  else
    CK(cudaMemcpy2DAsync(c->V + p.xoff, (size_t)p.px * 8, Vc, (size_t)p.ntot[0] * 8,
                         (size_t)p.ntot[0] * 8, rows, cudaMemcpyHostToDevice, c->stream));
  // Cartesian contexts: the stage kernels read ghost zones written by the
  // previous stage, so they are filled here; the wind's ghost zones are
  // filled by its boundary kernels before every stage
  if (c->cfg.geometry != PS_SPHERICAL) {
    ps::launch_fill_ghosts(c, c->V, c->stream);
    c->launches++;
  }
  CK(cudaGetLastError());
  launch_finish(c, ps::MODE_BEGIN);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(c->stream));
  return 0;
}

extern "C" int ps_get_state(ps_ctx *c, double *Vc)
{
  if (!c || !Vc) return PS_EINVAL;
  const ps::Params &p = c->p;
  const size_t rows = (size_t)p.ntot[1] * p.ntot[2] * p.nvar;
  if (p.px == p.ntot[0] && p.xoff == 0)
    CK(cudaMemcpyAsync(Vc, c->V, rows * p.ntot[0] * 8, cudaMemcpyDeviceToHost, c->stream));
  else
    CK(cudaMemcpy2DAsync(Vc, (size_t)p.ntot[0] * 8, c->V + p.xoff, (size_t)p.px * 8,
                         (size_t)p.ntot[0] * 8, rows, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return 0;
}

extern "C" int ps_set_time(ps_ctx *c, double t, double dt, long step)
{
  if (!c) return PS_EINVAL;
  ps::Scalars s;
  CK(cudaStreamSynchronize(c->stream));
  CK(cudaMemcpy(&s, c->sc, sizeof(s), cudaMemcpyDeviceToHost));
  s.t = t;
  s.dt = dt;
  s.step = step;
  c->host_step = step;
  s.last = 0;
  s.done = 0;
  s.inv_dt_hyp = 0.0;
  s.dt_cool = 1.e38;
  CK(cudaMemcpy(c->sc, &s, sizeof(s), cudaMemcpyHostToDevice));
  if (check_ready(c, "ps_set_time") == 0) {
    launch_finish(c, ps::MODE_BEGIN);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(c->stream));
  }
  return 0;
}

extern "C" int ps_get_time(ps_ctx *c, double *t, double *dt, long *step, double *inv)
{
  if (!c) return PS_EINVAL;
  ps::Scalars s;
  CK(cudaStreamSynchronize(c->stream));
  CK(cudaMemcpy(&s, c->sc, sizeof(s), cudaMemcpyDeviceToHost));
  if (t) *t = s.t;
  if (dt) *dt = s.dt;
  if (step) *step = (long)s.step;
  if (inv) *inv = s.inv_dt_hyp;
  return 0;
}

extern "C" int ps_sync(ps_ctx *c)
{
  if (!c) return PS_EINVAL;
  unsigned flags = 0;
  CK(cudaStreamSynchronize(c->stream));
  CK(cudaMemcpy(&flags, &c->sc->flags, sizeof(unsigned), cudaMemcpyDeviceToHost));
  return (int)flags;
}

extern "C" int ps_advance_step(ps_ctx *c, double dt, double *inv_dt_hyp)
{
  int r = check_ready(c, "ps_advance_step");
  if (r) return r;
  if (c->cfg.geometry == PS_SPHERICAL && !c->wind) {
    ps_set_error_msg("ps_advance_step: a spherical context needs ps_set_wind first");
    return PS_ESTATE;
  }
  if ((r = ps_wind_check(c, "ps_advance_step"))) return r;
  ps::Scalars s;
  CK(cudaStreamSynchronize(c->stream));
  CK(cudaMemcpy(&s, c->sc, sizeof(s), cudaMemcpyDeviceToHost));
  s.dt = dt;
  s.inv_dt_hyp = inv_dt_hyp ? *inv_dt_hyp : 0.0;
  s.done = 0;
  s.last = 0;
  CK(cudaMemcpy(c->sc, &s, sizeof(s), cudaMemcpyHostToDevice));
  launch_finish(c, ps::MODE_PREP);
  if (c->wind) {
    r = ps_wind_hydro_launches(c);
    if (r) return r;
  } else {
    CK(launch_stage(c, 1));
    CK(launch_stage(c, 2));
  }
  launch_finish(c, ps::MODE_INV);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(c->stream));
  CK(cudaMemcpy(&s, c->sc, sizeof(s), cudaMemcpyDeviceToHost));
  if (inv_dt_hyp) *inv_dt_hyp = s.inv_dt_hyp;
  return (int)s.flags;
}

static int build_graph(ps_ctx *c, int nsteps, cudaGraphExec_t *out)
{
  cudaGraph_t g;
  long before = c->launches;
  CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  for (int s = 0; s < nsteps; s++) {
    launch_stage(c, 1);
    launch_stage(c, 2);
    launch_finish(c, ps::MODE_STEP);
  }
  cudaError_t e = cudaStreamEndCapture(c->stream, &g);
  c->launches = before;  // captured, not yet launched
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
  return 0;
}

static int finish_step(ps_ctx *c, int) { return launch_finish(c, ps::MODE_STEP); }

int ps_cart_cool_launch(ps_ctx *c);

// One step with the operator-split source: the source before (odd steps)
// or after (even steps) AdvanceStep (Src/main.c:479-485), then the dt
// kernel.  Wind or Cartesian cooling context.
static int split_step_launches(ps_ctx *c, int odd)
{
  if (c->wind) return ps_wind_step_launches(c, odd, finish_step);
  int r = 0;
  if (odd) r = ps_cart_cool_launch(c);
  if (!r) CK(launch_stage(c, 1));
  if (!r) CK(launch_stage(c, 2));
  if (!r && !odd) r = ps_cart_cool_launch(c);
  if (!r) r = launch_finish(c, ps::MODE_STEP);
  return r;
}

// CUDA graphs of a step with the split source: [0] even step, [1] odd
// step, [2] even+odd
static int build_wind_graph(ps_ctx *c, int kind, cudaGraphExec_t *out)
{
  cudaGraph_t g;
  long before = c->launches;
  CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  int r = 0;
  if (kind == 0 || kind == 2) r = split_step_launches(c, 0);
  if (!r && (kind == 1 || kind == 2)) r = split_step_launches(c, 1);
  cudaError_t e = cudaStreamEndCapture(c->stream, &g);
  c->launches = before;
  if (r) return r;
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture (wind)");
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate (wind)");
  return 0;
}

static int run_wind(ps_ctx *c, int nsteps)
{
  const int ncool = c->p.cooling ? (c->sg ? 2 : 1) + (c->wind ? 0 : 1) : 0;
  const long per_step = (c->wind ? 7 + (ps::needs_shock_flags(c->p) ? 1 : 0) : 3) + ncool;
  for (int k = 0; k < 3; k++)
    if (!c->gw[k]) {
      int r = build_wind_graph(c, k, &c->gw[k]);
      if (r) return r;
    }
  int left = nsteps;
  while (left > 0) {
    const int odd = (int)(c->host_step & 1);
    if (!odd && left >= 2) {
      CK(cudaGraphLaunch(c->gw[2], c->stream));
      c->launches += 2 * per_step;
      c->host_step += 2;
      left -= 2;
    } else {
      CK(cudaGraphLaunch(c->gw[odd], c->stream));
      c->launches += per_step;
      c->host_step += 1;
      left -= 1;
    }
  }
  CK(cudaGetLastError());
  return 0;
}

extern "C" int ps_run(ps_ctx *c, int nsteps)
{
  int r = check_ready(c, "ps_run");
  if (r) return r;
  if (nsteps < 0) return PS_EINVAL;
  if (c->cfg.geometry == PS_SPHERICAL) {
    if (!c->wind) {
      ps_set_error_msg("ps_run: a spherical context needs ps_set_wind first");
      return PS_ESTATE;
    }
    if ((r = ps_wind_check(c, "ps_run"))) return r;
    return run_wind(c, nsteps);
  }
  if (c->cool_on && c->p.cooling) return run_wind(c, nsteps);
  const int G = 16;
  if (!c->g1) {
    r = build_graph(c, 1, &c->g1);
    if (r) return r;
  }
  if (nsteps >= G && !c->gN) {
    r = build_graph(c, G, &c->gN);
    if (r) return r;
    c->nG = G;
  }
  int left = nsteps;
  while (left >= G) {
    CK(cudaGraphLaunch(c->gN, c->stream));
    c->launches += 3L * G;
    left -= G;
  }
  while (left > 0) {
    CK(cudaGraphLaunch(c->g1, c->stream));
    c->launches += 3;
    left--;
  }
  CK(cudaGetLastError());
  return 0;
}

extern "C" double *ps_device_state(ps_ctx *c, int *pitch)
{
  if (!c) return nullptr;
  if (pitch) *pitch = c->p.px;
  return c->V + c->p.xoff;
}

extern "C" long ps_launch_count(const ps_ctx *c) { return c ? c->launches : -1; }

extern "C" int ps_get_dt_history(ps_ctx *c, double *out, int max)
{
  if (!c || !out || max < 0) return PS_EINVAL;
  int n = max < ps::kHist ? max : ps::kHist;
  CK(cudaStreamSynchronize(c->stream));
  CK(cudaMemcpy(out, c->hist, n * sizeof(double), cudaMemcpyDeviceToHost));
  return n;
}

extern "C" int ps_set_stream(ps_ctx *c, void *stream)
{
  if (!c) return PS_EINVAL;
  CK(cudaStreamSynchronize(c->stream));
  c->stream = stream ? static_cast<cudaStream_t>(stream) : c->own_stream;
  return 0;
}

// Device-side checkpoint of the state and the main-loop scalars (the
// role of the FAILSAFE backup in Src/failsafe.c:5-160, kept on the GPU).
extern "C" int ps_save_state(ps_ctx *c)
{
  if (!c) return PS_EINVAL;
  const size_t nbytes = (size_t)c->p.vstride * c->p.nvar * sizeof(double);
  if (!c->Vsave) {
    CK(cudaMalloc(&c->Vsave, nbytes));
    CK(cudaMalloc(&c->sc_save, sizeof(ps::Scalars)));
  }
  CK(cudaMemcpyAsync(c->Vsave, c->V, nbytes, cudaMemcpyDeviceToDevice, c->stream));
  CK(cudaMemcpyAsync(c->sc_save, c->sc, sizeof(ps::Scalars), cudaMemcpyDeviceToDevice,
                     c->stream));
  c->host_step_save = c->host_step;
  return 0;
}

extern "C" int ps_restore_state(ps_ctx *c)
{
  if (!c || !c->Vsave) {
    ps_set_error_msg("ps_restore_state: no saved state");
    return PS_ESTATE;
  }
  const size_t nbytes = (size_t)c->p.vstride * c->p.nvar * sizeof(double);
  CK(cudaMemcpyAsync(c->V, c->Vsave, nbytes, cudaMemcpyDeviceToDevice, c->stream));
  CK(cudaMemcpyAsync(c->sc, c->sc_save, sizeof(ps::Scalars), cudaMemcpyDeviceToDevice,
                     c->stream));
  c->host_step = c->host_step_save;
  return 0;
}

// Runs one step with a CUDA event around each of its three kernels and
// returns their durations in ms (stage 1, stage 2, finish).  Advances the
// state by one step like ps_run(ctx, 1).
extern "C" int ps_time_step_kernels(ps_ctx *c, double *ms)
{
  int r = check_ready(c, "ps_time_step_kernels");
  if (r) return r;
  if (!ms) return PS_EINVAL;
  if (c->cfg.geometry == PS_SPHERICAL && !c->wind) {
    ps_set_error_msg("ps_time_step_kernels: a spherical context needs ps_set_wind first");
    return PS_ESTATE;
  }
  cudaEvent_t ev[8];
  for (int i = 0; i < 8; i++) CK(cudaEventCreate(&ev[i]));
  if (c->wind) {
    // ms[0], ms[1]: the two stage kernels; ms[2]: the rest of the step
    // (boundary kernels, split source, dt kernel)
    const int odd = (int)(c->host_step & 1);
    CK(cudaEventRecord(ev[0], c->stream));
    if (odd) r = ps_wind_cool_launch(c);
    if (!r) r = ps_wind_bnd_launch(c, 1);
    CK(cudaEventRecord(ev[1], c->stream));
    if (!r) r = ps_wind_stage_launch(c, 1);
    CK(cudaEventRecord(ev[2], c->stream));
    if (!r) r = ps_wind_bnd_launch(c, 2);
    CK(cudaEventRecord(ev[3], c->stream));
    if (!r) r = ps_wind_stage_launch(c, 2);
    CK(cudaEventRecord(ev[4], c->stream));
    if (!r && !odd) r = ps_wind_cool_launch(c);
    launch_finish(c, ps::MODE_STEP);
    CK(cudaEventRecord(ev[5], c->stream));
    CK(cudaEventSynchronize(ev[5]));
    c->host_step++;
    float t[5];
    for (int i = 0; i < 5; i++) CK(cudaEventElapsedTime(&t[i], ev[i], ev[i + 1]));
    ms[0] = t[1];
    ms[1] = t[3];
    ms[2] = t[0] + t[2] + t[4];
  } else {
    // Cartesian: ms[0], ms[1] the stage kernels, ms[2] the dt kernel and
    // (with the split source) the cooling step
    const bool cool = c->cool_on && c->p.cooling;
    const int odd = (int)(c->host_step & 1);
    CK(cudaEventRecord(ev[0], c->stream));
    if (cool && odd) r = ps_cart_cool_launch(c);
    CK(cudaEventRecord(ev[1], c->stream));
    CK(launch_stage(c, 1));
    CK(cudaEventRecord(ev[2], c->stream));
    CK(launch_stage(c, 2));
    CK(cudaEventRecord(ev[3], c->stream));
    if (!r && cool && !odd) r = ps_cart_cool_launch(c);
    launch_finish(c, ps::MODE_STEP);
    CK(cudaEventRecord(ev[4], c->stream));
    CK(cudaEventSynchronize(ev[4]));
    if (cool) c->host_step++;
    float t[4];
    for (int i = 0; i < 4; i++) CK(cudaEventElapsedTime(&t[i], ev[i], ev[i + 1]));
    ms[0] = t[1];
    ms[1] = t[2];
    ms[2] = t[0] + t[3];
  }
  for (int i = 0; i < 8; i++) cudaEventDestroy(ev[i]);
  return r;
}

// SplitSource (Src/split_source.c:28-79): the BLONDIN pass with dt at time t.
// One split-source pass with the given dt at time t.  *dt_cool (may be
// NULL) gets the smallest cooling time step the cells of this pass asked
// for (1e38 when none did); the device's running minimum, which the
// device main loop's NextTimeStep reads, keeps including it.
static int split_source(ps_ctx *c, double dt, double t, double *dt_cool)
{
  int r = check_ready(c, "ps_split_source");
  if (r) return r;
  if (dt_cool) *dt_cool = 1.e38;
  if (!c->p.cooling || !(c->wind || c->cool_on)) return 0;
  ps::Scalars s;
  CK(cudaStreamSynchronize(c->stream));
  CK(cudaMemcpy(&s, c->sc, sizeof(s), cudaMemcpyDeviceToHost));
  const double running = s.dt_cool;
  s.dt = dt;
  s.t = t;
  s.done = 0;
  s.dt_cool = 1.e38;
  CK(cudaMemcpy(c->sc, &s, sizeof(s), cudaMemcpyHostToDevice));
  r = c->wind ? ps_wind_cool_launch(c) : ps_cart_cool_launch(c);
  if (r) return r;
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(c->stream));
  CK(cudaMemcpy(&s, c->sc, sizeof(s), cudaMemcpyDeviceToHost));
  if (dt_cool) *dt_cool = s.dt_cool;
  const double keep = running <= s.dt_cool ? running : s.dt_cool;
  CK(cudaMemcpy(&c->sc->dt_cool, &keep, sizeof(double), cudaMemcpyHostToDevice));
  return (int)s.flags;
}

extern "C" int ps_split_source(ps_ctx *c, double dt, double t)
{
  return split_source(c, dt, t, nullptr);
}

extern "C" int ps_split_source_dt(ps_ctx *c, double dt, double t, double *dt_cool)
{
  return split_source(c, dt, t, dt_cool);
}
