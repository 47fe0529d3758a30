// ps_batch.cu -- many independent line-driven wind models (uneven grid
// sizes, own parameters, own dt) advanced together: every phase of a step
// (split source, boundaries, the two stages, the dt kernel) is ONE launch
// covering all models, and a whole step (or step pair) is one CUDA graph.
// The tile shape of the stage kernels is chosen per grid size by a
// measuring autotuner (ps_batch_autotune).
//
// Each model keeps its own context (state, scratch, geometry, flux-bin
// lists, scalars); the batch holds a device table of per-model arguments
// and TMA descriptors and the work lists that map CTAs to (model, tile) or
// (model, cell block).  Results are identical to advancing each model on
// its own (the per-cell arithmetic does not depend on the tile shape).
#include "ps_batch_dev.cuh"
#include "ps_finish.cuh"
#include "ps_surrogate_cool.cuh"

#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <vector>

extern "C" void ps_set_error_msg(const char *msg);
int ps_wind_check(const ps_ctx *c, const char *who);

namespace ps {

template <int NV>
__global__ void k_batch_bnd_x1(const BatchModel *__restrict__ models,
                               const BlockItem *__restrict__ blocks, int stage)
{
  // a 256-cell block of the list per 64-thread CTA, 4 cells per thread
  const BlockItem bi = blocks[blockIdx.x];
  const WindStageArgs &A = models[bi.m].st[0];
  if (A.s.sc->done) return;
  bnd_x1_cells<NV, 4>(stage == 1 ? const_cast<double *>(A.s.Vn) : A.s.Vout, A.s.Us, A.s.p, A.w,
                      stage, bi.b * 256 + threadIdx.x, 64, A.s.p.nx[0] * A.s.p.nx[1]);
}

template <int NV>
__global__ void k_batch_bnd_x2(const BatchModel *__restrict__ models,
                               const BlockItem *__restrict__ blocks, int stage)
{
  const BlockItem bi = blocks[blockIdx.x];
  const WindStageArgs &A = models[bi.m].st[0];
  if (A.s.sc->done) return;
  const int q = bi.b * blockDim.x + threadIdx.x;
  if (q < A.s.p.ntot[0] * 2 * A.s.p.beg[1])
    bnd_x2_item<NV>(stage == 1 ? const_cast<double *>(A.s.Vn) : A.s.Vout, A.s.p, q);
}

// FlagShock of the models with SHOCK_FLATTENING MULTID, before stage 1
__global__ void k_batch_shock(const BatchModel *__restrict__ models,
                              const BlockItem *__restrict__ blocks)
{
  const BlockItem bi = blocks[blockIdx.x];
  const WindStageArgs &A = models[bi.m].st[0];
  if (A.s.sc->done) return;
  const Params &p = A.s.p;
  const int q = bi.b * blockDim.x + threadIdx.x;
  if (q < p.ntot[0] * p.ntot[1]) {
    const int i = q % p.ntot[0], j = q / p.ntot[0];
    const_cast<unsigned char *>(A.shock)[vcell(p, j, i)] = shock_zone(A.s.Vn, p, A.g, i, j);
  }
}

__global__ void k_batch_ode(const BatchModel *__restrict__ models,
                            const BlockItem *__restrict__ blocks, const double *const *xi,
                            const double *const *tr, const double *const *pre)
{
  const BlockItem bi = blocks[blockIdx.x];
  const WindStageArgs &A = models[bi.m].st[0];
  Scalars *sc = A.s.sc;
  if (sc->done) return;
  const int q = bi.b * blockDim.x + threadIdx.x;
  if (q < A.s.p.nx[0] * A.s.p.nx[1])
    ode_wind_cell(const_cast<double *>(A.s.Vn), xi[bi.m], tr[bi.m], A.s.p, A.w, A.g.x1, sc,
                  sc->dt, sc->t, q, pre[bi.m]);
}

__global__ void k_batch_blondin(const BatchModel *__restrict__ models,
                                const BlockItem *__restrict__ blocks, const double *const *xi,
                                const double *const *tr, const double *const *pre)
{
  const BlockItem bi = blocks[blockIdx.x];
  const WindStageArgs &A = models[bi.m].st[0];
  Scalars *sc = A.s.sc;
  if (sc->done) return;
  const int q = bi.b * blockDim.x + threadIdx.x;
  if (q < A.s.p.nx[0] * A.s.p.nx[1])
    blondin_cell(const_cast<double *>(A.s.Vn), xi[bi.m], tr[bi.m], A.s.p, A.w, A.g.x1, sc, sc->dt,
                 sc->t, q, pre[bi.m]);
}

// The split-source step with the surrogate: one CTA per 128-cell block of
// one model; the cells the judge rejects are queued as (model, cell).
__device__ __forceinline__ SgCoolArgs batch_cool_args(const BatchModel &M, const double *xi,
                                                      const double *tr, const double *pre)
{
  const WindStageArgs &A = M.st[0];
  SgCoolArgs c;
  c.V = const_cast<double *>(A.s.Vn);
  c.xi = xi;
  c.tr = tr;
  c.pre = pre;
  c.x1 = A.g.x1;
  c.p = A.s.p;
  c.w = A.w;
  c.sc = A.s.sc;
  return c;
}

__global__ void __launch_bounds__(128)
    k_batch_sg_cool(const BatchModel *__restrict__ models, const BlockItem *__restrict__ blocks,
                    int nitems, const double *const *xi, const double *const *tr,
                    const double *const *pre, SgNet net, SgBox bx, int use_net, int2 *queue,
                    int *qcount, unsigned long long *stats)
{
  extern __shared__ __align__(1024) unsigned char smem[];
  auto args_of = [&](int m) { return batch_cool_args(models[m], xi[m], tr[m], pre[m]); };
  sg_cool_items(net, bx, args_of, blocks, nitems, use_net, smem, queue, qcount, stats);
}

__global__ void k_batch_sg_fallback(const BatchModel *__restrict__ models, const double *const *xi,
                                    const double *const *tr, const double *const *pre,
                                    const int2 *__restrict__ queue, const int *__restrict__ qcount)
{
  const int cnt = *qcount;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < cnt; k += gridDim.x * blockDim.x) {
    const int2 e = queue[k];
    const SgCoolArgs A = batch_cool_args(models[e.x], xi[e.x], tr[e.x], pre[e.x]);
    blondin_cell(A.V, A.xi, A.tr, A.p, A.w, A.x1, A.sc, A.sc->dt, A.sc->t, e.y, A.pre);
  }
}

__global__ void k_batch_finish(const BatchModel *__restrict__ models, const int *__restrict__ list)
{
  finish_block(models[list[blockIdx.x]].fin);
}

// One block: the OR of every model's flags into *out.
__global__ void k_batch_gather_flags(const BatchModel *__restrict__ models, int n, unsigned *out)
{
  __shared__ unsigned all;
  if (threadIdx.x == 0) all = 0;
  __syncthreads();
  unsigned f = 0;
  for (int m = threadIdx.x; m < n; m += blockDim.x) f |= models[m].st[0].s.sc->flags;
  if (f) atomicOr(&all, f);
  __syncthreads();
  if (threadIdx.x == 0) *out = all;
}

// stage kernels for the 6-variable state with primitive PLM; the others
// are instantiated in ps_batch_c.cu (characteristic limiting), ps_batch7.cu
// and ps_batch_c7.cu (the 7-variable state of ENTROPY_SWITCH contexts)
const void *batch_kernel_c6(int shape, int lim, int solver, int stage);
// the 6-variable primitive-PLM set, one translation unit per tile shape
// (ps_batch6_s<shape>.cu), so that they build in parallel
const void *batch_kernel6_s0(int lim, int solver, int stage);
const void *batch_kernel6_s1(int lim, int solver, int stage);
const void *batch_kernel6_s2(int lim, int solver, int stage);
const void *batch_kernel6_s3(int lim, int solver, int stage);
const void *batch_kernel6_s4(int lim, int solver, int stage);
const void *batch_kernel6_s5(int lim, int solver, int stage);
const void *batch_kernel6_s6(int lim, int solver, int stage);
const void *batch_kernel7(int shape, int lim, int solver, int stage);
const void *batch_kernel_c7(int shape, int lim, int solver, int stage);
size_t batch_smem7(int shape);

static const void *batch_kernel(int nv, bool ch, int shape, int lim, int solver, int stage)
{
  if (nv == 7)
    return ch ? batch_kernel_c7(shape, lim, solver, stage)
              : batch_kernel7(shape, lim, solver, stage);
  if (ch) return batch_kernel_c6(shape, lim, solver, stage);
  switch (shape) {
    case 1: return batch_kernel6_s1(lim, solver, stage);
    case 2: return batch_kernel6_s2(lim, solver, stage);
    case 3: return batch_kernel6_s3(lim, solver, stage);
    case 4: return batch_kernel6_s4(lim, solver, stage);
    case 5: return batch_kernel6_s5(lim, solver, stage);
    case 6: return batch_kernel6_s6(lim, solver, stage);
    default: return batch_kernel6_s0(lim, solver, stage);
  }
}

static size_t batch_smem(int nv, int shape)
{
  return nv == 7 ? batch_smem7(shape) : batch_smem_nv<6>(shape);
}

}  // namespace ps

// ------------------------------------------------------------------
// host side
// ------------------------------------------------------------------

// The models are split into groups (balanced by cells) whose steps run as
// independent branches of the step graph: one group's latency-bound
// kernels (boundaries, the learned step's fallback, the dt kernel) overlap
// the other groups' stage kernels.  Each group has its own work lists.
struct BatchGroup {
  std::vector<int> models;
  ps::TileItem *d_items[ps::kNumShapes] = {};  // tiles per tile shape
  int nitems[ps::kNumShapes] = {};
  ps::BlockItem *d_cells = nullptr, *d_x2 = nullptr;
  int ncells_blocks = 0, nx2_blocks = 0;
  ps::BlockItem *d_shock = nullptr;  // total-box blocks of the MULTID models
  int nshock_blocks = 0;
  ps::BlockItem *d_cells128 = nullptr;  // 128-cell blocks (surrogate kernel)
  int ncells128 = 0;
  int *d_list = nullptr;             // the group's model indices (dt kernel)
  long cells = 0, queue_off = 0;     // its cells and its slice of the queue
  cudaStream_t st = nullptr;         // branch stream while a graph is captured
  cudaStream_t side[ps::kNumShapes] = {};  // tile-shape branches
  cudaEvent_t fork = nullptr, join[ps::kNumShapes] = {}, done = nullptr;
};

struct ps_batch {
  int n = 0;
  std::vector<ps_ctx *> ctx;
  ps::BatchModel *d_models = nullptr;
  std::vector<ps::BatchModel> h_models;
  std::vector<int> shape;              // chosen tile shape per model
  std::vector<BatchGroup> grp;
  int ngroups = 1;
  const double **d_xi = nullptr, **d_tr = nullptr, **d_pre = nullptr;
  long total_cells = 0;
  ps_surrogate *sg = nullptr;
  int sg_use_net = 1;
  int num_sms = 148;
  int2 *sg_queue = nullptr;
  int *sg_qcount = nullptr;            // one counter per group
  int lim = 0, solver = 0, cooling = 0, nvar = 6;
  bool char_lim = false;  // CHAR_LIMITING YES (its own stage kernels)
  cudaStream_t stream = nullptr;      // stream the work is issued on
  cudaStream_t own_stream = nullptr;  // stream created by the batch
  cudaEvent_t fork = nullptr;
  cudaGraphExec_t g[3] = {nullptr, nullptr, nullptr};
  long long host_step = 0;
  long launches = 0;
  unsigned *d_flags = nullptr;  // every model's flags OR-ed (ps_batch_sync)
  unsigned *h_flags = nullptr;  // pinned copy of it
};

static int batch_fail(const char *msg)
{
  ps_set_error_msg(msg);
  return PS_EINVAL;
}

static int batch_cuda(cudaError_t e, const char *where)
{
  char buf[512];
  std::snprintf(buf, sizeof(buf), "%s: %s", where, cudaGetErrorString(e));
  ps_set_error_msg(buf);
  return PS_ECUDA;
}

#define BCK(call)                                          \
  do {                                                     \
    cudaError_t e_ = (call);                               \
    if (e_ != cudaSuccess) return batch_cuda(e_, #call);   \
  } while (0)

static int encode_box(const ps::Params &p, double *base, int tx, int ty, CUtensorMap *tm)
{
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if (!encode) {
    cudaDriverEntryPointQueryResult q;
    void *fn = nullptr;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                                     cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn)
      return batch_fail("cuTensorMapEncodeTiled entry point not available");
    encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  cuuint64_t dims[4] = {(cuuint64_t)(p.ntot[0] + p.xoff), (cuuint64_t)p.ntot[1],
                        (cuuint64_t)p.ntot[2], (cuuint64_t)p.nvar};
  cuuint64_t strides[3] = {(cuuint64_t)p.px * 8, (cuuint64_t)p.px * p.ntot[1] * 8,
                           (cuuint64_t)p.vstride * 8};
  cuuint32_t box[4] = {(cuuint32_t)(tx + 4), (cuuint32_t)(ty + 4), 1u, (cuuint32_t)p.nvar};
  cuuint32_t estr[4] = {1, 1, 1, 1};
  CUresult r = encode(tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 4, base, dims, strides, box, estr,
                      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                      CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return batch_fail("ps_batch: tensor map rejected");
  return 0;
}

template <class T>
static int upload_list(const std::vector<T> &v, T **dst)
{
  cudaFree(*dst);
  *dst = nullptr;
  if (v.empty()) return 0;
  BCK(cudaMalloc(dst, v.size() * sizeof(T)));
  BCK(cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  return 0;
}

// Models of each group: sorted by cells, dealt out in turn so that every
// group gets a like share of each grid size.
static void batch_partition(ps_batch *b)
{
  std::vector<int> order(b->n);
  for (int m = 0; m < b->n; m++) order[m] = m;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    const ps::Params &px = b->ctx[x]->p, &py = b->ctx[y]->p;
    return (long)px.nx[0] * px.nx[1] > (long)py.nx[0] * py.nx[1];
  });
  for (BatchGroup &g : b->grp) g.models.clear();
  for (int k = 0; k < b->n; k++) b->grp[k % b->ngroups].models.push_back(order[k]);
  for (BatchGroup &g : b->grp) std::sort(g.models.begin(), g.models.end());
}

// Rebuilds the per-model descriptors and every group's work lists for the
// current shape choice and uploads them.
static int batch_upload(ps_batch *b)
{
  b->total_cells = 0;
  for (int m = 0; m < b->n; m++) {
    ps_ctx *c = b->ctx[m];
    ps::BatchModel &M = b->h_models[m];
    const ps::Params &p = c->p;
    const int sh = b->shape[m], tx = ps::kShapeX[sh], ty = ps::kShapeY[sh];
    int r = encode_box(p, c->V, tx, ty, &M.tm[0]);
    if (!r) r = encode_box(p, c->Vs, tx, ty, &M.tm[1]);
    if (r) return r;
    for (int st = 0; st < 2; st++) {
      ps::WindStageArgs A = c->wind->a;
      A.s.Vn = c->V;
      A.s.Vout = st == 0 ? c->Vs : c->V;
      A.s.Us = c->Us;
      for (int d = 0; d < 3; d++) {
        A.s.dtdx[d] = c->dtdx[d];
        A.s.inv_dx[d] = c->inv_dx[d];
      }
      A.s.sc = c->sc;
      A.s.p = p;
      M.st[st] = A;
    }
    std::memset(&M.fin, 0, sizeof(M.fin));
    M.fin.sc = c->sc;
    M.fin.hist_dt = c->hist;
    for (int d = 0; d < 3; d++) {
      M.fin.dtdx[d] = c->dtdx[d];
      M.fin.dx[d] = c->dx[d];
    }
    M.fin.p = p;
    M.fin.mode = ps::MODE_STEP;
    b->total_cells += (long)p.nx[0] * p.nx[1];
  }
  BCK(cudaMemcpy(b->d_models, b->h_models.data(), sizeof(ps::BatchModel) * b->n,
                 cudaMemcpyHostToDevice));
  long qoff = 0;
  for (BatchGroup &g : b->grp) {
    std::vector<ps::TileItem> items[ps::kNumShapes];
    std::vector<ps::BlockItem> cells, x2, cells128, shock;
    g.cells = 0;
    for (int m : g.models) {
      const ps::Params &p = b->ctx[m]->p;
      const int sh = b->shape[m], tx = ps::kShapeX[sh], ty = ps::kShapeY[sh];
      const int ntx = (p.nx[0] + tx - 1) / tx, nty = (p.nx[1] + ty - 1) / ty;
      for (int by = 0; by < nty; by++)
        for (int bx = 0; bx < ntx; bx++) items[sh].push_back({m, bx, by, 0});
      const int nc = (p.nx[0] * p.nx[1] + 255) / 256, n2 = (p.ntot[0] * 2 * p.beg[1] + 255) / 256;
      for (int k = 0; k < nc; k++) cells.push_back({m, k});
      const int nc128 = (p.nx[0] * p.nx[1] + 127) / 128;
      for (int k = 0; k < nc128; k++) cells128.push_back({m, k});
      for (int k = 0; k < n2; k++) x2.push_back({m, k});
      if (ps::needs_shock_flags(p))
        for (int k = 0; k < (p.ntot[0] * p.ntot[1] + 255) / 256; k++) shock.push_back({m, k});
      g.cells += (long)p.nx[0] * p.nx[1];
    }
    for (int sh = 0; sh < ps::kNumShapes; sh++) {
      if (int r = upload_list(items[sh], &g.d_items[sh])) return r;
      g.nitems[sh] = (int)items[sh].size();
    }
    if (int r = upload_list(cells, &g.d_cells)) return r;
    if (int r = upload_list(x2, &g.d_x2)) return r;
    if (int r = upload_list(cells128, &g.d_cells128)) return r;
    if (int r = upload_list(shock, &g.d_shock)) return r;
    if (int r = upload_list(g.models, &g.d_list)) return r;
    g.ncells_blocks = (int)cells.size();
    g.nx2_blocks = (int)x2.size();
    g.ncells128 = (int)cells128.size();
    g.nshock_blocks = (int)shock.size();
    g.queue_off = qoff;
    qoff += g.cells;
  }
  for (int k = 0; k < 3; k++) {
    if (b->g[k]) cudaGraphExecDestroy(b->g[k]);
    b->g[k] = nullptr;
  }
  return 0;
}

// The stage kernels of a group's tile-shape sets run side by side (a fork
// onto the shape streams and a join back), so that one set's tail overlaps
// the others' work; the sets touch disjoint models.
static int batch_stage(ps_batch *b, BatchGroup &g, int stage, cudaStream_t st0)
{
  int first = -1;
  for (int s = 0; s < ps::kNumShapes; s++)
    if (g.nitems[s] && first < 0) first = s;
  BCK(cudaEventRecord(g.fork, st0));
  for (int s = 0; s < ps::kNumShapes; s++) {
    if (!g.nitems[s]) continue;
    cudaStream_t st = s == first ? st0 : g.side[s];
    if (s != first) BCK(cudaStreamWaitEvent(st, g.fork, 0));
    const void *k = ps::batch_kernel(b->nvar, b->char_lim, s, b->lim, b->solver, stage);
    void *args[2] = {&b->d_models, &g.d_items[s]};
    BCK(cudaLaunchKernel(k, dim3(g.nitems[s]), dim3(ps::kShapeNT[s]), args,
                         ps::batch_smem(b->nvar, s), st));
    b->launches++;
    if (s != first) BCK(cudaEventRecord(g.join[s], st));
  }
  for (int s = 0; s < ps::kNumShapes; s++)
    if (g.nitems[s] && s != first) BCK(cudaStreamWaitEvent(st0, g.join[s], 0));
  return 0;
}

static int batch_bnd(ps_batch *b, BatchGroup &g, int stage, cudaStream_t st)
{
  if (g.models.empty()) return 0;
  if (b->nvar == 7) {
    ps::k_batch_bnd_x1<7><<<g.ncells_blocks, 64, 0, st>>>(b->d_models, g.d_cells, stage);
    ps::k_batch_bnd_x2<7><<<g.nx2_blocks, 256, 0, st>>>(b->d_models, g.d_x2, stage);
  } else {
    ps::k_batch_bnd_x1<6><<<g.ncells_blocks, 64, 0, st>>>(b->d_models, g.d_cells, stage);
    ps::k_batch_bnd_x2<6><<<g.nx2_blocks, 256, 0, st>>>(b->d_models, g.d_x2, stage);
  }
  b->launches += 2;
  if (stage == 1 && g.nshock_blocks) {
    ps::k_batch_shock<<<g.nshock_blocks, 256, 0, st>>>(b->d_models, g.d_shock);
    b->launches++;
  }
  return 0;
}

ps::SgNet ps_sg_net(const ps_surrogate *s);
ps::SgBox ps_sg_boxv(const ps_surrogate *s);
unsigned long long *ps_sg_stats_dev(ps_surrogate *s);

static int batch_cool(ps_batch *b, BatchGroup &g, cudaStream_t st)
{
  if (!b->cooling || g.models.empty()) return 0;
  if (b->sg) {
    const int gi = (int)(&g - b->grp.data());
    int *qcount = b->sg_qcount + gi;
    int2 *queue = b->sg_queue + g.queue_off;
    BCK(cudaMemsetAsync(qcount, 0, sizeof(int), st));
    const int grid = std::min(g.ncells128, b->num_sms * ps::kInfCtasPerSm);
    ps::k_batch_sg_cool<<<grid, 128, ps::kInfBytes, st>>>(
        b->d_models, g.d_cells128, g.ncells128, b->d_xi, b->d_tr, b->d_pre, ps_sg_net(b->sg),
        ps_sg_boxv(b->sg), b->sg_use_net, queue, qcount, ps_sg_stats_dev(b->sg));
    // one warp per CTA: the few queued cells spread over every SM instead
    // of sharing the FP64 pipes of the first few
    ps::k_batch_sg_fallback<<<4864, 32, 0, st>>>(b->d_models, b->d_xi, b->d_tr, b->d_pre, queue,
                                                 qcount);
    b->launches += 2;
    return 0;
  }
  if (b->cooling == 2) {   // the ODE path
    ps::k_batch_ode<<<g.ncells_blocks, 256, 0, st>>>(b->d_models, g.d_cells, b->d_xi, b->d_tr,
                                                     b->d_pre);
    b->launches++;
    return 0;
  }
  ps::k_batch_blondin<<<g.ncells_blocks, 256, 0, st>>>(b->d_models, g.d_cells, b->d_xi, b->d_tr,
                                                       b->d_pre);
  b->launches++;
  return 0;
}

static int batch_finish(ps_batch *b, BatchGroup &g, cudaStream_t st)
{
  if (g.models.empty()) return 0;
  ps::k_batch_finish<<<(unsigned)g.models.size(), 256, 0, st>>>(b->d_models, g.d_list);
  b->launches++;
  return 0;
}

// One step of one group on stream st.
static int batch_step_group(ps_batch *b, BatchGroup &g, int odd, cudaStream_t st)
{
  int r = 0;
  if (odd) r = batch_cool(b, g, st);
  for (int stage = 1; !r && stage <= 2; stage++) {
    r = batch_bnd(b, g, stage, st);
    if (!r) r = batch_stage(b, g, stage, st);
  }
  if (!r && !odd) r = batch_cool(b, g, st);
  if (!r) r = batch_finish(b, g, st);
  return r;
}

// The steps `odd` (a list of 0 / 1) of every group, each group's steps in
// order on its own stream (forked from and joined back to the batch's
// stream; a single group runs on the batch's stream itself).
static int batch_steps(ps_batch *b, const int *odd, int nsteps)
{
  if (b->ngroups == 1) {
    for (int k = 0; k < nsteps; k++)
      if (int r = batch_step_group(b, b->grp[0], odd[k], b->stream)) return r;
    return 0;
  }
  BCK(cudaEventRecord(b->fork, b->stream));
  for (BatchGroup &g : b->grp) {
    BCK(cudaStreamWaitEvent(g.st, b->fork, 0));
    for (int k = 0; k < nsteps; k++)
      if (int r = batch_step_group(b, g, odd[k], g.st)) return r;
    BCK(cudaEventRecord(g.done, g.st));
  }
  for (BatchGroup &g : b->grp) BCK(cudaStreamWaitEvent(b->stream, g.done, 0));
  return 0;
}

static void batch_free_groups(ps_batch *b)
{
  for (BatchGroup &g : b->grp) {
    for (int s = 0; s < ps::kNumShapes; s++) {
      cudaFree(g.d_items[s]);
      if (g.side[s]) cudaStreamDestroy(g.side[s]);
      if (g.join[s]) cudaEventDestroy(g.join[s]);
    }
    cudaFree(g.d_cells);
    cudaFree(g.d_x2);
    cudaFree(g.d_cells128);
    cudaFree(g.d_shock);
    cudaFree(g.d_list);
    if (g.st) cudaStreamDestroy(g.st);
    if (g.fork) cudaEventDestroy(g.fork);
    if (g.done) cudaEventDestroy(g.done);
  }
  b->grp.clear();
}

static int batch_make_groups(ps_batch *b, int ngroups)
{
  batch_free_groups(b);
  b->ngroups = std::max(1, std::min(ngroups, b->n));
  b->grp.resize(b->ngroups);
  for (BatchGroup &g : b->grp) {
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&g.st, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&g.fork, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&g.done, cudaEventDisableTiming)) != cudaSuccess)
      return batch_cuda(e, "ps_batch: group streams");
    for (int k = 0; k < ps::kNumShapes; k++)
      if ((e = cudaStreamCreateWithFlags(&g.side[k], cudaStreamNonBlocking)) != cudaSuccess ||
          (e = cudaEventCreateWithFlags(&g.join[k], cudaEventDisableTiming)) != cudaSuccess)
        return batch_cuda(e, "ps_batch: group streams");
  }
  batch_partition(b);
  return 0;
}

static void batch_free(ps_batch *b)
{
  if (!b) return;
  for (int k = 0; k < 3; k++)
    if (b->g[k]) cudaGraphExecDestroy(b->g[k]);
  cudaFree(b->d_models);
  batch_free_groups(b);
  cudaFree(b->d_xi);
  cudaFree(b->d_tr);
  cudaFree(b->d_pre);
  cudaFree(b->sg_queue);
  cudaFree(b->sg_qcount);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->own_stream) cudaStreamDestroy(b->own_stream);
  cudaFree(b->d_flags);
  if (b->h_flags) cudaFreeHost(b->h_flags);
  delete b;
}

// Default number of model groups: two (one for a single model).  On the
// 64-model benchmark batch two groups measured 13.64 ms a step against
// 13.74 ms for one: one group's cooling fallback (a few thousand cells, a
// latency-bound tail of about 0.3 ms on an otherwise idle GPU) overlaps
// the other group's work.  Four groups measured the same as two (13.64
// ms): the stage kernels fill the GPU either way, and each group pays the
// learned step's set-up and tail.
static int default_groups(int n) { return n >= 2 ? 2 : 1; }

extern "C" int ps_batch_create(ps_ctx **ctxs, int n, ps_batch **out)
{
  if (!ctxs || n <= 0 || !out) return batch_fail("ps_batch_create: bad arguments");
  *out = nullptr;
  for (int m = 0; m < n; m++) {
    ps_ctx *c = ctxs[m];
    if (!c || !c->wind) return batch_fail("ps_batch_create: every model needs ps_set_wind");
    if (ps_wind_check(c, "ps_batch_create")) return PS_ESTATE;
    if (c->p.limiter != ctxs[0]->p.limiter || c->p.solver != ctxs[0]->p.solver ||
        c->p.cooling != ctxs[0]->p.cooling || c->host_step != ctxs[0]->host_step ||
        c->p.nvar != ctxs[0]->p.nvar || c->p.char_lim != ctxs[0]->p.char_lim)
      return batch_fail("ps_batch_create: models must share limiter, solver, characteristic "
                        "limiting, cooling, variables and step");
  }
  ps_batch *b = new ps_batch();
  b->n = n;
  b->ctx.assign(ctxs, ctxs + n);
  b->h_models.resize(n);
  b->shape.assign(n, 0);
  b->lim = ctxs[0]->p.limiter;
  b->solver = ctxs[0]->p.solver;
  b->cooling = ctxs[0]->p.cooling;
  b->nvar = ctxs[0]->p.nvar;
  b->char_lim = ctxs[0]->p.char_lim != 0;
  b->host_step = ctxs[0]->host_step;
  cudaError_t e;
  if ((e = cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaMalloc(&b->d_models, sizeof(ps::BatchModel) * n)) != cudaSuccess ||
      (e = cudaMalloc(&b->d_xi, sizeof(double *) * n)) != cudaSuccess ||
      (e = cudaMalloc(&b->d_tr, sizeof(double *) * n)) != cudaSuccess ||
      (e = cudaMalloc(&b->d_pre, sizeof(double *) * n)) != cudaSuccess ||
      (e = cudaMalloc(&b->d_flags, sizeof(unsigned))) != cudaSuccess ||
      (e = cudaMallocHost(&b->h_flags, sizeof(unsigned))) != cudaSuccess ||
      (e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming)) != cudaSuccess) {
    batch_free(b);
    return batch_cuda(e, "ps_batch_create");
  }
  b->stream = b->own_stream;
  if (int r = batch_make_groups(b, default_groups(n))) {
    batch_free(b);
    return r;
  }
  {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&b->num_sms, cudaDevAttrMultiProcessorCount, dev);
  }
  std::vector<const double *> xi(n), tr(n), pre(n);
  for (int m = 0; m < n; m++) {
    xi[m] = ctxs[m]->wind->xi;
    tr[m] = ctxs[m]->wind->tr;
    pre[m] = ctxs[m]->wind->pre;
    cudaStreamSynchronize(ctxs[m]->stream);
  }
  cudaMemcpy(b->d_xi, xi.data(), sizeof(double *) * n, cudaMemcpyHostToDevice);
  cudaMemcpy(b->d_tr, tr.data(), sizeof(double *) * n, cudaMemcpyHostToDevice);
  cudaMemcpy(b->d_pre, pre.data(), sizeof(double *) * n, cudaMemcpyHostToDevice);
  for (int s = 0; s < ps::kNumShapes; s++) {
    for (int st = 1; st <= 2; st++) {
      e = cudaFuncSetAttribute(ps::batch_kernel(b->nvar, b->char_lim, s, b->lim, b->solver, st),
                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)ps::batch_smem(b->nvar, s));
      if (e != cudaSuccess) {
        batch_free(b);
        return batch_cuda(e, "ps_batch_create: smem attribute");
      }
    }
  }
  int r = batch_upload(b);
  if (r) {
    batch_free(b);
    return r;
  }
  *out = b;
  return 0;
}

// Number of model groups whose steps run as parallel branches (1 to the
// number of models); the models are dealt out by size.  No reference
// counterpart.
extern "C" int ps_batch_set_groups(ps_batch *b, int ngroups)
{
  if (!b || ngroups < 1) return batch_fail("ps_batch_set_groups: bad arguments");
  BCK(cudaStreamSynchronize(b->stream));
  if (int r = batch_make_groups(b, ngroups)) return r;
  if (b->sg) {   // queue counters, one per group
    cudaFree(b->sg_qcount);
    b->sg_qcount = nullptr;
    BCK(cudaMalloc(&b->sg_qcount, sizeof(int) * b->ngroups));
  }
  return batch_upload(b);
}

extern "C" int ps_batch_destroy(ps_batch *b)
{
  if (!b) return PS_EINVAL;
  cudaStreamSynchronize(b->stream);
  batch_free(b);
  return 0;
}

extern "C" int ps_batch_set_shape(ps_batch *b, int model, int shape)
{
  if (!b || model < -1 || model >= b->n || shape < 0 || shape >= ps::kNumShapes)
    return batch_fail("ps_batch_set_shape: bad arguments");
  if (model < 0)
    std::fill(b->shape.begin(), b->shape.end(), shape);
  else
    b->shape[model] = shape;
  BCK(cudaStreamSynchronize(b->stream));
  return batch_upload(b);
}

extern "C" int ps_batch_get_shape(const ps_batch *b, int model, int *tx, int *ty)
{
  if (!b || model < 0 || model >= b->n) return batch_fail("ps_batch_get_shape: bad arguments");
  if (tx) *tx = ps::kShapeX[b->shape[model]];
  if (ty) *ty = ps::kShapeY[b->shape[model]];
  return b->shape[model];
}

// For every distinct grid size of the batch, time the stage-1 kernel of
// those models with each candidate tile shape (CUDA events, `reps`
// launches after one warm-up) and keep the fastest.  The state is not
// changed: the scalars each model's stage 1 touches are saved and put back.
extern "C" int ps_batch_autotune(ps_batch *b, int reps)
{
  if (!b) return PS_EINVAL;
  if (reps <= 0) reps = 5;
  BCK(cudaStreamSynchronize(b->stream));
  std::vector<ps::Scalars> saved(b->n);
  for (int m = 0; m < b->n; m++)
    BCK(cudaMemcpy(&saved[m], b->ctx[m]->sc, sizeof(ps::Scalars), cudaMemcpyDeviceToHost));
  std::map<std::pair<int, int>, std::vector<int>> groups;
  for (int m = 0; m < b->n; m++) groups[{b->ctx[m]->p.nx[0], b->ctx[m]->p.nx[1]}].push_back(m);
  const std::vector<int> orig = b->shape;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  for (auto &g : groups) {
    float best = 1e30f;
    int best_s = 0;
    for (int s = 0; s < ps::kNumShapes; s++) {
      // only this group's models are timed: the others get no items
      std::vector<ps::TileItem> items;
      for (int m : g.second) {
        ps_ctx *c = b->ctx[m];
        const int tx = ps::kShapeX[s], ty = ps::kShapeY[s];
        const int ntx = (c->p.nx[0] + tx - 1) / tx, nty = (c->p.nx[1] + ty - 1) / ty;
        for (int by = 0; by < nty; by++)
          for (int bx = 0; bx < ntx; bx++) items.push_back({m, bx, by, 0});
        b->shape[m] = s;
      }
      int r = batch_upload(b);
      if (r) return r;
      ps::TileItem *d_items = nullptr;
      BCK(cudaMalloc(&d_items, items.size() * sizeof(ps::TileItem)));
      BCK(cudaMemcpy(d_items, items.data(), items.size() * sizeof(ps::TileItem),
                     cudaMemcpyHostToDevice));
      const void *k = ps::batch_kernel(b->nvar, b->char_lim, s, b->lim, b->solver, 1);
      void *args[2] = {&b->d_models, &d_items};
      BCK(cudaLaunchKernel(k, dim3((unsigned)items.size()), dim3(ps::kShapeNT[s]), args,
                           ps::batch_smem(b->nvar, s), b->stream));
      BCK(cudaEventRecord(e0, b->stream));
      for (int it = 0; it < reps; it++)
        BCK(cudaLaunchKernel(k, dim3((unsigned)items.size()), dim3(ps::kShapeNT[s]), args,
                             ps::batch_smem(b->nvar, s), b->stream));
      BCK(cudaEventRecord(e1, b->stream));
      BCK(cudaEventSynchronize(e1));
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      cudaFree(d_items);
      if (ms < best) {
        best = ms;
        best_s = s;
      }
    }
    for (int m : g.second) b->shape[m] = best_s;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  (void)orig;
  for (int m = 0; m < b->n; m++)
    BCK(cudaMemcpy(b->ctx[m]->sc, &saved[m], sizeof(ps::Scalars), cudaMemcpyHostToDevice));
  return batch_upload(b);
}

static int batch_graph(ps_batch *b, int kind, cudaGraphExec_t *out)
{
  cudaGraph_t g;
  const long before = b->launches;
  BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  static const int kSteps[3][2] = {{0, 0}, {1, 0}, {0, 1}};
  const int r = batch_steps(b, kSteps[kind], kind == 2 ? 2 : 1);
  cudaError_t e = cudaStreamEndCapture(b->stream, &g);
  b->launches = before;
  if (r) return r;
  if (e != cudaSuccess) return batch_cuda(e, "ps_batch: capture");
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return batch_cuda(e, "ps_batch: instantiate");
  return 0;
}

extern "C" int ps_batch_run(ps_batch *b, int nsteps)
{
  if (!b || nsteps < 0) return PS_EINVAL;
  long per_step = 0;   // kernels of one step over every group
  for (const BatchGroup &g : b->grp) {
    if (g.models.empty()) continue;
    int nshape = 0;
    for (int s = 0; s < ps::kNumShapes; s++) nshape += g.nitems[s] > 0;
    per_step += 4 + 2 * nshape + (b->cooling ? (b->sg ? 2 : 1) : 0) + 1 +
                (g.nshock_blocks ? 1 : 0);
  }
  for (int k = 0; k < 3; k++)
    if (!b->g[k]) {
      int r = batch_graph(b, k, &b->g[k]);
      if (r) return r;
    }
  b->host_step = b->ctx[0]->host_step;   // follows ps_restore_state of the contexts
  int left = nsteps;
  while (left > 0) {
    const int odd = (int)(b->host_step & 1);
    if (!odd && left >= 2) {
      BCK(cudaGraphLaunch(b->g[2], b->stream));
      b->launches += 2 * per_step;
      b->host_step += 2;
      left -= 2;
    } else {
      BCK(cudaGraphLaunch(b->g[odd], b->stream));
      b->launches += per_step;
      b->host_step += 1;
      left -= 1;
    }
  }
  for (ps_ctx *c : b->ctx) c->host_step = b->host_step;
  BCK(cudaGetLastError());
  return 0;
}

namespace ps {

// Up to kCopyList arrays copied by one launch, blockIdx.y = array: the
// state transfer between pinned host memory and the device when every host
// array is device-accessible (GPU loads or stores over the host link, which
// on this part run faster than the copy engines).
constexpr int kCopyList = 128;
struct CopyList {
  const double *src[kCopyList];
  double *dst[kCopyList];
  long long count[kCopyList];
};

__global__ void __launch_bounds__(256) k_copy_list(const __grid_constant__ CopyList L)
{
  const int m = blockIdx.y;
  const long long n = L.count[m], n2 = n / 2;
  const double2 *s2 = reinterpret_cast<const double2 *>(L.src[m]);
  double2 *d2 = reinterpret_cast<double2 *>(L.dst[m]);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n2;
       i += (long long)gridDim.x * blockDim.x)
    d2[i] = s2[i];
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) L.dst[m][n - 1] = L.src[m][n - 1];
}

}  // namespace ps

// The device address of a pinned (page-locked or registered) host array, or
// NULL when the array is not pinned or not 16-byte aligned.
static const void *pinned_device_ptr(const void *h)
{
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, h) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
  if (reinterpret_cast<uintptr_t>(a.devicePointer) % 16 != 0) return nullptr;
  return a.devicePointer;
}

// All models' arrays by the copy kernel when every host array is pinned and
// every device state is one linear block; returns 1 when it did the copies.
static int batch_copy_kernel(ps_batch *b, const double *const *host, bool to_device)
{
  for (int m = 0; m < b->n; m++) {
    const ps::Params &p = b->ctx[m]->p;
    if (p.px != p.ntot[0] || p.xoff != 0 || !pinned_device_ptr(host[m])) return 0;
  }
  for (int m0 = 0; m0 < b->n; m0 += ps::kCopyList) {
    ps::CopyList L;
    const int cnt = std::min(ps::kCopyList, b->n - m0);
    for (int k = 0; k < cnt; k++) {
      ps_ctx *c = b->ctx[m0 + k];
      const double *h = static_cast<const double *>(pinned_device_ptr(host[m0 + k]));
      L.count[k] = (long long)c->p.ntot[0] * c->p.ntot[1] * c->p.ntot[2] * c->p.nvar;
      L.src[k] = to_device ? h : c->V;
      L.dst[k] = to_device ? c->V : const_cast<double *>(h);
    }
    ps::k_copy_list<<<dim3(2 * (unsigned)b->num_sms, (unsigned)cnt), 256, 0, b->stream>>>(L);
    b->launches++;
  }
  return cudaGetLastError() == cudaSuccess ? 1 : -1;
}

// Every model's Data.Vc between the host arrays and the device by the copy
// engines, queued on the batch's stream: one linear copy per model when its
// rows lie back to back, else a 2-D copy.
static int batch_copy_engines(ps_batch *b, const double *const *host, bool to_device)
{
  for (int m = 0; m < b->n; m++) {
    ps_ctx *c = b->ctx[m];
    const ps::Params &p = c->p;
    const size_t rows = (size_t)p.ntot[1] * p.ntot[2] * p.nvar;
    double *h = const_cast<double *>(host[m]);
    cudaError_t e;
    if (p.px == p.ntot[0] && p.xoff == 0)
      e = to_device ? cudaMemcpyAsync(c->V, h, rows * p.ntot[0] * 8, cudaMemcpyHostToDevice,
                                      b->stream)
                    : cudaMemcpyAsync(h, c->V, rows * p.ntot[0] * 8, cudaMemcpyDeviceToHost,
                                      b->stream);
    else
      e = to_device
              ? cudaMemcpy2DAsync(c->V + p.xoff, (size_t)p.px * 8, h, (size_t)p.ntot[0] * 8,
                                  (size_t)p.ntot[0] * 8, rows, cudaMemcpyHostToDevice, b->stream)
              : cudaMemcpy2DAsync(h, (size_t)p.ntot[0] * 8, c->V + p.xoff, (size_t)p.px * 8,
                                  (size_t)p.ntot[0] * 8, rows, cudaMemcpyDeviceToHost, b->stream);
    if (e != cudaSuccess) return batch_cuda(e, to_device ? "ps_batch: state in" : "ps_batch: state out");
  }
  return 0;
}

static int batch_check_host(const ps_batch *b, const void *arr, const char *what)
{
  if (!b || !arr) return batch_fail(what);
  const double *const *h = static_cast<const double *const *>(arr);
  for (int m = 0; m < b->n; m++)
    if (!h[m]) return batch_fail(what);
  return 0;
}

// Every model's Data.Vc from host arrays (Vc[m], [nv][k][j][i] over its
// total box, pinned for the full transfer speed), all copies queued on the
// batch's stream; the models' time state is kept.
extern "C" int ps_batch_set_states(ps_batch *b, const double *const *Vc)
{
  if (int r = batch_check_host(b, Vc, "ps_batch_set_states: bad arguments")) return r;
  const int k = batch_copy_kernel(b, Vc, true);
  if (k < 0) return batch_fail("ps_batch_set_states: copy kernel launch failed");
  return k ? 0 : batch_copy_engines(b, Vc, true);
}

// Every model's Data.Vc into host arrays, queued on the batch's stream after
// the work issued so far, then one synchronisation.
extern "C" int ps_batch_get_states(ps_batch *b, double *const *Vc)
{
  if (int r = batch_check_host(b, Vc, "ps_batch_get_states: bad arguments")) return r;
  const int k = batch_copy_kernel(b, Vc, false);
  if (k < 0) return batch_fail("ps_batch_get_states: copy kernel launch failed");
  if (!k)
    if (int r = batch_copy_engines(b, Vc, false)) return r;
  BCK(cudaStreamSynchronize(b->stream));
  return 0;
}

// The same transfers by the copy engines only, queued without waiting, so
// that the copies of one batch overlap the steps of another batch on the
// GPU's multiprocessors; the host arrays (pinned) stay untouched until
// ps_batch_sync returns.
extern "C" int ps_batch_set_states_async(ps_batch *b, const double *const *Vc)
{
  if (int r = batch_check_host(b, Vc, "ps_batch_set_states_async: bad arguments")) return r;
  return batch_copy_engines(b, Vc, true);
}

extern "C" int ps_batch_get_states_async(ps_batch *b, double *const *Vc)
{
  if (int r = batch_check_host(b, Vc, "ps_batch_get_states_async: bad arguments")) return r;
  return batch_copy_engines(b, Vc, false);
}

// Waits for the batch's stream; every model's flags OR-ed, gathered by one
// small kernel and read back in one copy (a copy per model cost about 10 us
// each, 0.3 ms for 32 models, on the host's critical path between steps).
extern "C" int ps_batch_sync(ps_batch *b)
{
  if (!b) return PS_EINVAL;
  ps::k_batch_gather_flags<<<1, 256, 0, b->stream>>>(b->d_models, b->n, b->d_flags);
  BCK(cudaGetLastError());
  BCK(cudaMemcpyAsync(b->h_flags, b->d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost,
                      b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  return (int)*b->h_flags;
}

extern "C" int ps_batch_set_stream(ps_batch *b, void *stream)
{
  if (!b) return PS_EINVAL;
  BCK(cudaStreamSynchronize(b->stream));
  b->stream = stream ? static_cast<cudaStream_t>(stream) : b->own_stream;
  return 0;
}

extern "C" long ps_batch_launch_count(const ps_batch *b) { return b ? b->launches : -1; }

extern "C" int ps_batch_set_surrogate(ps_batch *b, ps_surrogate *s, int use_net)
{
  if (!b) return batch_fail("ps_batch_set_surrogate: null batch");
  if (s && b->cooling == 2)
    return batch_fail("ps_batch_set_surrogate: the learned step replaces BLONDIN's implicit "
                      "solve, not the ODE cooling path");
  BCK(cudaStreamSynchronize(b->stream));
  if (s && !b->sg_queue) {   // each group's slice of the queue and its counter
    BCK(cudaMalloc(&b->sg_queue, sizeof(int2) * (size_t)b->total_cells));
    BCK(cudaMalloc(&b->sg_qcount, sizeof(int) * b->ngroups));
  }
  b->sg = s;
  b->sg_use_net = use_net;
  for (int k = 0; k < 3; k++) {
    if (b->g[k]) cudaGraphExecDestroy(b->g[k]);
    b->g[k] = nullptr;
  }
  return 0;
}

// One step issued launch by launch with CUDA events between the phases:
// ms[0] = the stage-1 launches, ms[1] = the stage-2 launches, ms[2] = the
// rest (boundaries, split source, dt kernel).  Advances the models.
extern "C" int ps_batch_time_step_kernels(ps_batch *b, float *ms)
{
  if (!b || !ms) return PS_EINVAL;
  cudaEvent_t ev[8];
  for (int k = 0; k < 8; k++) BCK(cudaEventCreate(&ev[k]));
  b->host_step = b->ctx[0]->host_step;
  const int odd = (int)(b->host_step & 1);
  int r = 0;
  cudaStream_t st = b->stream;
  // phase by phase, every group's launches of a phase in turn on one stream
  BCK(cudaEventRecord(ev[0], st));
  for (BatchGroup &g : b->grp)
    if (!r && odd) r = batch_cool(b, g, st);
  for (BatchGroup &g : b->grp)
    if (!r) r = batch_bnd(b, g, 1, st);
  BCK(cudaEventRecord(ev[1], st));
  for (BatchGroup &g : b->grp)
    if (!r) r = batch_stage(b, g, 1, st);
  BCK(cudaEventRecord(ev[2], st));
  for (BatchGroup &g : b->grp)
    if (!r) r = batch_bnd(b, g, 2, st);
  BCK(cudaEventRecord(ev[3], st));
  for (BatchGroup &g : b->grp)
    if (!r) r = batch_stage(b, g, 2, st);
  BCK(cudaEventRecord(ev[4], st));
  for (BatchGroup &g : b->grp)
    if (!r && !odd) r = batch_cool(b, g, st);
  for (BatchGroup &g : b->grp)
    if (!r) r = batch_finish(b, g, st);
  BCK(cudaEventRecord(ev[5], st));
  BCK(cudaEventSynchronize(ev[5]));
  float t[5];
  for (int k = 0; k < 5; k++) cudaEventElapsedTime(&t[k], ev[k], ev[k + 1]);
  for (int k = 0; k < 8; k++) cudaEventDestroy(ev[k]);
  if (r) return r;
  BCK(cudaGetLastError());
  b->host_step++;
  for (ps_ctx *c : b->ctx) c->host_step = b->host_step;
  ms[0] = t[1];
  ms[1] = t[3];
  ms[2] = t[0] + t[2] + t[4];
  return 0;
}
