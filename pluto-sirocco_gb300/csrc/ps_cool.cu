// ps_cool.cu -- the operator-split BLONDIN step on Cartesian contexts at a
// constant ionisation parameter (the 3-D periodic cooling configuration):
// SplitSource (Src/split_source.c:28-79) with BlondinCooling
// (Src/Cooling/BLONDIN/cooling.c:50-165), xi and T_x fixed instead of read
// from sirocco_xi / sirocco_t_r.  Same per-cell solve as the wind's
// (bracket + Brent), or the learned step when a surrogate is attached.
#include "ps_wind_dev.cuh"

#include <cmath>
#include <cstdio>
#include <cstring>

extern "C" void ps_set_error_msg(const char *msg);
void ps_ctx_invalidate_graphs(ps_ctx *c);
int ps_sg_cool_launch(ps_ctx *c);

namespace ps {

void fill_ghosts_2d(double *V, const Params &p, cudaStream_t s);
void fill_ghosts_3d(double *V, const Params &p, cudaStream_t s);

__global__ void k_blondin_cart(double *V, const Params p, const WindParams w, Scalars *sc)
{
  if (sc->done) return;
  const double dt = sc->dt, t = sc->t;
  const long long n = (long long)p.nx[0] * p.nx[1] * p.nx[2];
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x)
    blondin_cell(V, nullptr, nullptr, p, w, nullptr, sc, dt, t, q, nullptr);
}

}  // namespace ps

extern "C" int ps_set_cooling(ps_ctx *c, const ps_cooling *cp)
{
  if (!c || !cp) {
    ps_set_error_msg("ps_set_cooling: null argument");
    return PS_EINVAL;
  }
  if (c->cfg.geometry != PS_CARTESIAN || !c->cfg.cooling) {
    ps_set_error_msg("ps_set_cooling: needs a Cartesian context with cooling = 1");
    return PS_EINVAL;
  }
  if (!(cp->xi > 0) || !(cp->t_x > 0) || !(cp->mu > 0) || !(cp->unit_density > 0) ||
      !(cp->unit_length > 0) || !(cp->unit_velocity > 0)) {
    ps_set_error_msg("ps_set_cooling: xi, t_x, mu and the units must be positive");
    return PS_EINVAL;
  }
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {
    ps_set_error_msg(cudaGetErrorString(e));
    return PS_ECUDA;
  }
  ps::WindParams &W = c->coolw;
  std::memset(&W, 0, sizeof(W));
  W.cooling = 1;
  W.unit_density = cp->unit_density;
  W.unit_length = cp->unit_length;
  W.unit_velocity = cp->unit_velocity;
  W.mu = cp->mu;
  W.kelvin = cp->unit_velocity * cp->unit_velocity * ps::kAmu / ps::kKB;
  W.t_x = cp->t_x;
  W.unit_pressure = cp->unit_density * cp->unit_velocity * cp->unit_velocity;
  W.unit_time = cp->unit_length / cp->unit_velocity;
  W.xi_const = cp->xi;
  ps::set_sg_units(W, c->cfg.gamma);
  c->cool_on = 1;
  ps_ctx_invalidate_graphs(c);
  return 0;
}

// The split-source launches of a Cartesian cooling context: the cooling
// step, then the ghost zones refilled from the cooled cells (the stage
// kernels of Cartesian contexts write the halo of the next stage
// themselves, so a change between steps has to be mirrored).
int ps_cart_cool_launch(ps_ctx *c)
{
  if (!c->p.cooling || !c->cool_on) return 0;
  if (c->sg) {
    const int r = ps_sg_cool_launch(c);
    if (r) return r;
  } else {
    const long long n = (long long)c->p.nx[0] * c->p.nx[1] * c->p.nx[2];
    const long long nb = (n + 127) / 128;
    ps::k_blondin_cart<<<(unsigned)(nb < 152 * 64 ? nb : 152 * 64), 128, 0, c->stream>>>(
        c->V, c->p, c->coolw, c->sc);
    c->launches++;
  }
  if (c->p.dims == 2)
    ps::fill_ghosts_2d(c->V, c->p, c->stream);
  else
    ps::fill_ghosts_3d(c->V, c->p, c->stream);
  c->launches++;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    ps_set_error_msg(cudaGetErrorString(e));
    return PS_ECUDA;
  }
  return 0;
}
