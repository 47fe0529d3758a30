// ps_wind.cu -- the 2-D spherical line-driven disk wind on the GPU:
// boundary kernels (internal floors and the problem's side conditions),
// the spherical stage kernel with VGradCalc and LineForce fused in, and the
// BLONDIN heating/cooling kernel; plus the host-side set-up of the
// geometry factors and of the per-cell flux-bin lists, and the step
// sequence with the Strang alternation of the split source.
//
// Reference (paths inside the reference project):
//   Boundary, floors          Src/boundary.c:56-500, problem UserDefBoundary
//   geometry                  Src/set_geometry.c:62-250, Src/States/plm_coeffs.c:30-74
//   PLM (general grid)        Src/States/plm_states.c:135-150, plm_coeffs.h:128-150
//   curvilinear RHS           Src/MHD/rhs.c:234-351, 423-630
//   sources                   Src/MHD/rhs_source.c:101-420
//   VGradCalc, bilinear       Src/LineDriven/line_connect.c:504-777
//   LineForce                 Src/LineDriven/line_connect.c:815-903
//   xi initialisation         Src/LineDriven/line_connect.c:287-306
//   BlondinCooling            Src/Cooling/BLONDIN/cooling.c:50-319
//   Strang order              Src/main.c:479-485
#include "ps_ctx.cuh"
#include "ps_physics.cuh"
#include "ps_stage.cuh"
#include "ps_tma.cuh"
#include "ps_wind.cuh"
#include "ps_wind_kernels.cuh"

#include <cudaTypedefs.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

extern "C" void ps_set_error_msg(const char *msg);

#include "ps_wind_dev.cuh"

namespace ps {

template <int NV>
__global__ void k_wind_bnd_x1(double *V, double *Us, const Params p, const WindParams w,
                              Scalars *sc, int stage)
{
  // 256 cells per 64-thread CTA, 4 cells per thread
  if (sc->done) return;
  bnd_x1_cells<NV, 4>(V, Us, p, w, stage, blockIdx.x * 256 + threadIdx.x, 64, p.nx[0] * p.nx[1]);
}

template <int NV>
__global__ void k_wind_bnd_x2(double *V, const Params p, Scalars *sc)
{
  if (sc->done) return;
  const int n = p.ntot[0] * 2 * p.beg[1];
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x)
    bnd_x2_item<NV>(V, p, q);
}

// FlagShock (Src/flag_shock.c:38-200) at the start of a step: the shocked
// zones of the total box, read by the PLM of both stages.
__global__ void k_wind_shock(unsigned char *S, const double *V, const Params p, const SphGeom g,
                             Scalars *sc)
{
  if (sc->done) return;
  const int n = p.ntot[0] * p.ntot[1];
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const int i = q % p.ntot[0], j = q / p.ntot[0];
    S[vcell(p, j, i)] = shock_zone(V, p, g, i, j);
  }
}

__global__ void k_wind_init_xi(const double *V, double *xi, double *tr, const Params p,
                               const WindParams w, const double *x1)
{
  const int n = p.nx[0] * p.nx[1];
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x)
    init_xi_cell(V, xi, tr, p, w, x1, q);
}

// CoolingSource (ODE path) over the active cells
__global__ void k_ode_cool(double *V, const double *xi_s, const double *tr_s, const Params p,
                           const WindParams w, const double *x1, Scalars *sc, const double *pre)
{
  if (sc->done) return;
  const double dt = sc->dt, t = sc->t;
  const int n = p.nx[0] * p.nx[1];
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x)
    ode_wind_cell(V, xi_s, tr_s, p, w, x1, sc, dt, t, q, pre);
}

__global__ void k_blondin(double *V, const double *xi_s, const double *tr_s, const Params p,
                          const WindParams w, const double *x1, Scalars *sc, const double *pre)
{
  if (sc->done) return;
  const double dt = sc->dt, t = sc->t;
  const int n = p.nx[0] * p.nx[1];
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x)
    blondin_cell(V, xi_s, tr_s, p, w, x1, sc, dt, t, q, pre);
}

// the single-model stage kernels (ps_wind_kernels.cuh): the primitive-PLM
// 6-variable set here, the others in ps_wind_k.cu
const void *stage_kernel_sph_other(int nv, bool ch, int lim, int solver, int stage);

static const void *stage_kernel_sph(int nv, bool ch, int lim, int solver, int stage)
{
  if (nv == 6 && !ch) return stage_kernel_sph_nv<6, false>(lim, solver, stage);
  return stage_kernel_sph_other(nv, ch, lim, solver, stage);
}

// Tile of the single-model wind kernels: cells per direction, ghost width
// loaded around them (the tensor-map box), and threads per CTA.
void wind_tile_2d(int *t, int *threads)
{
  t[0] = WindTile::X; t[1] = WindTile::Y; t[2] = WindTile::Z;
  t[3] = WindTile::HX; t[4] = WindTile::HY; t[5] = WindTile::HZ;
  *threads = TileGeom<WindTile>::NT;
}

}  // namespace ps

// ------------------------------------------------------------------
// host side
// ------------------------------------------------------------------

using ps::WindDev;

static int wind_fail(const char *msg)
{
  ps_set_error_msg(msg);
  return PS_EINVAL;
}

static int wind_cuda(cudaError_t e, const char *where)
{
  char buf[512];
  std::snprintf(buf, sizeof(buf), "%s: %s", where, cudaGetErrorString(e));
  ps_set_error_msg(buf);
  return PS_ECUDA;
}

void ps_wind_free(ps::WindDev *w)
{
  if (!w) return;
  cudaFree(w->t_fit);
  cudaFree(w->m_fit);
  cudaFree(w->geo);
  cudaFree(w->off);
  cudaFree(w->ent);
  cudaFree(w->dvds);
  cudaFree(w->pre);
  cudaFree(w->xi);
  cudaFree(w->tr);
  cudaFree(w->shock);
  delete w;
}

extern "C" int ps_set_wind(ps_ctx *c, const ps_wind *wp, const double *flux_r,
                           const double *flux_t, const double *flux_p)
{
  if (!c || !wp) return wind_fail("ps_set_wind: null argument");
  const ps::Params &p = c->p;
  if (c->cfg.geometry != PS_SPHERICAL || p.dims != 2 || p.nvar != (p.entropy ? 7 : 6))
    return wind_fail("ps_set_wind: needs a 2-D spherical context with NVAR = 6 (7 with the "
                     "entropy switch)");
  if (c->grid_mask != 3) return wind_fail("ps_set_wind: call ps_set_grid for both directions first");
  if (wp->line_force && (!flux_r || !flux_t || !flux_p))
    return wind_fail("ps_set_wind: the line force needs the three flux arrays");
  if (wp->nangles < 0 || wp->nangles > 64) return wind_fail("ps_set_wind: at most 64 flux bins");

  const int n0 = p.ntot[0], n1 = p.ntot[1];
  const double *x1 = c->hx[0], *x1m = c->hxl[0], *x1p = c->hxr[0], *dx1 = c->hdx[0];
  const double *x2 = c->hx[1], *x2m = c->hxl[1], *x2p = c->hxr[1], *dx2 = c->hdx[1];
  const double UL = wp->unit_length, UV = wp->unit_velocity, UD = wp->unit_density;

  // geometry (Src/set_geometry.c:62-240) and PLM weights (plm_coeffs.c:30-74)
  enum {
    G_X1, G_DX1, G_INVDX1, G_RINV, G_ABSX1, G_ABSX1P, G_A1F, G_DVR, G_RDR, G_RTINV, G_G0, G_X11A,
    G_X22A, G_LOCR, G_XGC1, G_FX, G_INVDVR, N1ARR
  };
  enum { H_X2, H_DX2, H_INVDX2, H_DMU, H_SXP, H_SPABS, H_SN, H_CT, H_SIN2, H_COS2, H_X11B, H_X22B,
         H_XGC2, H_FY, H_INVDMU, N2ARR };
  std::vector<double> a1((size_t)N1ARR * n0, 0.0), a2((size_t)N2ARR * n1, 0.0);
  std::vector<double> plm((size_t)12 * (n0 > n1 ? n0 : n1), 0.0);
  const int nmax = n0 > n1 ? n0 : n1;
  auto A1 = [&](int k, int i) -> double & { return a1[(size_t)k * n0 + i]; };
  auto A2 = [&](int k, int j) -> double & { return a2[(size_t)k * n1 + j]; };
  const double gm_cgs = ps::kG * wp->cent_mass;
  const double gm_code = gm_cgs / (UL * UV * UV);
  for (int i = 0; i < n0; i++) {
    const double xL = x1m[i], xR = x1p[i];
    A1(G_X1, i) = x1[i];
    A1(G_DX1, i) = dx1[i];
    A1(G_INVDX1, i) = 1.0 / (dx1[i]);
    A1(G_RINV, i) = 1.0 / x1[i];
    A1(G_ABSX1, i) = 1.0 / std::fabs(x1[i]);
    A1(G_ABSX1P, i) = std::fabs(x1p[i]);
    A1(G_A1F, i) = x1p[i] * x1p[i];
    A1(G_DVR, i) = std::fabs(x1p[i] * x1p[i] * x1p[i] - x1m[i] * x1m[i] * x1m[i]) / 3.0;
    A1(G_INVDVR, i) = 1.0 / A1(G_DVR, i);
    A1(G_RDR, i) = std::fabs(x1[i]) * dx1[i];
    const double rt = (xR * xR * xR - xL * xL * xL) / (xR * xR - xL * xL) / 1.5;
    A1(G_RTINV, i) = 1.0 / rt;
    A1(G_G0, i) = ps::BodyForceVector_r(x1[i], gm_code);
    A1(G_XGC1, i) = x1[i] + 2.0 * x1[i] * dx1[i] * dx1[i] / (12.0 * x1[i] * x1[i] + dx1[i] * dx1[i]);
    A1(G_LOCR, i) = x1[i] * UL;
    if (i >= 1 && i + 1 < n0) {
      A1(G_X11A, i) = (x1[i - 1] + x1[i]) / 2.0 * UL;
      A1(G_X22A, i) = (x1[i + 1] + x1[i]) / 2.0 * UL;
      A1(G_FX, i) = (A1(G_LOCR, i) - A1(G_X11A, i)) / (A1(G_X22A, i) - A1(G_X11A, i));
    }
  }
  for (int j = 0; j < n1; j++) {
    const double xL = x2m[j], xR = x2p[j];
    A2(H_X2, j) = x2[j];
    A2(H_DX2, j) = dx2[j];
    A2(H_INVDX2, j) = 1.0 / (dx2[j]);
    A2(H_DMU, j) = std::fabs(std::cos(xL) - std::cos(xR));
    A2(H_INVDMU, j) = 1.0 / A2(H_DMU, j);
    A2(H_SXP, j) = std::fabs(std::sin(xR));
    A2(H_SPABS, j) = std::fabs(std::fabs(std::sin(xR)));
    A2(H_SN, j) = 1.0 / std::fabs(std::fabs(std::sin(x2[j])));
    A2(H_CT, j) = 1.0 / std::tan(x2[j]);
    A2(H_SIN2, j) = std::sin(x2[j]);
    A2(H_COS2, j) = std::cos(x2[j]);
    double xg = std::sin(xR) - std::sin(xL) + xL * std::cos(xL) - xR * std::cos(xR);
    xg /= std::cos(xL) - std::cos(xR);
    A2(H_XGC2, j) = xg;
    if (j >= 1 && j + 1 < n1) {
      A2(H_X11B, j) = (x2[j - 1] + x2[j]) / 2.0;
      A2(H_X22B, j) = (x2[j + 1] + x2[j]) / 2.0;
      A2(H_FY, j) = (x2[j] - A2(H_X11B, j)) / (A2(H_X22B, j) - A2(H_X11B, j));
    }
  }
  for (int d = 0; d < 2; d++) {
    const int nt = d == 0 ? n0 : n1;
    const double *dx = d == 0 ? dx1 : dx2, *xr = d == 0 ? x1p : x2p;
    for (int i = 1; i <= nt - 2; i++) {
      const double xgm = d == 0 ? A1(G_XGC1, i - 1) : A2(H_XGC2, i - 1);
      const double xg0 = d == 0 ? A1(G_XGC1, i) : A2(H_XGC2, i);
      const double xgp = d == 0 ? A1(G_XGC1, i + 1) : A2(H_XGC2, i + 1);
      double *P = plm.data() + (size_t)d * 6 * nmax;
      P[0 * nmax + i] = (xgp - xg0) / (xr[i] - xg0);       // cp
      P[1 * nmax + i] = (xg0 - xgm) / (xg0 - xr[i - 1]);   // cm
      P[2 * nmax + i] = dx[i] / (xgp - xg0);               // wp
      P[3 * nmax + i] = dx[i] / (xg0 - xgm);               // wm
      P[4 * nmax + i] = (xr[i] - xg0) / dx[i];             // dp
      P[5 * nmax + i] = (xg0 - xr[i - 1]) / dx[i];         // dm
    }
  }

  // per-cell flux-bin lists and the static offsets of VGradCalc
  const int na = wp->line_force ? wp->nangles : 0;
  const size_t ncell = (size_t)n0 * n1;
  std::vector<int> off((size_t)p.nx[0] * p.nx[1] + 1, 0), ang;
  std::vector<double> eFr, eFt, eF1, eF2, eC1a, eC1b, eC2a, eC2b, eIds;
  for (int jj = 0; jj < p.nx[1]; jj++) {
    for (int ii = 0; ii < p.nx[0]; ii++) {
      const int i = ii + p.beg[0], j = jj + p.beg[1];
      const size_t cc = (size_t)j * n0 + i;
      off[(size_t)jj * p.nx[0] + ii] = (int)ang.size();
      for (int a = 0; a < na; a++) {
        const size_t q = (size_t)a * ncell + cc;
        const double fr = flux_r[q], ft = flux_t[q], fp = flux_p[q];
        if (fr == 0.0 && ft == 0.0) continue;  // contributes exactly +0 in LineForce
        double maxds = std::fabs(A1(G_X22A, i) - A1(G_X11A, i));
        if (maxds > (x1[i] * UL * std::fabs(A2(H_X22B, j) - A2(H_X11B, j))))
          maxds = x1[i] * UL * std::fabs(A2(H_X22B, j) - A2(H_X11B, j));
        maxds /= 2.0;
        const double mod_flux = std::sqrt(std::pow(fr, 2) + std::pow(ft, 2) + std::pow(fp, 2));
        double ro = 0.0, to = 0.0, ds = -999;
        if (mod_flux != 0.0) {
          const double x = x1[i] * std::sin(x2[j]) * UL;
          const double z = x1[i] * std::cos(x2[j]) * UL;
          const double th = (a + 0.5) * (2.0 * ps::kPI) / 36.0;
          const double ddx1 = maxds * std::sin(th), ddx2 = maxds * std::cos(th);
          ds = std::sqrt(ddx1 * ddx1 + ddx2 * ddx2);
          ro = std::sqrt((x + ddx1) * (x + ddx1) + (z + ddx2) * (z + ddx2));
          to = std::atan((x + ddx1) / (z + ddx2));
        }
        // VGradCalc's static part (line_connect.c:628-738): the bilinear
        // weights of the offset point and the projections of (v_r, v_theta)
        // at the centre and at the offset point on the bin direction
        const double th = (a + 0.5) * (2.0 * ps::kPI) / 36.0;
        const double sa = std::sin(th), ca = std::cos(th);
        const double st = std::sin(to), ctt = std::cos(to);
        const double s2 = A2(H_SIN2, j), c2 = A2(H_COS2, j);
        ang.push_back(a);
        eFr.push_back(fr);
        eFt.push_back(ft);
        eF1.push_back((ro - A1(G_X11A, i)) / (A1(G_X22A, i) - A1(G_X11A, i)));
        eF2.push_back((to - A2(H_X11B, j)) / (A2(H_X22B, j) - A2(H_X11B, j)));
        eC1a.push_back(UV * (sa * s2 + ca * c2));
        eC1b.push_back(UV * (sa * c2 - ca * s2));
        eC2a.push_back(UV * (sa * st + ca * ctt));
        eC2b.push_back(UV * (sa * ctt - ca * st));
        eIds.push_back(ds == -999 ? 0.0 : 1.0 / ds);
      }
    }
  }
  off[(size_t)p.nx[0] * p.nx[1]] = (int)ang.size();
  const long nent = (long)ang.size();

  WindDev *w = new WindDev();
  cudaError_t e;
  const size_t geo_n = a1.size() + a2.size() + plm.size();
#define WTRY(call)                               \
  do {                                           \
    e = (call);                                  \
    if (e != cudaSuccess) {                      \
      ps_wind_free(w);                           \
      return wind_cuda(e, #call);                \
    }                                            \
  } while (0)
  WTRY(cudaMalloc(&w->geo, geo_n * sizeof(double)));
  WTRY(cudaMemcpy(w->geo, a1.data(), a1.size() * sizeof(double), cudaMemcpyHostToDevice));
  WTRY(cudaMemcpy(w->geo + a1.size(), a2.data(), a2.size() * sizeof(double),
                  cudaMemcpyHostToDevice));
  WTRY(cudaMemcpy(w->geo + a1.size() + a2.size(), plm.data(), plm.size() * sizeof(double),
                  cudaMemcpyHostToDevice));
  WTRY(cudaMalloc(&w->off, off.size() * sizeof(int)));
  WTRY(cudaMemcpy(w->off, off.data(), off.size() * sizeof(int), cudaMemcpyHostToDevice));
  const long ne = nent > 0 ? nent : 1;
  WTRY(cudaMalloc(&w->ent, 9 * ne * sizeof(double)));
  WTRY(cudaMalloc(&w->dvds, ne * sizeof(double)));
  if (nent > 0) {
    const std::vector<double> *cols[9] = {&eFr, &eFt, &eF1, &eF2, &eC1a, &eC1b, &eC2a, &eC2b, &eIds};
    for (int k = 0; k < 9; k++)
      WTRY(cudaMemcpy(w->ent + k * ne, cols[k]->data(), nent * sizeof(double),
                      cudaMemcpyHostToDevice));
  }
  WTRY(cudaMalloc(&w->xi, (size_t)p.vstride * sizeof(double)));
  WTRY(cudaMalloc(&w->tr, (size_t)p.vstride * sizeof(double)));
  WTRY(cudaMemset(w->xi, 0, (size_t)p.vstride * sizeof(double)));
  WTRY(cudaMemset(w->tr, 0, (size_t)p.vstride * sizeof(double)));
  if (ps::needs_shock_flags(p)) {
    WTRY(cudaMalloc(&w->shock, (size_t)p.vstride));
    WTRY(cudaMemset(w->shock, 0, (size_t)p.vstride));
  }
  w->a.shock = w->shock;
  w->nent = nent;

  ps::SphGeom &G = w->a.g;
  const double *g1 = w->geo, *g2 = w->geo + a1.size(), *gp = w->geo + a1.size() + a2.size();
  G.x1 = g1 + (size_t)G_X1 * n0;
  G.dx1 = g1 + (size_t)G_DX1 * n0;
  G.inv_dx1 = g1 + (size_t)G_INVDX1 * n0;
  G.rinv = g1 + (size_t)G_RINV * n0;
  G.inv_absx1 = g1 + (size_t)G_ABSX1 * n0;
  G.inv_dVr = g1 + (size_t)G_INVDVR * n0;
  G.absx1p = g1 + (size_t)G_ABSX1P * n0;
  G.A1f = g1 + (size_t)G_A1F * n0;
  G.dVr = g1 + (size_t)G_DVR * n0;
  G.rdr = g1 + (size_t)G_RDR * n0;
  G.rtinv = g1 + (size_t)G_RTINV * n0;
  G.g0 = g1 + (size_t)G_G0 * n0;
  G.fx = g1 + (size_t)G_FX * n0;
  G.x2 = g2 + (size_t)H_X2 * n1;
  G.dx2 = g2 + (size_t)H_DX2 * n1;
  G.inv_dx2 = g2 + (size_t)H_INVDX2 * n1;
  G.dmu = g2 + (size_t)H_DMU * n1;
  G.sxp = g2 + (size_t)H_SXP * n1;
  G.spabs = g2 + (size_t)H_SPABS * n1;
  G.inv_sn = g2 + (size_t)H_SN * n1;
  G.inv_dmu = g2 + (size_t)H_INVDMU * n1;
  G.ct = g2 + (size_t)H_CT * n1;
  G.sin2 = g2 + (size_t)H_SIN2 * n1;
  G.cos2 = g2 + (size_t)H_COS2 * n1;
  G.fy = g2 + (size_t)H_FY * n1;
  for (int d = 0; d < 2; d++) {
    const double *P = gp + (size_t)d * 6 * nmax;
    G.cp[d] = P + 0 * nmax;
    G.cm[d] = P + 1 * nmax;
    G.wp[d] = P + 2 * nmax;
    G.wm[d] = P + 3 * nmax;
    G.dp[d] = P + 4 * nmax;
    G.dm[d] = P + 5 * nmax;
  }
  ps::LineList &L = w->a.L;
  L.off = w->off;
  L.Fr = w->ent + 0 * ne;
  L.Ft = w->ent + 1 * ne;
  L.fr1 = w->ent + 2 * ne;
  L.fr2 = w->ent + 3 * ne;
  L.c1a = w->ent + 4 * ne;
  L.c1b = w->ent + 5 * ne;
  L.c2a = w->ent + 6 * ne;
  L.c2b = w->ent + 7 * ne;
  L.inv_ds = w->ent + 8 * ne;
  L.lq = w->dvds;

  ps::WindParams &W = w->a.w;
  std::memset(&W, 0, sizeof(W));
  W.body_force = wp->body_force;
  W.line_force = wp->line_force;
  W.floors = wp->floors;
  W.cooling = c->cfg.cooling;
  W.unit_density = UD;
  W.unit_length = UL;
  W.unit_velocity = UV;
  W.mu = wp->mu;
  W.kelvin = UV * UV * ps::kAmu / ps::kKB;
  W.dfloor = wp->dfloor / UD;
  W.tfloor = 5.e2;
  W.pfloor = W.dfloor * W.tfloor / (W.kelvin * W.mu);
  W.inv_dfloor = 1.0 / W.dfloor;
  W.kmu = W.kelvin * W.mu;
  W.krad = wp->krad;
  W.alpharad = wp->alpharad;
  W.sigma_e = ps::kSigmaT / ps::kAmu / 1.18;
  W.unit_acc = UV * UV / UL;
  W.lx = wp->l_star * wp->frac_x;
  W.t_x = wp->t_x;
  W.unit_pressure = UD * UV * UV;
  W.unit_time = UL / UV;
  ps::set_sg_units(W, c->cfg.gamma);
  {
    // t = sigma_e rho_cgs v_th / (dv/ds), v_th = sqrt(2 kB T / m_p),
    // T = p / rho KELVIN mu  =>  t = C sqrt(rho p) / (dv/ds) in code units
    const double C = W.sigma_e * UD * std::sqrt(W.kelvin * W.mu * 2.0 * ps::kKB / ps::kMP);
    W.lf_a0 = std::log(W.krad) + W.alpharad * std::log(C);
    W.lf_cf = W.sigma_e / ps::kC / W.unit_acc;
    // KRAD = ALPHARAD = 999 selects the tabulated force multiplier
    // (line_connect.c:183, 858, 884); the table comes with ps_set_mfit
    W.mfit = (W.krad == 999 && W.alpharad == 999) ? 1 : 0;
    W.nm = 0;
    W.lt0 = std::log10(C);
  }
  {
    // the ODE cooling path: E_cost of Radiat and KELVIN times
    // MeanMolecularWeight with COOLING TABULATED and the default mass
    // fractions (Src/mean_mol_weight.c:138-141, Src/pluto.h:692-720)
    W.ode_e_cost = UL / UD / std::pow(UV, 3.0);
    const double AH = 1.008, AHe = 4.004, AZ = 30.0, xH = 0.7110, xHe = 0.2741;
    const double xZ = (1.0 - xH - xHe);
    const double fHe = (xHe / AHe * AH / xH), fZ = (xZ / AZ * AH / xH);
    const double mu0 = (AH + fHe * AHe + fZ * AZ) / (2.0 + 3.0 * fHe + fZ * (1.0 + AZ * 0.5));
    W.ode_mu0_kelvin = W.kelvin * mu0;
  }

  w->k1 = ps::stage_kernel_sph(p.nvar, p.char_lim != 0, p.limiter, p.solver, 1);
  w->k2 = ps::stage_kernel_sph(p.nvar, p.char_lim != 0, p.limiter, p.solver, 2);
  w->smem = p.nvar == 7 ? ps::stage_smem_bytes<7, ps::WindTile>()
                        : ps::stage_smem_bytes<6, ps::WindTile>();
  if (!w->k1 || !w->k2) {
    ps_wind_free(w);
    return wind_fail("ps_set_wind: no kernel for this configuration");
  }
  WTRY(cudaFuncSetAttribute(w->k1, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)w->smem));
  WTRY(cudaFuncSetAttribute(w->k2, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)w->smem));
#undef WTRY
  if (c->wind) ps_wind_free(c->wind);
  c->wind = w;
  for (int k = 0; k < 3; k++) {
    if (c->gw[k]) cudaGraphExecDestroy(c->gw[k]);
    c->gw[k] = nullptr;
  }
  // sirocco_xi / sirocco_t_r from the current state (read_sirocco_heatcool, flag 0)
  ps::k_wind_init_xi<<<256, 256, 0, c->stream>>>(c->V, w->xi, w->tr, p, W, G.x1);
  c->launches++;
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return wind_cuda(e, "ps_set_wind: xi");
  return 0;
}

// Boundary() before stage `stage` of the wind (floors, x1 then x2 ghosts);
// before stage 1 with SHOCK_FLATTENING MULTID also FlagShock.
int ps_wind_bnd_launch(ps_ctx *c, int stage)
{
  WindDev *w = c->wind;
  const ps::Params &p = c->p;
  const int nb = (p.nx[0] * p.nx[1] + 255) / 256;
  const int nb2 = (p.ntot[0] * 2 * p.beg[1] + 255) / 256;
  double *Vin = stage == 1 ? c->V : c->Vs;
  if (p.nvar == 7) {
    ps::k_wind_bnd_x1<7><<<nb, 64, 0, c->stream>>>(Vin, c->Us, p, w->a.w, c->sc, stage);
    ps::k_wind_bnd_x2<7><<<nb2, 256, 0, c->stream>>>(Vin, p, c->sc);
  } else {
    ps::k_wind_bnd_x1<6><<<nb, 64, 0, c->stream>>>(Vin, c->Us, p, w->a.w, c->sc, stage);
    ps::k_wind_bnd_x2<6><<<nb2, 256, 0, c->stream>>>(Vin, p, c->sc);
  }
  c->launches += 2;
  if (stage == 1 && ps::needs_shock_flags(p)) {
    const int nb3 = (p.ntot[0] * p.ntot[1] + 255) / 256;
    ps::k_wind_shock<<<nb3, 256, 0, c->stream>>>(w->shock, c->V, p, w->a.g, c->sc);
    c->launches++;
  }
  return 0;
}

// Stage kernel `stage` of the wind.
int ps_wind_stage_launch(ps_ctx *c, int stage)
{
  WindDev *w = c->wind;
  ps::WindStageArgs A = w->a;
  A.s.Vn = c->V;
  A.s.Vout = stage == 1 ? c->Vs : c->V;
  A.s.Us = c->Us;
  for (int d = 0; d < 3; d++) {
    A.s.dtdx[d] = c->dtdx[d];
    A.s.inv_dx[d] = c->inv_dx[d];
  }
  A.s.sc = c->sc;
  A.s.p = c->p;
  void *args[2] = {stage == 1 ? &c->tmV : &c->tmVs, &A};
  cudaError_t e = cudaLaunchKernel(stage == 1 ? w->k1 : w->k2, c->grid, c->block, args, w->smem,
                                   c->stream);
  c->launches++;
  if (e != cudaSuccess) return wind_cuda(e, "wind stage launch");
  return 0;
}

// The hydro part of one wind step (AdvanceStep).
int ps_wind_hydro_launches(ps_ctx *c)
{
  for (int stage = 1; stage <= 2; stage++) {
    int r = ps_wind_bnd_launch(c, stage);
    if (!r) r = ps_wind_stage_launch(c, stage);
    if (r) return r;
  }
  return 0;
}

// SplitSource with BLONDIN (Src/split_source.c:52-53) for the device dt/time.
int ps_sg_cool_launch(ps_ctx *c);

int ps_wind_cool_launch(ps_ctx *c)
{
  WindDev *w = c->wind;
  const ps::Params &p = c->p;
  if (!p.cooling) return 0;
  if (p.cooling == 2) {   // the ODE path
    const int nb = (p.nx[0] * p.nx[1] + 127) / 128;
    ps::k_ode_cool<<<nb, 128, 0, c->stream>>>(c->V, w->xi, w->tr, p, w->a.w, w->a.g.x1, c->sc,
                                              w->pre);
    c->launches++;
    return 0;
  }
  if (c->sg) return ps_sg_cool_launch(c);
  const int nb = (p.nx[0] * p.nx[1] + 127) / 128;
  ps::k_blondin<<<nb, 128, 0, c->stream>>>(c->V, w->xi, w->tr, p, w->a.w, w->a.g.x1, c->sc,
                                           w->pre);
  c->launches++;
  return 0;
}

// One step of the wind: the split source before (odd steps) or after
// (even steps) the hydro (Src/main.c:479-485), then the dt kernel.
int ps_wind_step_launches(ps_ctx *c, int odd, int (*finish)(ps_ctx *, int))
{
  int r = 0;
  if (odd) r = ps_wind_cool_launch(c);
  if (!r) r = ps_wind_hydro_launches(c);
  if (!r && !odd) r = ps_wind_cool_launch(c);
  if (!r) r = finish(c, 1);
  return r;
}

// read_sirocco_heatcool with flag 1 (Src/LineDriven/line_connect.c:267-497):
// per-cell xi and radiation temperature (used by BLONDIN once g_time > 3)
// and the prefactors of the five rates.  Arrays are [j][i] over the total
// box (the prefactors: six such arrays in the file's order comp_h, comp_c,
// xray_h, brem_c, line_c, xi_ion; xi_ion is not used by BLONDIN).  A NULL
// argument leaves that part as it is; ps_set_wind starts from xi and T_x
// of the initial state and prefactors 1.
void ps_ctx_invalidate_graphs(ps_ctx *c);

extern "C" int ps_set_sirocco(ps_ctx *c, const double *xi, const double *t_r, const double *pre)
{
  if (!c || !c->wind) return wind_fail("ps_set_sirocco: needs ps_set_wind first");
  WindDev *w = c->wind;
  const ps::Params &p = c->p;
  const int n0 = p.ntot[0], n1 = p.ntot[1];
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return wind_cuda(e, "ps_set_sirocco");
  auto upload = [&](const double *src, double *dst) -> cudaError_t {
    // host [j][i] rows of n0 -> device rows of px
    return cudaMemcpy2D(dst + p.xoff, (size_t)p.px * sizeof(double), src,
                        (size_t)n0 * sizeof(double),
                        (size_t)n0 * sizeof(double), (size_t)n1, cudaMemcpyHostToDevice);
  };
  if (xi && (e = upload(xi, w->xi)) != cudaSuccess) return wind_cuda(e, "ps_set_sirocco: xi");
  if (t_r && (e = upload(t_r, w->tr)) != cudaSuccess) return wind_cuda(e, "ps_set_sirocco: t_r");
  if (pre) {
    if (!w->pre) {
      if ((e = cudaMalloc(&w->pre, 5 * (size_t)p.vstride * sizeof(double))) != cudaSuccess)
        return wind_cuda(e, "ps_set_sirocco: prefactors");
      cudaMemset(w->pre, 0, 5 * (size_t)p.vstride * sizeof(double));
    }
    const size_t plane = (size_t)n0 * n1;
    // file order comp_h, comp_c, xray_h, brem_c, line_c -> device order ch, cc, xh, lc, bc
    const int src_of[5] = {0, 1, 2, 4, 3};
    for (int k = 0; k < 5; k++)
      if ((e = upload(pre + src_of[k] * plane, w->pre + (size_t)k * p.vstride)) != cudaSuccess)
        return wind_cuda(e, "ps_set_sirocco: prefactors");
  }
  ps_ctx_invalidate_graphs(c);
  return 0;
}

// The tabulated force multiplier of KRAD = ALPHARAD = 999 runs
// (read_sirocco_fluxes, line_connect.c:182-257): t at npoints and every
// cell's M, [point][j][i] over the total box, as M_UV_data.dat holds them;
// the log10 of each is kept, as the reader does.
extern "C" int ps_set_mfit(ps_ctx *c, int npoints, const double *t_fit, const double *m_fit)
{
  if (!c || !c->wind) return wind_fail("ps_set_mfit: needs ps_set_wind first");
  WindDev *w = c->wind;
  if (!w->a.w.mfit) return wind_fail("ps_set_mfit: the wind's KRAD and ALPHARAD are not 999");
  if (npoints < 1 || npoints > 4096 || !t_fit || !m_fit)
    return wind_fail("ps_set_mfit: bad arguments");
  const ps::Params &p = c->p;
  const int n0 = p.ntot[0], n1 = p.ntot[1];
  const size_t plane = (size_t)n0 * n1;
  std::vector<double> lt(npoints), lm((size_t)npoints * plane);
  for (int k = 0; k < npoints; k++) lt[k] = std::log10(t_fit[k]);
  for (size_t q = 0; q < lm.size(); q++) lm[q] = std::log10(m_fit[q]);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return wind_cuda(e, "ps_set_mfit");
  cudaFree(w->t_fit);
  cudaFree(w->m_fit);
  w->t_fit = w->m_fit = nullptr;
  if ((e = cudaMalloc(&w->t_fit, npoints * sizeof(double))) != cudaSuccess ||
      (e = cudaMalloc(&w->m_fit, (size_t)npoints * p.vstride * sizeof(double))) != cudaSuccess)
    return wind_cuda(e, "ps_set_mfit: allocation");
  if ((e = cudaMemcpy(w->t_fit, lt.data(), npoints * sizeof(double), cudaMemcpyHostToDevice)) !=
      cudaSuccess)
    return wind_cuda(e, "ps_set_mfit: t");
  for (int k = 0; k < npoints; k++)
    if ((e = cudaMemcpy2D(w->m_fit + (size_t)k * p.vstride + p.xoff, (size_t)p.px * sizeof(double),
                          lm.data() + (size_t)k * plane, (size_t)n0 * sizeof(double),
                          (size_t)n0 * sizeof(double), (size_t)n1, cudaMemcpyHostToDevice)) !=
        cudaSuccess)
      return wind_cuda(e, "ps_set_mfit: M");
  w->a.L.t_fit = w->t_fit;
  w->a.L.m_fit = w->m_fit;
  w->a.w.nm = npoints;
  ps_ctx_invalidate_graphs(c);
  return 0;
}

// A wind whose KRAD and ALPHARAD ask for the table cannot step without it.
int ps_wind_check(const ps_ctx *c, const char *who)
{
  if (c->wind && c->wind->a.w.mfit && c->wind->a.w.nm == 0) {
    char buf[160];
    std::snprintf(buf, sizeof(buf), "%s: KRAD = ALPHARAD = 999 needs ps_set_mfit", who);
    ps_set_error_msg(buf);
    return PS_ESTATE;
  }
  return 0;
}
