// ps_stage.cuh -- one RK stage of the unsplit HD update, fused into a single
// kernel per stage: TMA load of a haloed tile of the primitive state, PLM
// reconstruction, Riemann solve and flux difference for every active
// direction, conservative update, conversion back to primitives, ghost-zone
// fill for the next stage, and (stage 1) the per-cell inverse time step
// with its block/grid maximum.
//
// Reference (paths inside the reference project):
//   UpdateStage        Src/Time_Stepping/update_stage.c:35-410
//   States (PLM)       Src/States/plm_states.c:83-338
//   RightHandSide      Src/MHD/rhs.c:188-209 (Cartesian branch)
//   AdvanceStep (RK2)  Src/Time_Stepping/rk_step.c:114-261
//   Boundary           Src/boundary.c:56-760 (outflow/periodic/reflective)
#pragma once

#include "ps_hydro.cuh"
#include "ps_physics.cuh"
#include "ps_tma.cuh"

namespace ps {

constexpr int BC_OUTFLOW = 1, BC_REFLECTIVE = 2, BC_AXISYM = 3, BC_EQTSYM = 4,
              BC_PERIODIC = 5;

// Tile of active cells processed by one CTA (one thread per cell) and the
// ghost width loaded around it.
template <int DIMS> struct TileT;
template <> struct TileT<2> {
  static constexpr int X = 32, Y = 8, Z = 1, HX = 2, HY = 2, HZ = 0;
};
template <> struct TileT<3> {
  static constexpr int X = 16, Y = 4, Z = 4, HX = 2, HY = 2, HZ = 2;
};
// 2-D tiles of other shapes (chosen per grid size by the batch autotuner);
// XT extra threads (whole warps) share the halo work of the PLM and
// Riemann phases, which have more items than the tile has cells; they own
// no cell.
// MB: the CTAs per multiprocessor the kernel is compiled for (its
// register budget, __launch_bounds__'s second argument).
template <int TX, int TY, int XT = 0, int MB = 1> struct Tile2D {
  static constexpr int X = TX, Y = TY, Z = 1, HX = 2, HY = 2, HZ = 0, EXTRA = XT, MINB = MB;
};

template <class TL, class = void> struct TileExtra {
  static constexpr int value = 0;
};
template <class TL> struct TileExtra<TL, decltype((void)TL::EXTRA)> {
  static constexpr int value = TL::EXTRA;
};
template <class TL, class = void> struct TileMinBlocks {
  static constexpr int value = 1;
};
template <class TL> struct TileMinBlocks<TL, decltype((void)TL::MINB)> {
  static constexpr int value = TL::MINB;
};

template <class TL> struct TileGeom {
  static constexpr int SX = TL::X + 2 * TL::HX, SY = TL::Y + 2 * TL::HY, SZ = TL::Z + 2 * TL::HZ;
  static constexpr int VS = SX * SY * SZ;            // cells in the haloed tile
  static constexpr int NC = TL::X * TL::Y * TL::Z;   // cells of the tile (owning threads)
  static constexpr int NT = NC + TileExtra<TL>::value;  // threads per CTA
  __host__ __device__ static constexpr int t(int d)
  {
    return d == 0 ? TL::X : (d == 1 ? TL::Y : TL::Z);
  }
  __host__ __device__ static constexpr int ext(int d, int D, int add)
  {
    return t(d) + (d == D ? add : 0);
  }
  __host__ __device__ static constexpr int np(int D)
  {
    return ext(0, D, 2) * ext(1, D, 2) * ext(2, D, 2);
  }
  __host__ __device__ static constexpr int nf(int D)
  {
    return ext(0, D, 1) * ext(1, D, 1) * ext(2, D, 1);
  }
  __host__ __device__ static constexpr int mx(int a, int b) { return a > b ? a : b; }
  static constexpr int NPMAX = mx(mx(np(0), np(1)), TL::Z > 1 ? np(2) : 0);
  static constexpr int NFMAX = mx(mx(nf(0), nf(1)), TL::Z > 1 ? nf(2) : 0);
};

template <int NV, class TL>
constexpr size_t stage_smem_bytes()
{
  using G = TileGeom<TL>;
  return sizeof(double) * (size_t)(NV * G::VS + 2 * NV * G::NPMAX + NV * G::NFMAX + 2 * G::NFMAX
                                   + 2 + G::NT / 32);
}

// Write one cell of a primitive array and every ghost cell that the
// standard boundary conditions fill from it (Src/boundary.c:617-760).
template <int DIMS, int NV>
__device__ __forceinline__ void store_with_ghosts(double *__restrict__ V, const Params &p,
                                                  int gi, int gj, int gk, const double (&v)[NV])
{
  const long long row = (long long)p.ntot[1] * p.px;
  const long long base = (long long)gk * row + (long long)gj * p.px + gi;
#pragma unroll
  for (int nv = 0; nv < NV; nv++) V[nv * p.vstride + base] = v[nv];
  const int g[3] = {gi, gj, gk};
  const long long st[3] = {1, (long long)p.px, row};
#pragma unroll
  for (int d = 0; d < DIMS; d++) {
    const int c = g[d], b = p.beg[d], n = p.nx[d], e = b + n - 1;
#pragma unroll
    for (int side = 0; side < 2; side++) {
      const int type = p.bc[2 * d + side];
      int t0 = -1, t1 = -1;
      bool flip = false;
      if (type == BC_OUTFLOW) {
        if (side == 0 && c == b) { t0 = b - 1; t1 = b - 2; }
        if (side == 1 && c == e) { t0 = e + 1; t1 = e + 2; }
      } else if (type == BC_PERIODIC) {
        if (side == 0 && c >= e - 1) t0 = c - n;
        if (side == 1 && c <= b + 1) t0 = c + n;
      } else if (type == BC_REFLECTIVE || type == BC_AXISYM || type == BC_EQTSYM) {
        flip = true;
        if (side == 0 && c <= b + 1) t0 = 2 * b - 1 - c;
        if (side == 1 && c >= e - 1) t0 = 2 * e + 1 - c;
      }
#pragma unroll
      for (int w = 0; w < 2; w++) {
        const int t = w == 0 ? t0 : t1;
        if (t < 0) continue;
        const long long q = base + (long long)(t - c) * st[d];
#pragma unroll
        for (int nv = 0; nv < NV; nv++) {
          const bool neg = flip && (nv == VX1 + d);
          V[nv * p.vstride + q] = neg ? -1 * v[nv] : v[nv];
        }
      }
    }
  }
}

// Ghost zones of a state that did not come from a stage kernel (a state
// copied in from the host): the boundary cells rewrite their ghosts, as
// Boundary() does before the first stage.
template <int DIMS, int NV>
__global__ void k_fill_ghosts(double *V, const Params p)
{
  const long long n = (long long)p.nx[0] * p.nx[1] * p.nx[2];
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(q % p.nx[0]), j = (int)((q / p.nx[0]) % p.nx[1]),
              k = (int)(q / ((long long)p.nx[0] * p.nx[1]));
    const bool edge = (i < 2 || i >= p.nx[0] - 2) || (j < 2 || j >= p.nx[1] - 2) ||
                      (DIMS == 3 && (k < 2 || k >= p.nx[2] - 2));
    if (!edge) continue;
    const int gi = i + p.beg[0], gj = j + p.beg[1], gk = k + p.beg[2];
    const long long cell = ((long long)gk * p.ntot[1] + gj) * p.px + gi;
    double v[NV];
#pragma unroll
    for (int nv = 0; nv < NV; nv++) v[nv] = V[nv * p.vstride + cell];
    store_with_ghosts<DIMS, NV>(V, p, gi, gj, gk, v);
  }
}

// The Cartesian stage kernels whose products no add absorbs run on the
// integer pipes (ps_dmul.cuh, the same bits as the FP64 unit's): the
// 5-variable set of the blast and the cooling cube.
template <int NV>
constexpr bool kIntProductsCart = NV == NFLX;

// PLM of one cell along one direction on the uniform grid: + and - states
// of all variables (limited_slope_t<LIM, INT>; a cell whose operands leave
// the integer forms' range is done again with INT = false, the same bits)
template <int NV, int LIM, bool INT, class G>
__device__ __forceinline__ void plm_cart_cell(const double *__restrict__ sv,
                                              double *__restrict__ svp,
                                              double *__restrict__ svm, int s0, int sst, int q,
                                              bool &bad)
{
#pragma unroll
  for (int nv = 0; nv < NV; nv++) {
    const double vm1 = sv[nv * G::VS + s0 - sst], v0 = sv[nv * G::VS + s0],
                 vp1 = sv[nv * G::VS + s0 + sst];
    const double dvp = vp1 - v0, dvm = v0 - vm1;
    const double dv = limited_slope_t<LIM, INT>(dvp, dvm, bad);
    svp[nv * G::NPMAX + q] = v0 + dv * 0.5;
    svm[nv * G::NPMAX + q] = v0 - dv * 0.5;
  }
}

// The end of a stage for one own cell: with STAGE 2 the RK2 average
// U = U0 / 2 + U / 2 with U0 from V^n (halvings are exact, so this is the
// reference's 0.5 U0 + 0.5 U); then ConsToPrim.  U holds the stage's
// conserved state on entry and the (repaired) state on return.  Products
// by dmul_t<INT> (ps_dmul.cuh).
template <int NV, int STAGE, bool INT>
__device__ __forceinline__ unsigned stage_out(double (&U)[NV], double (&v)[NV],
                                              const StageArgs &a, const Params &p,
                                              long long cell, int ent, bool &bad)
{
  if constexpr (STAGE == 2) {
    double v0[NV], U0[NV];
#pragma unroll
    for (int nv = 0; nv < NV; nv++) v0[nv] = a.Vn[nv * p.vstride + cell];
    prim_to_cons_t<NV, INT>(v0, U0, p.igmm1, bad);
#pragma unroll
    for (int nv = 0; nv < NV; nv++) U[nv] = dhalf_t<INT>(U0[nv], bad) + dhalf_t<INT>(U[nv], bad);
  }
  return cons_to_prim_t<NV, INT>(U, v, p.gmm1, ent, bad);
}

// One direction of the unsplit update on the tile held in shared memory.
template <int D, int NV, int LIM, int SOLVER, class TL>
__device__ __forceinline__ void sweep(const double *__restrict__ sv, double *__restrict__ svp,
                                      double *__restrict__ svm, double *__restrict__ sf,
                                      double *__restrict__ spr, double *__restrict__ scm,
                                      double (&U)[NV], double &cdt, bool own, int cx, int cy,
                                      int cz, int gcell, const StageArgs &a, bool stage1)
{
  using G = TileGeom<TL>;
  constexpr int PX = G::ext(0, D, 2), PY = G::ext(1, D, 2), PZ = G::ext(2, D, 2);
  constexpr int FX = G::ext(0, D, 1), FY = G::ext(1, D, 1), FZ = G::ext(2, D, 1);
  constexpr int NP = PX * PY * PZ, NF = FX * FY * FZ;
  constexpr int SST = D == 0 ? 1 : (D == 1 ? G::SX : G::SX * G::SY);  // smem stride along D
  constexpr int VN = VX1 + D;
  constexpr bool IP = kIntProductsCart<NV>;
  const double gam = a.p.gamma;

  // (1) PLM: + and - states of cells -1 .. T_D along D
  for (int q = threadIdx.x; q < NP; q += G::NT) {
    const int ix = q % PX, iy = (q / PX) % PY, iz = q / (PX * PY);
    const int sx = ix + TL::HX - (D == 0), sy = iy + TL::HY - (D == 1),
              sz = iz + TL::HZ - (D == 2);
    const int s0 = (sz * G::SY + sy) * G::SX + sx;
    bool bad = false;
    plm_cart_cell<NV, LIM, IP, G>(sv, svp, svm, s0, SST, q, bad);
    if (IP && bad) plm_cart_cell<NV, LIM, false, G>(sv, svp, svm, s0, SST, q, bad);
  }
  __syncthreads();

  // (2) Riemann problem at faces 0 .. T_D along D (face f sits between
  //     cells f-1 and f; its left state is the + state of PLM entry f,
  //     its right state the - state of PLM entry f+1)
  for (int q = threadIdx.x; q < NF; q += G::NT) {
    const int fx = q % FX, fy = (q / FX) % FY, fz = q / (FX * FY);
    const int pl = (fz * PY + fy) * PX + fx;
    constexpr int PST = D == 0 ? 1 : (D == 1 ? PX : PX * PY);
    const int pr_ = pl + PST;
    double vL[NV], vR[NV], f[NV], pr, cm;
#pragma unroll
    for (int nv = 0; nv < NV; nv++) {
      vL[nv] = svp[nv * G::NPMAX + pl];
      vR[nv] = svm[nv * G::NPMAX + pr_];
    }
    bool bad = false;
    riemann_t<NV, SOLVER, VN, IP>(vL, vR, gam, a.p.igmm1, f, pr, cm, false, bad);
    if constexpr (IP) {
      if (bad) riemann_t<NV, SOLVER, VN, false>(vL, vR, gam, a.p.igmm1, f, pr, cm, false, bad);
    }
#pragma unroll
    for (int nv = 0; nv < NV; nv++) sf[nv * G::NFMAX + q] = f[nv];
    spr[q] = pr;
    scm[q] = cm;
  }
  __syncthreads();

  // (3) flux difference and update of the owned cell
  if (own) {
    const int ql = (cz * FY + cy) * FX + cx;
    constexpr int FST = D == 0 ? 1 : (D == 1 ? FX : FX * FY);
    const int qr = ql + FST;
    const double scrh = a.dtdx[D][gcell];
    double rhs[NV];
    bool bad = !IP;
    if constexpr (IP) {
#pragma unroll
      for (int nv = 0; nv < NV; nv++)
        rhs[nv] = -dmul_int(scrh, sf[nv * G::NFMAX + qr] - sf[nv * G::NFMAX + ql], bad);
    }
    if (bad) {
#pragma unroll
      for (int nv = 0; nv < NV; nv++)
        rhs[nv] = -__dmul_rn(scrh, sf[nv * G::NFMAX + qr] - sf[nv * G::NFMAX + ql]);
    }
    rhs[VN] = fma(-scrh, spr[qr] - spr[ql], rhs[VN]);
#pragma unroll
    for (int nv = 0; nv < NV; nv++) U[nv] += rhs[nv];
    if (stage1) {
      bool badc = !IP;
      double h = 0.0;
      if constexpr (IP) h = dhalf_int(scm[ql] + scm[qr], badc);
      if (badc) h = 0.5 * (scm[ql] + scm[qr]);
      cdt = fma(h, a.inv_dx[D][gcell], cdt);
    }
  }
  __syncthreads();
}

template <int DIMS, int NV, int LIM, int SOLVER, int STAGE>
__global__ void __launch_bounds__(TileGeom<TileT<DIMS>>::NT)
    k_stage(const __grid_constant__ CUtensorMap tm, const StageArgs a)
{
  using TL = TileT<DIMS>;
  using G = TileGeom<TL>;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  double *sv = reinterpret_cast<double *>(smem_raw);
  double *svp = sv + NV * G::VS;
  double *svm = svp + NV * G::NPMAX;
  double *sf = svm + NV * G::NPMAX;
  double *spr = sf + NV * G::NFMAX;
  double *scm = spr + G::NFMAX;
  uint64_t *bar = reinterpret_cast<uint64_t *>(scm + G::NFMAX);
  unsigned &s_flags = *reinterpret_cast<unsigned *>(bar + 1);
  unsigned long long *s_red = reinterpret_cast<unsigned long long *>(bar + 2);

  if (a.sc->done) return;

  const Params &p = a.p;
  const int tid = threadIdx.x;
  const int ox = blockIdx.x * TL::X, oy = blockIdx.y * TL::Y, oz = blockIdx.z * TL::Z;

  if (tid == 0) {
    s_flags = 0;
    mbar_init(bar, 1);
  }
  __syncthreads();
  if (tid == 0) {
    mbar_expect_tx(bar, (uint32_t)(NV * G::VS * sizeof(double)));
    tma_load_4d(sv, &tm, ox + p.beg[0] - TL::HX, oy + p.beg[1] - TL::HY,
                DIMS == 3 ? oz + p.beg[2] - TL::HZ : 0, 0, bar);
  }
  const bool landed = mbar_wait_bounded(bar, 0, 1u << 22);
  if (!__syncthreads_and(landed)) {
    // block-uniform exit; thread 0 gives the copy a last bounded chance to
    // land before the CTA's shared memory is released
    if (tid == 0) {
      atomicOr(&a.sc->flags, F_TMA_TIMEOUT);
      mbar_wait_bounded(bar, 0, 1u << 22);
    }
    return;
  }

  const int cx = tid % TL::X, cy = (tid / TL::X) % TL::Y, cz = tid / (TL::X * TL::Y);
  const bool own = tid < G::NC && (ox + cx < p.nx[0]) && (oy + cy < p.nx[1]) && (oz + cz < p.nx[2]);
  const int gi = p.beg[0] + ox + cx, gj = p.beg[1] + oy + cy, gk = p.beg[2] + oz + cz;
  const long long cell = ((long long)gk * p.ntot[1] + gj) * p.px + gi;

  constexpr bool IP = kIntProductsCart<NV>;
  double U[NV];
  double cdt = 0.0;
  if (own) {
    if constexpr (STAGE == 1) {
      double v[NV];
      const int s0 = ((cz + TL::HZ) * G::SY + cy + TL::HY) * G::SX + cx + TL::HX;
#pragma unroll
      for (int nv = 0; nv < NV; nv++) v[nv] = sv[nv * G::VS + s0];
      bool bad = false;
      prim_to_cons_t<NV, IP>(v, U, p.igmm1, bad);
      if (IP && bad) prim_to_cons_t<NV, false>(v, U, p.igmm1, bad);
    } else {
#pragma unroll
      for (int nv = 0; nv < NV; nv++) U[nv] = a.Us[nv * p.vstride + cell];
    }
  }

  sweep<0, NV, LIM, SOLVER, TL>(sv, svp, svm, sf, spr, scm, U, cdt, own, cx, cy, cz, gi, a,
                                STAGE == 1);
  sweep<1, NV, LIM, SOLVER, TL>(sv, svp, svm, sf, spr, scm, U, cdt, own, cx, cy, cz, gj, a,
                                STAGE == 1);
  if constexpr (DIMS == 3)
    sweep<2, NV, LIM, SOLVER, TL>(sv, svp, svm, sf, spr, scm, U, cdt, own, cx, cy, cz, gk, a,
                                  STAGE == 1);

  unsigned flags = 0;
  if (own) {
    // U^{n+1} = 1/2 U0 + 1/2 (U* + dt L(V*)), U0 = PrimToCons(V^n), then
    // the primitive state (the integer form first, again on the FP64 unit
    // if it hands back)
    double v[NV], Uw[NV];
    bool bad = false;
#pragma unroll
    for (int nv = 0; nv < NV; nv++) Uw[nv] = U[nv];
    unsigned f = stage_out<NV, STAGE, IP>(Uw, v, a, p, cell, 0, bad);
    if (IP && bad) {
#pragma unroll
      for (int nv = 0; nv < NV; nv++) Uw[nv] = U[nv];
      f = stage_out<NV, STAGE, false>(Uw, v, a, p, cell, 0, bad);
    }
#pragma unroll
    for (int nv = 0; nv < NV; nv++) U[nv] = Uw[nv];
    flags |= f;
#pragma unroll
    for (int nv = 0; nv < NV; nv++)
      if (is_nan_bits(v[nv])) flags |= F_NAN;
    if constexpr (STAGE == 1) {
#pragma unroll
      for (int nv = 0; nv < NV; nv++) a.Us[nv * p.vstride + cell] = U[nv];
    }
    store_with_ghosts<DIMS, NV>(a.Vout, p, gi, gj, gk, v);
  }
  if (flags) atomicOr(&s_flags, flags);

  if constexpr (STAGE == 1) {
    unsigned long long b = (unsigned long long)__double_as_longlong(cdt);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      unsigned long long ob = __shfl_xor_sync(0xffffffffu, b, o);
      b = ob > b ? ob : b;
    }
    if ((tid & 31) == 0) s_red[tid >> 5] = b;
  }
  __syncthreads();
  if (tid == 0) {
    if constexpr (STAGE == 1) {
      unsigned long long b = 0;
#pragma unroll
      for (int w = 0; w < G::NT / 32; w++) b = s_red[w] > b ? s_red[w] : b;
      atomicMax(&a.sc->cdt_bits, b);
    }
    if (s_flags) atomicOr(&a.sc->flags, s_flags);
  }
}

}  // namespace ps
