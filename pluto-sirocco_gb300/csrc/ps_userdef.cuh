// ps_userdef.cuh -- the line-driven wind problem's user hooks on the device,
// named after the functions of the problem's init.c that PLUTO calls every
// stage (Boundary(), Src/boundary.c:126-128 and its per-side loop;
// RightHandSideSource, Src/MHD/rhs_source.c:253-274):
//
//   UserDefBoundary(d, NULL, 0, grid)   -> UserDefBoundary_Internal
//   UserDefBoundary(d, box, X1_BEG, g)  -> UserDefBoundary_X1Beg
//   UserDefBoundary(d, box, X1_END, g)  -> UserDefBoundary_X1End
//   UserDefBoundary(d, box, X2_BEG, g)  -> UserDefBoundary_X2Beg
//   BodyForceVector(v, g, x1, x2, x3)   -> BodyForceVector_r
//
// with the semantics of the production disk-wind problem
// (Test_Problems/LineDrivenWind/cv_idl/init.c:155-382): density and
// pressure floors on every cell (side 0, :199-316; the problem of this
// library's tests has the same floors), inflow-only copy of the first active
// cell at X1_BEG (:319-328), outflow-only copy of the last one at X1_END
// (:331-340), and at X2_BEG the hybrid condition -- velocities reflected
// (v_theta flipped), density and pressure copied from the first active row
// (:343-356); point-mass gravity g_r = -G M / r^2 (:367-382).  A side is a
// user side when its boundary code is PS_BC_USERDEF; the kernels call these
// functions for it.
//
// The midplane branch of cv_idl's side-0 loop (:262-306) writes the ghost
// row next to the last theta cell; every configuration of that problem sets
// X2_END to a standard boundary, which overwrites that row before it is
// read, so it has no effect and is not carried here.
#pragma once

#include "ps_hydro.cuh"
#include "ps_physics.cuh"
#include "ps_wind.cuh"

namespace ps {

// side 0: density and pressure floors of one cell's primitive state;
// returns true if the cell was repaired (its conservative state then has to
// be formed again, PrimToCons3D of the problem's loop).
//
// The problem's loop keeps the sound speed: cs = sqrt(gamma p / rho),
// p' = cs^2 dfloor / gamma, T = p' / dfloor KELVIN mu, and at T < tfloor
// p' = dfloor tfloor / (KELVIN mu), which is pfloor.  Algebraically
// p' = (p / rho) dfloor and T = (p / rho) KELVIN mu: one division in place
// of a square root and four divisions (the FP64 pipe bounds this pass, and
// most cells of the wind sit at the density floor), within 2 ulp of the
// loop's sequence.  The threshold tests run on the bit patterns.
template <int NV>
__device__ __forceinline__ bool UserDefBoundary_Internal(double (&v)[NV], const WindParams &w,
                                                         double gamma)
{
  (void)gamma;
  bool convert = false;
  if (lt_pos(v[RHO], w.dfloor)) {
    const bool neg = lt0(v[RHO]);
    const double rho = neg ? w.dfloor : v[RHO];
    const double pr = v[PRS] / rho;
    const double dfact = neg ? 1.0 : rho * w.inv_dfloor;
    v[RHO] = w.dfloor;
    v[VX1] = dfact * v[VX1];
    v[VX2] = dfact * v[VX2];
    v[VX3] = dfact * v[VX3];
    v[PRS] = lt_pos(pr * w.kmu, w.tfloor) ? w.pfloor : pr * w.dfloor;
    if constexpr (NV > NFLX) v[NFLX] = 0.0;
    convert = true;
  }
  if (lt_pos(v[PRS], w.pfloor)) {
    v[PRS] = w.pfloor;
    convert = true;
  }
  return convert;
}

// X1_BEG: variable nv of a ghost cell from the first active cell of its row,
// radial velocity limited to inflow
__device__ __forceinline__ double UserDefBoundary_X1Beg(int nv, double v_first)
{
  return nv == VX1 ? dmin(v_first, 0.0) : v_first;
}

// X1_END: from the last active cell of the row, radial velocity limited to
// outflow
__device__ __forceinline__ double UserDefBoundary_X1End(int nv, double v_last)
{
  return nv == VX1 ? dmax(v_last, 0.0) : v_last;
}

// X2_BEG: v_mirror is the variable at the active cell mirrored across the
// boundary (row 2 JBEG - 1 - j), v_first at the first active row; density,
// pressure and (with the entropy switch, which ComputeEntropy derives from
// them after Boundary) the entropy come from v_first
template <int NV>
__device__ __forceinline__ double UserDefBoundary_X2Beg(int nv, double v_mirror, double v_first)
{
  if (nv == RHO || nv == PRS || (NV == NFLX + 2 && nv == NV - 1)) return v_first;
  return nv == VX2 ? v_mirror * -1.0 : v_mirror;
}

// radial component of the point-mass gravity at x1 (code units; gm_code =
// G M / (UNIT_LENGTH UNIT_VELOCITY^2)); the other components are zero
__host__ __device__ __forceinline__ double BodyForceVector_r(double x1, double gm_code)
{
  return -1.0 * gm_code / (x1 * x1);
}

}  // namespace ps
