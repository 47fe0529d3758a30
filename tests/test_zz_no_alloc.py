"""ps_advance_step_noalloc: the entry point for callers that cannot allocate
device memory (their memory belongs to a framework allocator or a fixed
pool, or they run where cudaMalloc is not allowed).  The caller owns the
state buffer; the library takes its stage scratch from a fixed array.

The result must equal the regular AdvanceStep entry point (ps_advance_step,
which allocates its scratch in ps_create) bit for bit, the tolerance used
by every parity test here, over two calls in a row so that the second call
runs on scratch left behind by the first.  This file is named to be
collected last, and it also passes when run alone in a fresh process."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


# (dims, nx, limiter, solver, boundary): the 2-D and 3-D tiles and tensor
# maps, every ghost-zone rule the entry point accepts, both limiters and
# both Riemann solvers; each within the 32768-cell scratch
CASES = [
    (2, (64, 64, 1), "mc", "hllc", "outflow"),
    (2, (40, 56, 1), "vl", "hllc", "reflective"),
    (3, (16, 16, 16), "mc", "hll", "periodic"),
    (3, (12, 20, 8), "vl", "hllc", "outflow"),
]


def _case(dims, nx, limiter, solver, bc):
    import psgb
    cfg = psgb.make_config(dims=dims, nx=nx, limiter=limiter, solver=solver, bc=bc,
                           cfl=0.4, cfl_max_var=1.1, tstop=10.0, first_dt=1e-4)
    grid = psgb.Grid(cfg)
    return cfg, grid, psgb.blast_state(cfg, grid)


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _active(V, dims):
    return V[:, 2:-2, 2:-2, 2:-2] if dims == 3 else V[:, 0, 2:-2, 2:-2]


@pytest.mark.parametrize("dims,nx,limiter,solver,bc", CASES,
                         ids=["2d-mc-hllc-outflow", "2d-vl-hllc-reflective",
                              "3d-mc-hll-periodic", "3d-vl-hllc-outflow"])
def test_noalloc_matches_advance_step_on_two_calls(built, dims, nx, limiter, solver, bc):
    import torch
    import psgb

    cfg, grid, V0 = _case(dims, nx, limiter, solver, bc)
    ref = psgb.Solver(cfg, grid)
    ref.set_state(V0)
    ref.set_time(0.0, 1e-4, 0)

    state = torch.from_numpy(V0.copy()).cuda()  # the caller's own device buffer
    dx = [np.ascontiguousarray(grid.arrays[d][3]) for d in range(3)]
    L = psgb.lib()
    dt = 1e-4
    for _ in range(2):
        flags_ref, inv_ref = ref.advance_step(dt, 0.0)
        inv = ctypes.c_double(0.0)
        rc = L.ps_advance_step_noalloc(ctypes.byref(cfg), _dp(dx[0]), _dp(dx[1]), _dp(dx[2]),
                                       ctypes.c_void_p(state.data_ptr()), dt, ctypes.byref(inv),
                                       None)
        assert rc == 0, L.ps_last_error().decode()
        assert flags_ref == 0
        assert inv.value == inv_ref
        got = _active(state.cpu().numpy(), dims)
        want = _active(ref.get_state(), dims)
        assert np.array_equal(got, want), f"max |diff| {np.abs(got - want).max():.3e}"
        dt_hyp = 1.0 / inv_ref
        dt_hyp *= cfg.cfl
        dt = min(dt_hyp, cfg.cfl_max_var * dt)
    ref.close()


def test_noalloc_rejects_the_wind_numerics_switches(built):
    import torch
    import psgb
    cfg, grid, _ = _case(2, (32, 32, 1), "mc", "hllc", "outflow")
    dx = [np.ascontiguousarray(grid.arrays[d][3]) for d in range(3)]
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")  # rejected before any use
    for field in ("char_limiting", "shock_flattening", "entropy_switch"):
        setattr(cfg, field, 1)
        inv = ctypes.c_double(0.0)
        rc = psgb.lib().ps_advance_step_noalloc(ctypes.byref(cfg), _dp(dx[0]), _dp(dx[1]),
                                                _dp(dx[2]), ctypes.c_void_p(buf.data_ptr()),
                                                1e-4, ctypes.byref(inv), None)
        assert rc == -1, field
        assert b"spherical wind context" in psgb.lib().ps_last_error()
        setattr(cfg, field, 0)


def test_noalloc_rejects_grids_beyond_the_scratch(built):
    import torch
    import psgb
    cfg = psgb.make_config(dims=2, nx=(256, 256, 1))
    grid = psgb.Grid(cfg)
    dx = [np.ascontiguousarray(grid.arrays[d][3]) for d in range(3)]
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")  # rejected before any use
    inv = ctypes.c_double(0.0)
    rc = psgb.lib().ps_advance_step_noalloc(ctypes.byref(cfg), _dp(dx[0]), _dp(dx[1]),
                                            _dp(dx[2]), ctypes.c_void_p(buf.data_ptr()), 1e-4,
                                            ctypes.byref(inv), None)
    assert rc == -1
    assert b"32768" in psgb.lib().ps_last_error()
