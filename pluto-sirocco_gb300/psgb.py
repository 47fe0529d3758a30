"""ctypes binding of libps_gb300.so (include/ps_gb300.h) for Python callers.

The library is the product; this module only marshals arrays.  It raises
if the library is missing: there is no CPU fallback.
"""
import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libps_gb300.so")
PROBE_PATH = os.path.join(PKG, "libps_probe.so")

CARTESIAN, SPHERICAL = 0, 3
LIM = {"mc": 0, "vl": 1, "mm": 2}
SOLVER = {"hllc": 0, "hll": 1}
BC = {"outflow": 1, "reflective": 2, "axisymmetric": 3, "eqtsymmetric": 4,
      "periodic": 5, "userdef": 8}
GRID = {"uniform": 0, "log": 1, "ratio": 2}
FLAGS = {0x01: "nan", 0x02: "cons2prim", 0x04: "negative_density", 0x08: "dt_too_small",
         0x10: "tma_timeout"}

# Exported entry points declared in include/ps_gb300.h.
EXPORTS = ["ps_last_error", "ps_grid_build", "ps_init_blast", "ps_create", "ps_destroy",
           "ps_set_grid", "ps_set_state", "ps_get_state", "ps_set_time", "ps_get_time",
           "ps_advance_step", "ps_run", "ps_sync", "ps_device_state", "ps_launch_count",
           "ps_get_dt_history", "ps_set_stream", "ps_save_state",
           "ps_restore_state", "ps_time_step_kernels", "ps_advance_step_noalloc",
           "ps_init_wind", "ps_wind_synthetic_flux", "ps_wind_synthetic_flux_dense",
           "ps_set_wind", "ps_split_source",
           "ps_batch_create", "ps_batch_destroy", "ps_batch_run", "ps_batch_sync",
           "ps_batch_set_stream", "ps_batch_launch_count", "ps_batch_set_shape",
           "ps_batch_get_shape", "ps_batch_autotune", "ps_batch_time_step_kernels",
           "ps_sg_create", "ps_sg_destroy", "ps_sg_set_params", "ps_sg_get_params",
           "ps_sg_save", "ps_sg_load",
           "ps_sg_label", "ps_sg_set_data", "ps_sg_train", "ps_sg_grad", "ps_sg_predict",
           "ps_sg_stats", "ps_set_surrogate", "ps_batch_set_surrogate", "ps_sg_collect",
           "ps_set_cooling", "ps_write_dbl", "ps_read_dbl", "ps_read_sirocco_fluxes",
           "ps_read_sirocco_heatcool", "ps_read_sirocco_prefactors", "ps_set_sirocco",
           "ps_read_m_uv_fit", "ps_set_mfit", "ps_batch_set_states", "ps_batch_get_states",
           "ps_batch_set_states_async", "ps_batch_get_states_async", "ps_batch_set_groups",
           "ps_split_source_dt"]


class Config(ctypes.Structure):
    _fields_ = [("dims", ctypes.c_int), ("nx", ctypes.c_int * 3), ("nvar", ctypes.c_int),
                ("geometry", ctypes.c_int), ("limiter", ctypes.c_int), ("solver", ctypes.c_int),
                ("bc", ctypes.c_int * 6), ("gamma", ctypes.c_double), ("cfl", ctypes.c_double),
                ("cfl_max_var", ctypes.c_double), ("tstop", ctypes.c_double),
                ("first_dt", ctypes.c_double), ("cooling", ctypes.c_int),
                ("char_limiting", ctypes.c_int), ("shock_flattening", ctypes.c_int),
                ("entropy_switch", ctypes.c_int)]


class Wind(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in
                ("unit_density", "unit_length", "unit_velocity", "mu", "rho_0", "cent_mass",
                 "t_iso", "l_star", "f_x", "f_uv", "t_x", "krad", "alpharad", "dfloor")] + \
               [(n, ctypes.c_int) for n in ("body_force", "line_force", "floors", "nangles")]


# The line-driven disk wind problem: 512 x 256 (r, theta) by default,
# r log-spaced 1e10..1e12 cm, theta uniform 0..pi/2; 7 solar masses;
# halo 1e-20 g/cm^3; disk-plane layer 1e-9 g/cm^3 at 4e4 K; L_x = 1e37 erg/s;
# M = 0.2 t^-0.6, M_max = 4400.
WIND_PARAMS = dict(unit_density=1e-14, unit_length=1e9, unit_velocity=1e9, mu=0.6,
                   rho_0=1.0e-9, cent_mass=1.4e34, t_iso=4.0e4, l_star=1.0e37, f_x=1.0,
                   f_uv=1.0, t_x=5.6e7, krad=0.2, alpharad=-0.6, dfloor=1.0e-20)


def make_wind(line_force=1, body_force=1, floors=1, nangles=36, **over):
    w = Wind()
    for k, v in dict(WIND_PARAMS, **over).items():
        setattr(w, k, v)
    w.body_force, w.line_force, w.floors, w.nangles = body_force, line_force, floors, nangles
    return w


_lib = None


class Cooling(ctypes.Structure):
    _fields_ = [("unit_density", ctypes.c_double), ("unit_length", ctypes.c_double),
                ("unit_velocity", ctypes.c_double), ("mu", ctypes.c_double),
                ("t_x", ctypes.c_double), ("xi", ctypes.c_double)]


class SgBox(ctypes.Structure):
    _fields_ = [("lo", ctypes.c_double * 4), ("hi", ctypes.c_double * 4),
                ("t_x", ctypes.c_double), ("mu", ctypes.c_double)]


def lib():
    """Load the library (raises OSError if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError(f"{LIB_PATH} not built: run pluto-sirocco_gb300/build.py")
        L = ctypes.CDLL(LIB_PATH)
        D, I, P, DP = ctypes.c_double, ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)
        L.ps_last_error.restype = ctypes.c_char_p
        L.ps_grid_build.argtypes = [I, I, I, D, D, D, DP, DP, DP, DP]
        L.ps_init_blast.argtypes = [ctypes.POINTER(Config), DP, DP, DP, D, D, D, D,
                                    ctypes.c_long, DP]
        L.ps_create.argtypes = [ctypes.POINTER(Config), ctypes.POINTER(P)]
        L.ps_destroy.argtypes = [P]
        L.ps_set_grid.argtypes = [P, I, DP, DP, DP, DP]
        L.ps_set_state.argtypes = [P, DP]
        L.ps_get_state.argtypes = [P, DP]
        L.ps_set_time.argtypes = [P, D, D, ctypes.c_long]
        L.ps_get_time.argtypes = [P, DP, DP, ctypes.POINTER(ctypes.c_long), DP]
        L.ps_advance_step.argtypes = [P, D, DP]
        L.ps_run.argtypes = [P, I]
        L.ps_sync.argtypes = [P]
        L.ps_device_state.argtypes = [P, ctypes.POINTER(I)]
        L.ps_device_state.restype = ctypes.c_void_p
        L.ps_launch_count.argtypes = [P]
        L.ps_launch_count.restype = ctypes.c_long
        L.ps_get_dt_history.argtypes = [P, DP, I]
        L.ps_set_stream.argtypes = [P, P]
        L.ps_save_state.argtypes = [P]
        L.ps_restore_state.argtypes = [P]
        L.ps_time_step_kernels.argtypes = [P, DP]
        L.ps_advance_step_noalloc.argtypes = [ctypes.POINTER(Config), DP, DP, DP,
                                              ctypes.c_void_p, D, DP, ctypes.c_void_p]
        L.ps_init_wind.argtypes = [ctypes.POINTER(Config), ctypes.POINTER(Wind), DP, DP, DP, DP,
                                   DP, DP, DP, DP]
        L.ps_wind_synthetic_flux.argtypes = [ctypes.POINTER(Config), ctypes.POINTER(Wind), DP,
                                             DP, DP, DP, DP]
        L.ps_wind_synthetic_flux_dense.argtypes = [ctypes.POINTER(Config),
                                                   ctypes.POINTER(Wind), DP, DP, DP, DP, DP]
        L.ps_set_wind.argtypes = [P, ctypes.POINTER(Wind), DP, DP, DP]
        L.ps_split_source.argtypes = [P, D, D]
        L.ps_split_source_dt.argtypes = [P, D, D, DP]
        L.ps_batch_create.argtypes = [ctypes.POINTER(P), I, ctypes.POINTER(P)]
        L.ps_batch_destroy.argtypes = [P]
        L.ps_batch_run.argtypes = [P, I]
        L.ps_batch_sync.argtypes = [P]
        L.ps_batch_set_states.argtypes = [P, ctypes.POINTER(DP)]
        L.ps_batch_get_states.argtypes = [P, ctypes.POINTER(DP)]
        L.ps_batch_set_states_async.argtypes = [P, ctypes.POINTER(DP)]
        L.ps_batch_get_states_async.argtypes = [P, ctypes.POINTER(DP)]
        L.ps_batch_set_stream.argtypes = [P, P]
        L.ps_batch_set_groups.argtypes = [P, I]
        L.ps_batch_launch_count.argtypes = [P]
        L.ps_batch_launch_count.restype = ctypes.c_long
        L.ps_batch_set_shape.argtypes = [P, I, I]
        L.ps_batch_get_shape.argtypes = [P, I, ctypes.POINTER(I), ctypes.POINTER(I)]
        L.ps_batch_autotune.argtypes = [P, I]
        L.ps_batch_time_step_kernels.argtypes = [P, ctypes.POINTER(ctypes.c_float)]
        FP = ctypes.POINTER(ctypes.c_float)
        DP = ctypes.POINTER(ctypes.c_double)
        IP = ctypes.POINTER(ctypes.c_int)
        Lg = ctypes.c_long
        L.ps_sg_create.argtypes = [ctypes.POINTER(SgBox), ctypes.POINTER(P)]
        L.ps_sg_destroy.argtypes = [P]
        L.ps_sg_set_params.argtypes = [P, FP]
        L.ps_sg_get_params.argtypes = [P, FP]
        L.ps_sg_save.argtypes = [P, ctypes.c_char_p]
        L.ps_sg_load.argtypes = [ctypes.c_char_p, ctypes.POINTER(P)]
        L.ps_sg_label.argtypes = [P, DP, Lg, DP, DP]
        L.ps_sg_set_data.argtypes = [P, DP, DP, Lg]
        L.ps_sg_train.argtypes = [P, I, I, ctypes.c_float, ctypes.c_float, ctypes.c_ulonglong, FP]
        L.ps_sg_grad.argtypes = [P, DP, DP, I, FP, FP]
        L.ps_sg_predict.argtypes = [P, DP, Lg, I, DP, IP, DP]
        L.ps_sg_stats.argtypes = [P, ctypes.POINTER(ctypes.c_longlong), I]
        L.ps_set_surrogate.argtypes = [P, P, I]
        L.ps_batch_set_surrogate.argtypes = [P, P, I]
        L.ps_sg_collect.argtypes = [P, DP, Lg, ctypes.POINTER(Lg)]
        L.ps_set_cooling.argtypes = [P, ctypes.POINTER(Cooling)]
        L.ps_write_dbl.argtypes = [P, ctypes.c_char_p, I, ctypes.c_char_p]
        L.ps_read_dbl.argtypes = [P, ctypes.c_char_p]
        CP = ctypes.POINTER(Config)
        LP = ctypes.POINTER(ctypes.c_long)
        L.ps_read_sirocco_fluxes.argtypes = [CP, D, DP, DP, ctypes.c_char_p, I, DP, DP, DP, LP]
        L.ps_read_sirocco_heatcool.argtypes = [CP, D, DP, DP, ctypes.c_char_p, DP, DP, LP]
        L.ps_read_sirocco_prefactors.argtypes = [CP, D, DP, DP, ctypes.c_char_p, DP, LP]
        L.ps_set_sirocco.argtypes = [P, DP, DP, DP]
        L.ps_read_m_uv_fit.argtypes = [CP, D, DP, DP, ctypes.c_char_p, ctypes.c_int, DP, DP, LP]
        L.ps_set_mfit.argtypes = [P, ctypes.c_int, DP, DP]
        _lib = L
    return _lib


_probe = None


def probe():
    """The measurement helpers (libps_probe.so, not part of the C ABI): the
    FP64 issue-rate probe of the roofline, the fast-math check, the
    partial-warp FP64 timing and the bounded-wait failure check."""
    global _probe
    if _probe is None:
        if not os.path.exists(PROBE_PATH):
            raise OSError(f"{PROBE_PATH} not built: run pluto-sirocco_gb300/ps_build.py")
        L = ctypes.CDLL(PROBE_PATH)
        DP = ctypes.POINTER(ctypes.c_double)
        L.ps_probe_fp64_flops.argtypes = [ctypes.c_int]
        L.ps_probe_fp64_flops.restype = ctypes.c_double
        L.ps_probe_fastmath.argtypes = [ctypes.c_int, DP, DP, DP, ctypes.c_long]
        L.ps_probe_fp64_lanes.argtypes = [ctypes.c_int] * 5
        L.ps_probe_fp64_lanes.restype = ctypes.c_double
        L.ps_probe_dmul_rate.argtypes = [ctypes.c_int] * 4
        L.ps_probe_dmul_rate.restype = ctypes.c_double
        L.ps_probe_dmul_check.argtypes = [ctypes.c_int, ctypes.c_ulonglong, ctypes.c_longlong,
                                          ctypes.POINTER(ctypes.c_ulonglong)]
        L.ps_probe_wait_timeout.argtypes = [ctypes.c_int, ctypes.c_int,
                                            ctypes.POINTER(ctypes.c_int)]
        _probe = L
    return _probe


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def make_config(dims=2, nx=(256, 256, 1), nvar=5, limiter="mc", solver="hllc",
                bc="outflow", gamma=5.0 / 3.0, cfl=0.4, cfl_max_var=1.1, tstop=10.0,
                first_dt=1e-4, cooling=0):
    c = Config()
    c.dims = dims
    n = list(nx) + [1] * (3 - len(nx))
    c.nx[:] = n[:3]
    c.nvar = nvar
    c.geometry = CARTESIAN
    c.limiter = LIM[limiter]
    c.solver = SOLVER[solver]
    bcs = [bc] * 6 if isinstance(bc, str) else list(bc)
    c.bc[:] = [BC[b] for b in bcs]
    c.gamma = gamma
    c.cfl = cfl
    c.cfl_max_var = cfl_max_var
    c.tstop = tstop
    c.first_dt = first_dt
    c.cooling = cooling
    return c


def check(rc, what):
    if rc < 0:
        raise RuntimeError(f"{what} failed ({rc}): {lib().ps_last_error().decode()}")
    return rc


WIND_BC = ["userdef", "outflow", "axisymmetric", "reflective", "outflow", "outflow"]
# the production disk-wind problem (Test_Problems/LineDrivenWind/cv_idl): its
# X2-beg is the hybrid user side (pluto_sirocco_sub.py:78-81)
CVIDL_BC = ["userdef", "outflow", "userdef", "reflective", "outflow", "outflow"]


def make_wind_config(nr=512, nt=256, cooling=1, limiter="vl", solver="hll", cfl=0.4,
                     first_dt=1e-4, char_limiting=0, shock_flattening=0, entropy_switch=0,
                     bc=None):
    """The wind's configuration.  entropy_switch: 0 NO, 1 SELECTIVE, 2 ALWAYS
    (the entropy becomes a seventh variable).  bc: six boundary names
    (default WIND_BC)."""
    c = make_config(dims=2, nx=(nr, nt, 1), nvar=7 if entropy_switch else 6, limiter=limiter,
                    solver=solver, bc=list(bc or WIND_BC),
                    cfl=cfl, cfl_max_var=1.1, tstop=1e10, first_dt=first_dt, cooling=cooling)
    c.geometry = SPHERICAL
    c.char_limiting = char_limiting
    c.shock_flattening = shock_flattening
    c.entropy_switch = entropy_switch
    return c


class WindGrid:
    """r log-spaced on [10, 1000] x UNIT_LENGTH, theta uniform on [0, pi/2]."""

    def __init__(self, cfg):
        g = nghost(cfg)
        self.ngh = [g, g, 0]
        self.ntot = [cfg.nx[0] + 2 * g, cfg.nx[1] + 2 * g, 1]
        self.arrays = [build_grid(cfg.nx[0], g, 10.0, 1000.0, "log"),
                       build_grid(cfg.nx[1], g, 0.0, 1.5707963267948966, "uniform"),
                       build_grid(1, 0, 0.0, 1.0, "uniform")]

    def x(self, d):
        return self.arrays[d][0]


def nghost(cfg):
    """Ghost zones per side of an active direction (GetNghost): 2, or 3
    with MULTID shock flattening."""
    return 3 if cfg.shock_flattening else 2


def wind_state(cfg, wind, grid):
    V = np.zeros((cfg.nvar, 1, grid.ntot[1], grid.ntot[0]))
    a1, a2 = grid.arrays[0], grid.arrays[1]
    check(lib().ps_init_wind(ctypes.byref(cfg), ctypes.byref(wind), _dp(a1[0]), _dp(a1[1]),
                             _dp(a1[2]), _dp(a1[3]), _dp(a2[0]), _dp(a2[1]), _dp(a2[2]),
                             _dp(V)), "ps_init_wind")
    return V


def wind_flux(cfg, wind, grid, dense=False):
    """Synthetic directional UV flux, [angle][k][j][i] over the total box:
    L_UV/(4 pi r^2) in the bin of each cell's radial direction
    (ps_wind_synthetic_flux), or with dense=True in every bin: weight 1 in
    the radial bin and 0.05/(1 + |d|) d bins away, split into (F_r, F_theta)
    by the cosine and sine of the bin's angle from the radial one -- a stand-in
    for SIROCCO's fluxes, which fill most bins.  Values are rounded through
    13 significant digits as the flux files carry them."""
    shape = (wind.nangles, 1, grid.ntot[1], grid.ntot[0])
    fr, ft, fp = np.zeros(shape), np.zeros(shape), np.zeros(shape)
    fn = lib().ps_wind_synthetic_flux_dense if dense else lib().ps_wind_synthetic_flux
    check(fn(ctypes.byref(cfg), ctypes.byref(wind), _dp(grid.x(0)), _dp(grid.x(1)), _dp(fr),
             _dp(ft), _dp(fp)), "ps_wind_synthetic_flux")
    return fr, ft, fp


def build_grid(n, ngh, xbeg=0.0, xend=1.0, kind="uniform", ratio=1.0):
    nt = n + 2 * ngh
    x, xl, xr, dx = (np.zeros(nt) for _ in range(4))
    check(lib().ps_grid_build(GRID[kind], n, ngh, xbeg, xend, ratio, _dp(x), _dp(xl), _dp(xr),
                              _dp(dx)), "ps_grid_build")
    return x, xl, xr, dx


class Grid:
    """Grid arrays of the total box for every direction (as SetGrid builds them)."""

    def __init__(self, cfg, xbeg=(0.0, 0.0, 0.0), xend=(1.0, 1.0, 1.0)):
        self.ngh = [2 if d < cfg.dims else 0 for d in range(3)]
        self.ntot = [cfg.nx[d] + 2 * self.ngh[d] for d in range(3)]
        self.arrays = [build_grid(cfg.nx[d], self.ngh[d], xbeg[d], xend[d]) for d in range(3)]

    def x(self, d):
        return self.arrays[d][0]


def blast_state(cfg, grid, p_amb=0.1, p_in=10.0, r_in=0.1, noise=0.01, seed=1):
    V = np.zeros((cfg.nvar, grid.ntot[2], grid.ntot[1], grid.ntot[0]))
    check(lib().ps_init_blast(ctypes.byref(cfg), _dp(grid.x(0)), _dp(grid.x(1)), _dp(grid.x(2)),
                              p_amb, p_in, r_in, noise, seed, _dp(V)), "ps_init_blast")
    return V


# The 3-D periodic cooling configuration: BLONDIN at constant xi = 1e2 with
# T_x = 5.6e7 K; code density 1 is 1e-10 g/cm^3 (n_H ~ 4e13 cm^-3), which
# puts the cooling time of much of the 1e4-1e7 K gas near the time step
# (code time unit 1 s).
COOL_PARAMS = dict(unit_density=1e-10, unit_length=1e9, unit_velocity=1e9, mu=0.6, t_x=5.6e7,
                   xi=1e2)
AMU, KB = 1.66053886e-24, 1.3806505e-16


def make_cooling(**over):
    c = Cooling()
    for k, v in dict(COOL_PARAMS, **over).items():
        setattr(c, k, v)
    return c


def cube_config(n=512, cooling=1, first_dt=1e-3):
    """n^3 on [0,1]^3, periodic, PLM-MC, HLLC, RK2, CFL 0.4, gamma 5/3."""
    nx = n if isinstance(n, (tuple, list)) else (n, n, n)
    return make_config(dims=3, nx=tuple(nx), limiter="mc", solver="hllc", bc="periodic", cfl=0.4,
                       cfl_max_var=1.1, tstop=1e10, first_dt=first_dt, cooling=cooling)


def cube_state(cfg, grid, seed=5, sigma=0.5, t_lo=1e4, t_hi=1e7, cooling=None):
    """Initial state of the 3-D cooling configuration: rho = exp(sigma g -
    sigma^2/2) with g a unit-variance Gaussian random field of power
    spectrum k^-2 (white noise filtered by 1/|k| with numpy's FFT, seeded),
    T drawn log-uniform in [t_lo, t_hi] per cell, v = 0,
    p = rho T / (KELVIN mu) in code units; ghost cells periodic."""
    cp = cooling or make_cooling()
    nx, ny, nz = cfg.nx[0], cfg.nx[1], cfg.nx[2]
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((nz, ny, nx))
    f = np.fft.rfftn(w)
    del w
    kz = np.fft.fftfreq(nz)[:, None, None]
    ky = np.fft.fftfreq(ny)[None, :, None]
    kx = np.fft.rfftfreq(nx)[None, None, :]
    k2 = kz * kz + ky * ky + kx * kx
    k2[0, 0, 0] = 1.0
    f /= np.sqrt(k2)
    f[0, 0, 0] = 0.0
    del k2
    g = np.fft.irfftn(f, s=(nz, ny, nx), axes=(0, 1, 2))
    del f
    g /= g.std()
    rho = np.exp(sigma * g - 0.5 * sigma * sigma)
    del g
    T = 10.0 ** rng.uniform(np.log10(t_lo), np.log10(t_hi), (nz, ny, nx))
    kelvin = cp.unit_velocity ** 2 * AMU / KB
    V = np.zeros((cfg.nvar, nz + 4, ny + 4, nx + 4))
    act = (slice(2, -2), slice(2, -2), slice(2, -2))
    V[(0,) + act] = rho
    V[(4,) + act] = rho * T / (kelvin * cp.mu)
    del rho, T
    for v in (0, 4):
        V[v] = np.pad(V[(v,) + act], 2, mode="wrap")
    return V


def cube_solver(n, cooling=None, seed=5):
    """Device context of the 3-D cooling configuration with its initial state."""
    cfg = cube_config(n)
    g = Grid(cfg)
    s = Solver(cfg, g)
    s.set_state(cube_state(cfg, g, seed=seed, cooling=cooling))
    s.set_time(0.0, cfg.first_dt, 0)
    s.set_cooling(cooling or make_cooling())
    return s


class Solver:
    """One device context (ps_ctx) on the current CUDA device."""

    def __init__(self, cfg, grid):
        self.cfg = cfg
        self.grid = grid
        self.ctx = ctypes.c_void_p()
        check(lib().ps_create(ctypes.byref(cfg), ctypes.byref(self.ctx)), "ps_create")
        for d in range(cfg.dims):
            x, xl, xr, dx = grid.arrays[d]
            check(lib().ps_set_grid(self.ctx, d, _dp(x), _dp(xl), _dp(xr), _dp(dx)),
                  "ps_set_grid")

    def close(self):
        if self.ctx:
            lib().ps_destroy(self.ctx)
            self.ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, V):
        V = np.ascontiguousarray(V, dtype=np.float64)
        check(lib().ps_set_state(self.ctx, _dp(V)), "ps_set_state")

    def get_state(self, out=None):
        g = self.grid
        shape = (self.cfg.nvar, g.ntot[2], g.ntot[1], g.ntot[0])
        V = np.zeros(shape) if out is None else out
        if V.shape != shape or V.dtype != np.float64 or not V.flags.c_contiguous:
            raise ValueError("output array must be C-contiguous float64 of shape %s" % (shape,))
        check(lib().ps_get_state(self.ctx, _dp(V)), "ps_get_state")
        return V

    def write_dbl(self, directory, nfile, names=None):
        check(lib().ps_write_dbl(self.ctx, os.fsencode(directory), nfile,
                                 names.encode() if names else None), "ps_write_dbl")

    def read_dbl(self, path):
        check(lib().ps_read_dbl(self.ctx, os.fsencode(path)), "ps_read_dbl")

    def set_sirocco(self, xi=None, t_r=None, pre=None):
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64)
                for a in (xi, t_r, pre)]
        self._sirocco = arrs
        check(lib().ps_set_sirocco(self.ctx, *[None if a is None else _dp(a) for a in arrs]),
              "ps_set_sirocco")

    def set_mfit(self, t_fit, m_fit):
        """The tabulated force multiplier (KRAD = ALPHARAD = 999): t values
        and M [point][j][i] (or [point][k][j][i]) over the total box."""
        t, m = (np.ascontiguousarray(a, dtype=np.float64) for a in (t_fit, m_fit))
        self._mfit = (t, m)
        check(lib().ps_set_mfit(self.ctx, len(t), _dp(t), _dp(m)), "ps_set_mfit")

    def set_cooling(self, cooling):
        check(lib().ps_set_cooling(self.ctx, ctypes.byref(cooling)), "ps_set_cooling")

    def set_wind(self, wind, flux=None):
        if flux is None:
            shape = (max(wind.nangles, 1), 1, self.grid.ntot[1], self.grid.ntot[0])
            flux = (np.zeros(shape),) * 3
        self._flux = [np.ascontiguousarray(f, dtype=np.float64) for f in flux]
        check(lib().ps_set_wind(self.ctx, ctypes.byref(wind), *(_dp(f) for f in self._flux)),
              "ps_set_wind")

    def set_time(self, t, dt, step=0):
        check(lib().ps_set_time(self.ctx, t, dt, step), "ps_set_time")

    def time(self):
        t, dt, inv = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        st = ctypes.c_long()
        check(lib().ps_get_time(self.ctx, ctypes.byref(t), ctypes.byref(dt), ctypes.byref(st),
                                ctypes.byref(inv)), "ps_get_time")
        return t.value, dt.value, st.value, inv.value

    def run(self, nsteps, wait=True):
        """nsteps steps on the device; wait=False only queues them on the
        context's stream (sync() then returns the flags)."""
        check(lib().ps_run(self.ctx, nsteps), "ps_run")
        return self.sync() if wait else 0

    def advance_step(self, dt, inv_dt_hyp=0.0):
        inv = ctypes.c_double(inv_dt_hyp)
        rc = check(lib().ps_advance_step(self.ctx, dt, ctypes.byref(inv)), "ps_advance_step")
        return rc, inv.value

    def split_source(self, dt, t):
        return check(lib().ps_split_source(self.ctx, dt, t), "ps_split_source")

    def split_source_dt(self, dt, t):
        """(flags, dt_cool of this pass)."""
        out = ctypes.c_double()
        rc = check(lib().ps_split_source_dt(self.ctx, dt, t, ctypes.byref(out)),
                   "ps_split_source_dt")
        return rc, out.value

    def sync(self):
        return check(lib().ps_sync(self.ctx), "ps_sync")

    def dt_history(self, n):
        out = np.zeros(n)
        k = check(lib().ps_get_dt_history(self.ctx, _dp(out), n), "ps_get_dt_history")
        return out[:k]

    def launches(self):
        return lib().ps_launch_count(self.ctx)

    def save(self):
        check(lib().ps_save_state(self.ctx), "ps_save_state")

    def restore(self):
        check(lib().ps_restore_state(self.ctx), "ps_restore_state")

    def time_step_kernels(self):
        ms = np.zeros(3)
        check(lib().ps_time_step_kernels(self.ctx, _dp(ms)), "ps_time_step_kernels")
        return ms

    def set_stream(self, stream_handle):
        check(lib().ps_set_stream(self.ctx, ctypes.c_void_p(stream_handle)), "ps_set_stream")

    def device_state(self):
        pitch = ctypes.c_int()
        ptr = lib().ps_device_state(self.ctx, ctypes.byref(pitch))
        return ptr, pitch.value


class Batch:
    """Independent wind models advanced together (ps_batch)."""

    def __init__(self, solvers):
        self.solvers = list(solvers)
        arr = (ctypes.c_void_p * len(self.solvers))(*[s.ctx.value for s in self.solvers])
        self.h = ctypes.c_void_p()
        check(lib().ps_batch_create(arr, len(self.solvers), ctypes.byref(self.h)),
              "ps_batch_create")

    def close(self):
        if self.h:
            lib().ps_batch_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, nsteps, wait=True):
        """nsteps steps of every model; wait=False only queues them (sync()
        then returns the flags)."""
        check(lib().ps_batch_run(self.h, nsteps), "ps_batch_run")
        return self.sync() if wait else 0

    def set_states_async(self, arrays):
        """set_states by the copy engines, queued without waiting (the
        arrays, pinned, are in use until sync())."""
        self._check_states(arrays)
        self._state_refs = list(arrays)
        ptrs = (ctypes.POINTER(ctypes.c_double) * len(arrays))(*[_dp(a) for a in arrays])
        check(lib().ps_batch_set_states_async(self.h, ptrs), "ps_batch_set_states_async")

    def get_states_async(self, arrays):
        """get_states by the copy engines, queued without waiting."""
        self._check_states(arrays)
        self._out_refs = list(arrays)
        ptrs = (ctypes.POINTER(ctypes.c_double) * len(arrays))(*[_dp(a) for a in arrays])
        check(lib().ps_batch_get_states_async(self.h, ptrs), "ps_batch_get_states_async")

    def set_states(self, arrays):
        """Every model's state from host arrays (one per model, each the
        shape get_state() returns; pinned memory for full copy speed)."""
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in arrays]
        self._check_states(arrs)
        self._state_refs = arrs
        ptrs = (ctypes.POINTER(ctypes.c_double) * len(arrs))(*[_dp(a) for a in arrs])
        check(lib().ps_batch_set_states(self.h, ptrs), "ps_batch_set_states")

    def _check_states(self, arrays):
        if len(arrays) != len(self.solvers):
            raise ValueError("one array per model")
        for a, sv in zip(arrays, self.solvers):
            g = sv.grid
            want = sv.cfg.nvar * g.ntot[0] * g.ntot[1] * g.ntot[2]
            if a.size != want or a.dtype != np.float64 or not a.flags.c_contiguous:
                raise ValueError("a state array does not match its model's [nv][k][j][i] box")

    def get_states(self, arrays):
        """Every model's state into the given host arrays (written in place)."""
        self._check_states(arrays)
        ptrs = (ctypes.POINTER(ctypes.c_double) * len(arrays))(*[_dp(a) for a in arrays])
        check(lib().ps_batch_get_states(self.h, ptrs), "ps_batch_get_states")

    def sync(self):
        return check(lib().ps_batch_sync(self.h), "ps_batch_sync")

    def set_stream(self, handle):
        check(lib().ps_batch_set_stream(self.h, ctypes.c_void_p(handle)), "ps_batch_set_stream")

    def set_groups(self, n):
        check(lib().ps_batch_set_groups(self.h, n), "ps_batch_set_groups")

    def launches(self):
        return lib().ps_batch_launch_count(self.h)

    def set_shape(self, shape, model=-1):
        check(lib().ps_batch_set_shape(self.h, model, shape), "ps_batch_set_shape")

    def shape(self, model):
        tx, ty = ctypes.c_int(), ctypes.c_int()
        lib().ps_batch_get_shape(self.h, model, ctypes.byref(tx), ctypes.byref(ty))
        return tx.value, ty.value

    def autotune(self, reps=5):
        check(lib().ps_batch_autotune(self.h, reps), "ps_batch_autotune")

    def time_step_kernels(self):
        ms = (ctypes.c_float * 3)()
        check(lib().ps_batch_time_step_kernels(self.h, ms), "ps_batch_time_step_kernels")
        return np.array(ms[:], dtype=np.float64)


# Grid sizes and parameter ranges of the batched-wind configuration.
BATCH_GRIDS = [(128, 64), (256, 128), (384, 192), (512, 256)]


def batch_models(n=64, seed=4):
    """Per-model (grid, L_x, krad, alpha) drawn with numpy's seeded generator:
    L_x log-uniform in 1e36..1e38 erg/s, k uniform in 0.1..0.4, alpha
    uniform in 0.5..0.7 (M = k t^-alpha), grid uniform over BATCH_GRIDS."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        g = BATCH_GRIDS[int(rng.integers(0, len(BATCH_GRIDS)))]
        lx = 10 ** rng.uniform(36.0, 38.0)
        k = rng.uniform(0.1, 0.4)
        a = rng.uniform(0.5, 0.7)
        out.append(dict(grid=g, l_star=lx, krad=k, alpharad=-a))
    return out


def wind_model_solver(spec, cooling=1, line_force=1, char_limiting=0, shock_flattening=0,
                      entropy_switch=0, dense_flux=False):
    """One wind context for a batch spec (see batch_models)."""
    nr, nt = spec["grid"]
    cfg = make_wind_config(nr, nt, cooling=cooling, char_limiting=char_limiting,
                           shock_flattening=shock_flattening, entropy_switch=entropy_switch)
    w = make_wind(line_force=line_force, l_star=spec["l_star"], krad=spec["krad"],
                  alpharad=spec["alpharad"])
    g = WindGrid(cfg)
    s = Solver(cfg, g)
    s.set_state(wind_state(cfg, w, g))
    s.set_time(0.0, 1e-4, 0)
    s.set_wind(w, wind_flux(cfg, w, g, dense=dense_flux) if line_force else None)
    return s


# ----------------------------------------------------------------------
# learned cooling step
# ----------------------------------------------------------------------

N_SG_PARAMS = 4545
SG_ACCEPT, SG_OUT_OF_BOX, SG_REJECT, SG_BELOW_MIN = 0, 1, 2, 3
# log-uniform draws of the training set: n_H [cm^-3], T [K], xi, dt [s]
SG_DRAW_BOX = ((-2.0, 12.0), (4.0, 8.0), (-1.0, 5.0), (-5.0, 0.0))


def _np_dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Surrogate:
    """The learned BLONDIN step (ps_surrogate)."""

    def __init__(self, lo, hi, t_x=5.6e7, mu=0.6):
        b = SgBox()
        b.lo[:] = [float(v) for v in lo]
        b.hi[:] = [float(v) for v in hi]
        b.t_x, b.mu = t_x, mu
        self.box = b
        self.h = ctypes.c_void_p()
        check(lib().ps_sg_create(ctypes.byref(b), ctypes.byref(self.h)), "ps_sg_create")

    def close(self):
        if self.h:
            lib().ps_sg_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self):
        p = np.zeros(N_SG_PARAMS, dtype=np.float32)
        check(lib().ps_sg_get_params(self.h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float))),
              "ps_sg_get_params")
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        check(lib().ps_sg_set_params(self.h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float))),
              "ps_sg_set_params")

    def save(self, path):
        """The box and the parameters to a file (ps_sg_save)."""
        check(lib().ps_sg_save(self.h, os.fsencode(path)), "ps_sg_save")

    @classmethod
    def load(cls, path):
        """A surrogate from a file written by save() (ps_sg_load)."""
        self = cls.__new__(cls)
        self.h = ctypes.c_void_p()
        check(lib().ps_sg_load(os.fsencode(path), ctypes.byref(self.h)), "ps_sg_load")
        self.box = None
        return self

    def label(self, tuples, t_cool=False):
        t = np.ascontiguousarray(tuples, dtype=np.float64)
        out = np.zeros(len(t))
        tc = np.zeros(len(t)) if t_cool else None
        check(lib().ps_sg_label(self.h, _np_dp(t), len(t), _np_dp(out),
                                _np_dp(tc) if t_cool else None), "ps_sg_label")
        return (out, tc) if t_cool else out

    def set_data(self, tuples, t_new):
        t = np.ascontiguousarray(tuples, dtype=np.float64)
        y = np.ascontiguousarray(t_new, dtype=np.float64)
        check(lib().ps_sg_set_data(self.h, _np_dp(t), _np_dp(y), len(t)), "ps_sg_set_data")

    def train(self, steps, batch=8192, lr=3e-3, lr_end=3e-5, seed=3):
        hist = np.zeros(steps, dtype=np.float32)
        flags = check(lib().ps_sg_train(self.h, steps, batch, lr, lr_end, seed,
                                        hist.ctypes.data_as(ctypes.POINTER(ctypes.c_float))),
                      "ps_sg_train")
        return hist, flags

    def grad(self, tuples, t_new):
        t = np.ascontiguousarray(tuples, dtype=np.float64)
        y = np.ascontiguousarray(t_new, dtype=np.float64)
        g = np.zeros(N_SG_PARAMS, dtype=np.float32)
        loss = ctypes.c_float()
        flags = check(lib().ps_sg_grad(self.h, _np_dp(t), _np_dp(y), len(t),
                                       g.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                       ctypes.byref(loss)), "ps_sg_grad")
        return g, loss.value, flags

    def predict(self, tuples, use_net=1):
        t = np.ascontiguousarray(tuples, dtype=np.float64)
        out = np.zeros(len(t))
        st = np.zeros(len(t), dtype=np.int32)
        t0 = np.zeros(len(t))
        check(lib().ps_sg_predict(self.h, _np_dp(t), len(t), use_net, _np_dp(out),
                                  st.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _np_dp(t0)),
              "ps_sg_predict")
        return out, st, t0

    def stats(self, reset=True):
        """accepted, out of box, rejected, below 1e4 K, judge evaluations, stiff cells"""
        out = (ctypes.c_longlong * 6)()
        check(lib().ps_sg_stats(self.h, out, int(reset)), "ps_sg_stats")
        return list(out)


def sg_draws(n, seed=3, box=SG_DRAW_BOX):
    """Log-uniform (n_H, T, xi, dt) draws over `box` (numpy, seeded)."""
    rng = np.random.default_rng(seed)
    return np.stack([10.0 ** rng.uniform(lo, hi, n) for lo, hi in box], axis=1)


def sg_collect(solver, cap=1 << 22):
    """(n_H, T, xi, dt) of the cells the next split-source step would solve."""
    out = np.zeros((cap, 4))
    n = ctypes.c_long()
    check(lib().ps_sg_collect(solver.ctx, _np_dp(out), cap, ctypes.byref(n)), "ps_sg_collect")
    return out[:n.value].copy()


def sg_box_of(tuples, pad=0.05):
    """log10 bounding box of a tuple set, padded by `pad` decades."""
    lt = np.log10(tuples)
    return lt.min(axis=0) - pad, lt.max(axis=0) + pad


def wind_training_tuples(specs, steps=(0, 40, 120, 240), per_model=4000, seed=3, cooling=1):
    """Tuples from wind runs: each spec run on the GPU, sampled at the given
    step numbers (`per_model` cells drawn at random from each snapshot)."""
    rng = np.random.default_rng(seed)
    rows = []
    for sp in specs:
        s = wind_model_solver(sp, cooling=cooling)
        done = 0
        for st in steps:
            if st > done:
                s.run(st - done)
                done = st
            t = sg_collect(s)
            if len(t):
                k = rng.choice(len(t), size=min(per_model, len(t)), replace=False)
                rows.append(t[k])
        s.close()
    return np.concatenate(rows) if rows else np.zeros((0, 4))


def sg_stiff_draws(sg, n, seed=3, box=SG_DRAW_BOX, ratio=(-1.0, 2.0)):
    """Log-uniform (n_H, T, xi) draws whose dt is a log-uniform multiple
    10^ratio of the cell's own cooling time (clipped to the dt range of
    `box`): the stiff cells, where the prediction is what the Newton steps
    start from."""
    rng = np.random.default_rng(seed + 1000)
    t = sg_draws(n, seed=seed, box=box)
    _, tc = sg.label(t, t_cool=True)
    dt = tc * 10.0 ** rng.uniform(ratio[0], ratio[1], n)
    t[:, 3] = np.clip(dt, 10.0 ** box[3][0], 10.0 ** box[3][1])
    return t


def train_surrogate(wind_tuples, n_draws=500000, steps=20000, batch=8192, seed=3, t_x=5.6e7,
                    mu=0.6, stiff_frac=0.5):
    """The learned cooling step: log-uniform draws (a fraction `stiff_frac`
    of them with dt drawn relative to the cooling time) plus wind tuples,
    labelled by the reference method on the GPU and trained with Adam on the
    GPU.  The box is the bounding box of the training tuples with
    T >= 1e4 K.  Returns (surrogate, loss history, tuples, labels)."""
    n_stiff = int(n_draws * stiff_frac)
    probe = Surrogate(*zip(*SG_DRAW_BOX), t_x=t_x, mu=mu)
    parts = [sg_draws(n_draws - n_stiff, seed=seed), sg_stiff_draws(probe, n_stiff, seed=seed)]
    probe.close()
    if len(wind_tuples):
        parts.append(wind_tuples)
    tup = np.concatenate(parts)
    tup = tup[tup[:, 1] >= 1e4]
    lo, hi = sg_box_of(tup)
    sg = Surrogate(lo, hi, t_x=t_x, mu=mu)
    lab = sg.label(tup)
    sg.set_data(tup, lab)
    hist, _ = sg.train(steps, batch=batch, seed=seed)
    return sg, hist, tup, lab


# ----------------------------------------------------------------------
# SIROCCO files
# ----------------------------------------------------------------------

def read_sirocco_fluxes(cfg, grid, directory, unit_length=1e9, max_angles=64):
    """(fr, ft, fp, matched): [angle][1][j][i] arrays over the total box."""
    n0, n1 = cfg.nx[0] + 4, cfg.nx[1] + 4
    arr = [np.zeros((max_angles, 1, n1, n0)) for _ in range(3)]
    m = ctypes.c_long()
    na = check(lib().ps_read_sirocco_fluxes(ctypes.byref(cfg), unit_length, _dp(grid.x(0)),
                                            _dp(grid.x(1)), os.fsencode(directory), max_angles,
                                            *[_dp(a) for a in arr], ctypes.byref(m)),
               "ps_read_sirocco_fluxes")
    return arr[0][:na].copy(), arr[1][:na].copy(), arr[2][:na].copy(), m.value


def read_sirocco_heatcool(cfg, grid, path, xi, t_r, unit_length=1e9):
    m = ctypes.c_long()
    check(lib().ps_read_sirocco_heatcool(ctypes.byref(cfg), unit_length, _dp(grid.x(0)),
                                         _dp(grid.x(1)), os.fsencode(path), _dp(xi), _dp(t_r),
                                         ctypes.byref(m)), "ps_read_sirocco_heatcool")
    return m.value


def read_m_uv_fit(cfg, grid, path, max_points=256, unit_length=1e9):
    """M_UV_data.dat -> (t [n], M [n][j][i] over the total box, cells matched);
    cells without a record keep M = 1."""
    t = np.zeros(max_points)
    m = np.ones((max_points, grid.ntot[1], grid.ntot[0]))
    mc = ctypes.c_long()
    n = lib().ps_read_m_uv_fit(ctypes.byref(cfg), unit_length, _dp(grid.x(0)), _dp(grid.x(1)),
                               os.fsencode(path), max_points, _dp(t), _dp(m), ctypes.byref(mc))
    check(n, "ps_read_m_uv_fit")
    return t[:n].copy(), m[:n].copy(), mc.value


def read_sirocco_prefactors(cfg, grid, path, pre, unit_length=1e9):
    m = ctypes.c_long()
    check(lib().ps_read_sirocco_prefactors(ctypes.byref(cfg), unit_length, _dp(grid.x(0)),
                                           _dp(grid.x(1)), os.fsencode(path), _dp(pre),
                                           ctypes.byref(m)), "ps_read_sirocco_prefactors")
    return m.value
