"""ctypes wrapper of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker.  The product never imports it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

LIM = {"mc": 0, "vl": 1, "mm": 2}
SOLVER = {"hllc": 0, "hll": 1}
BC = {"outflow": 1, "reflective": 2, "axisymmetric": 3, "eqtsymmetric": 4, "periodic": 5,
      "userdef": 8}


class OrConfig(ctypes.Structure):
    _fields_ = [("dims", ctypes.c_int), ("nx", ctypes.c_int * 3), ("nvar", ctypes.c_int),
                ("geometry", ctypes.c_int), ("limiter", ctypes.c_int), ("solver", ctypes.c_int),
                ("bc", ctypes.c_int * 6), ("gridtype", ctypes.c_int * 3),
                ("xbeg", ctypes.c_double * 3), ("xend", ctypes.c_double * 3),
                ("ratio", ctypes.c_double * 3), ("gamma", ctypes.c_double),
                ("cfl", ctypes.c_double), ("cfl_max_var", ctypes.c_double),
                ("tstop", ctypes.c_double), ("first_dt", ctypes.c_double),
                ("cooling", ctypes.c_int), ("body_force", ctypes.c_int),
                ("line_force", ctypes.c_int), ("floors", ctypes.c_int),
                ("unit_density", ctypes.c_double), ("unit_length", ctypes.c_double),
                ("unit_velocity", ctypes.c_double), ("mu", ctypes.c_double),
                ("rho_0", ctypes.c_double), ("cent_mass", ctypes.c_double),
                ("t_iso", ctypes.c_double), ("l_star", ctypes.c_double),
                ("f_x", ctypes.c_double), ("f_uv", ctypes.c_double), ("t_x", ctypes.c_double),
                ("krad", ctypes.c_double), ("alpharad", ctypes.c_double),
                ("dfloor", ctypes.c_double), ("xi_const", ctypes.c_double),
                ("char_limiting", ctypes.c_int), ("shock_flattening", ctypes.c_int),
                ("entropy_switch", ctypes.c_int)]


_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        P, D, I = ctypes.c_void_p, ctypes.c_double, ctypes.c_int
        DP = ctypes.POINTER(ctypes.c_double)
        L.or_create.restype = P
        L.or_create.argtypes = [ctypes.POINTER(OrConfig)]
        L.or_destroy.argtypes = [P]
        L.or_state.restype = DP
        L.or_state.argtypes = [P]
        L.or_ntot.argtypes = [P, I]
        L.or_nghost.argtypes = [P, I]
        L.or_grid.restype = DP
        L.or_grid.argtypes = [P, I, I]
        L.or_init_blast.argtypes = [P, D, D, D, D, ctypes.c_long]
        L.or_run.argtypes = [P, I]
        L.or_time.argtypes = [P, DP, DP, ctypes.POINTER(ctypes.c_long)]
        L.or_set_time.argtypes = [P, D, D, ctypes.c_long]
        L.or_history.argtypes = [P, DP, DP, I]
        L.or_init_wind.argtypes = [P]
        L.or_wind_reset.argtypes = [P]
        L.or_set_flux.argtypes = [P, I, DP, DP, DP]
        L.or_set_mfit.argtypes = [P, I, DP, DP]
        L.or_cooling.argtypes = [P, D, D]
        L.or_blondin_point.restype = D
        L.or_blondin_point.argtypes = [D, D, D, D, D, D]
        L.or_set_sirocco.argtypes = [P, DP, DP, DP]
        L.or_sirocco_xi.restype = DP
        L.or_sirocco_xi.argtypes = [P]
        _lib = L
    return _lib


# Parameters of the line-driven disk-wind configuration (the [Parameters]
# block of oracle/ref_cfg/wind2d/pluto.ini and the units of its
# definitions.h).
WIND = dict(mu=0.6, rho_0=1.0e-9, cent_mass=1.4e34, t_iso=4.0e4, l_star=1.0e37, f_x=1.0,
            f_uv=1.0, t_x=5.6e7, krad=0.2, alpharad=-0.6, dfloor=1.0e-20,
            unit_density=1e-14, unit_length=1e9, unit_velocity=1e9)
WIND_GRID = dict(xbeg=(10.0, 0.0, 0.0), xend=(1000.0, 1.5707963267948966, 1.0),
                 gridtype=("log", "uniform", "uniform"))
NANGLES = 36


MFIT_POINTS = 21


def synthetic_mfit(x1, x2, ntot, ngh=2, npoints=MFIT_POINTS):
    """Synthetic force-multiplier table in the form M_UV_data.dat holds it
    (read_sirocco_fluxes with KRAD = ALPHARAD = 999): t at npoints, log-spaced
    1e-6..1e4, and per active cell M(t) = k t^a with k and a varying smoothly
    over the grid; values rounded through 13 significant digits as the text
    file carries them.  Returns t [npoints] and M [npoints][k][j][i] over the
    total box (ghost cells 1)."""
    import math
    t = np.array([float("%.12e" % 10.0 ** (-6.0 + 10.0 * n / (npoints - 1)))
                  for n in range(npoints)])
    m = np.ones((npoints, ntot[2], ntot[1], ntot[0]))
    for j in range(ngh, ntot[1] - ngh):
        for i in range(ngh, ntot[0] - ngh):
            k = 0.2 * (1.0 + 0.3 * math.sin(2.0 * x2[j]))
            a = -0.6 + 0.05 * math.cos(x2[j]) * math.log10(x1[i] / 10.0)
            for n in range(npoints):
                m[n, :, j, i] = float("%.12e" % (k * t[n] ** a))
    return t, m


def dense_flux_bins(theta, f0, na=NANGLES):
    """The dense synthetic flux of one cell at polar angle theta with
    L_UV/(4 pi r^2) = f0: every bin a carries f0 w(d) at the angle
    d 2pi/na from the radial bin a0 (d = a - a0), w = 1 at d = 0 and
    0.05/(1 + |d|) elsewhere, split into (F_r, F_theta) = (cos, sin) of that
    angle; values rounded through 13 significant digits."""
    import math
    a0 = int(math.floor(theta / (2 * 3.14159265358979 / 36)))
    fr, ft = [], []
    for a in range(na):
        d = a - a0
        w = 1.0 if d == 0 else 0.05 / (1.0 + abs(d))
        ang = d * (2.0 * math.pi / na)
        fr.append(float("%.12e" % (f0 * w * math.cos(ang))))
        ft.append(float("%.12e" % (f0 * w * math.sin(ang))))
    return fr, ft


def synthetic_flux(x1, x2, ntot, l_uv=1.0e37, unit_length=1e9, na=NANGLES, ngh=2, dense=False):
    """Synthetic directional UV flux: L_UV/(4 pi r^2) in the angle bin that
    contains the radial direction of each active cell, zero elsewhere; the
    values are rounded through the 13-significant-digit text of the
    directional_flux_*.dat files the reference reads.  dense: every bin
    carries flux instead (dense_flux_bins).  Arrays are [angle][k][j][i]
    over the total box (ghost cells zero)."""
    import math
    fr = np.zeros((na, ntot[2], ntot[1], ntot[0]))
    ft = np.zeros_like(fr)
    for j in range(ngh, ntot[1] - ngh):
        a = int(math.floor(x2[j] / (2 * 3.14159265358979 / 36)))
        for i in range(ngh, ntot[0] - ngh):
            r = x1[i] * unit_length
            if dense:
                bfr, bft = dense_flux_bins(x2[j], l_uv / (4 * math.pi * r * r), na)
                fr[:, :, j, i] = np.array(bfr)[:, None]
                ft[:, :, j, i] = np.array(bft)[:, None]
            else:
                fr[a, :, j, i] = float("%.12e" % (l_uv / (4 * math.pi * r * r)))
    return fr, ft, np.zeros_like(fr)


class Oracle:
    def __init__(self, dims=2, nx=(64, 64, 1), nvar=5, limiter="mc", solver="hllc",
                 bc="outflow", gamma=5.0 / 3.0, cfl=0.4, cfl_max_var=1.1, tstop=10.0,
                 first_dt=1e-4, cooling=0, geometry=0, gridtype=("uniform",) * 3,
                 xbeg=(0.0, 0.0, 0.0), xend=(1.0, 1.0, 1.0), body_force=0, line_force=0,
                 floors=0, params=None, char_limiting=0, shock_flattening=0, entropy_switch=0):
        c = OrConfig()
        c.dims = dims
        n = list(nx) + [1] * (3 - len(nx))
        c.nx[:] = n[:3]
        c.nvar = nvar
        c.geometry = geometry
        c.limiter = LIM[limiter]
        c.solver = SOLVER[solver]
        bcs = [bc] * 6 if isinstance(bc, str) else list(bc)
        c.bc[:] = [BC[b] for b in bcs]
        c.gridtype[:] = [{"uniform": 0, "log": 1, "ratio": 2}[g] for g in gridtype]
        c.xbeg[:] = list(xbeg)
        c.xend[:] = list(xend)
        c.ratio[:] = [1.0, 1.0, 1.0]
        c.gamma = gamma
        c.cfl = cfl
        c.cfl_max_var = cfl_max_var
        c.tstop = tstop
        c.first_dt = first_dt
        c.cooling = cooling
        c.body_force, c.line_force, c.floors = body_force, line_force, floors
        c.char_limiting = char_limiting
        c.shock_flattening = shock_flattening
        c.entropy_switch = entropy_switch
        for k, v in (params or {}).items():
            setattr(c, k, v)
        self.cfg = c
        self.nvar = nvar
        self.dims = dims
        self.s = lib().or_create(ctypes.byref(c))
        self.ntot = [lib().or_ntot(self.s, d) for d in range(3)]
        self.ngh = [lib().or_nghost(self.s, d) for d in range(3)]

    def __del__(self):
        try:
            if self.s:
                lib().or_destroy(self.s)
                self.s = None
        except Exception:
            pass

    @property
    def V(self):
        n = self.nvar * self.ntot[0] * self.ntot[1] * self.ntot[2]
        a = np.ctypeslib.as_array(lib().or_state(self.s), shape=(n,))
        return a.reshape(self.nvar, self.ntot[2], self.ntot[1], self.ntot[0])

    def grid(self, d, which=0):
        a = np.ctypeslib.as_array(lib().or_grid(self.s, d, which), shape=(self.ntot[d],))
        return a.copy()

    def init_blast(self, p_amb=0.1, p_in=10.0, r_in=0.1, noise=0.01, seed=1):
        lib().or_init_blast(self.s, p_amb, p_in, r_in, noise, seed)

    def run(self, nsteps):
        return lib().or_run(self.s, nsteps)

    def init_wind(self):
        lib().or_init_wind(self.s)

    def set_flux(self, fr, ft, fp):
        fr, ft, fp = (np.ascontiguousarray(a, dtype=np.float64) for a in (fr, ft, fp))
        self._flux = (fr, ft, fp)
        dp = ctypes.POINTER(ctypes.c_double)
        lib().or_set_flux(self.s, fr.shape[0], fr.ctypes.data_as(dp), ft.ctypes.data_as(dp),
                          fp.ctypes.data_as(dp))

    def set_mfit(self, t, m):
        """Tabulated force multiplier: t [npoints], M [npoints][k][j][i]."""
        t, m = (np.ascontiguousarray(a, dtype=np.float64) for a in (t, m))
        dp = ctypes.POINTER(ctypes.c_double)
        lib().or_set_mfit(self.s, len(t), t.ctypes.data_as(dp), m.ctypes.data_as(dp))

    def set_sirocco(self, xi=None, t_r=None, pre=None):
        """Per-cell sirocco_xi, sirocco_t_r and prefactors (6 arrays, file
        order), each over the total box."""
        dp = ctypes.POINTER(ctypes.c_double)
        keep = [None if a is None else np.ascontiguousarray(a, dtype=np.float64)
                for a in (xi, t_r, pre)]
        lib().or_set_sirocco(self.s, *[None if a is None else a.ctypes.data_as(dp) for a in keep])

    def cooling(self, dt, t):
        lib().or_cooling(self.s, dt, t)

    def time(self):
        t, dt = ctypes.c_double(), ctypes.c_double()
        st = ctypes.c_long()
        lib().or_time(self.s, ctypes.byref(t), ctypes.byref(dt), ctypes.byref(st))
        return t.value, dt.value, st.value

    def history(self, n):
        a, b = np.zeros(n), np.zeros(n)
        k = lib().or_history(self.s, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                             b.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), n)
        return a[:k], b[:k]

    def active(self, V=None):
        """Active-cell view [nv, (k,) j, i] as written to .dbl files."""
        V = self.V if V is None else V
        g = [self.ngh[d] for d in range(3)]
        a = V[:, g[2]:self.ntot[2] - g[2], g[1]:self.ntot[1] - g[1], g[0]:self.ntot[0] - g[0]]
        return a[:, 0] if self.dims == 2 else a


WIND_BC = ["userdef", "outflow", "axisymmetric", "reflective", "outflow", "outflow"]
# the production problem (Test_Problems/LineDrivenWind/cv_idl): X2-beg is
# its hybrid user side (pluto_sirocco_sub.py:78-81)
CVIDL_BC = ["userdef", "outflow", "userdef", "reflective", "outflow", "outflow"]


def wind_oracle(nr=64, nt=32, cooling=1, line_force=1, cfl=0.4, first_dt=1e-4, char_limiting=0,
                shock_flattening=0, solver="hll", entropy_switch=0, mfit=False, ode_cooling=0,
                dense_flux=False, bc=None, initial=None, **params):
    """The 2-D spherical line-driven disk wind (PLM van Leer, HLL, RK2,
    userdef/outflow/axisymmetric/reflective boundaries, point-mass gravity,
    floors, BLONDIN cooling and the line force), initialised.  mfit: the
    tabulated force multiplier (KRAD = ALPHARAD = 999, synthetic table).
    bc: the six boundary codes (default WIND_BC).  initial: active-cell
    state [nv][j][i] to start from instead of this problem's Init (the
    reference's own first snapshot of another problem)."""
    if mfit:
        params = dict(params, krad=999.0, alpharad=999.0)
    o = Oracle(dims=2, nx=(nr, nt, 1), nvar=7 if entropy_switch else 6, limiter="vl",
               solver=solver,
               bc=bc or WIND_BC,
               cfl=cfl, cfl_max_var=1.1, tstop=1e10, first_dt=first_dt,
               cooling=2 if (cooling and ode_cooling) else cooling, geometry=3, gridtype=WIND_GRID["gridtype"], xbeg=WIND_GRID["xbeg"],
               xend=WIND_GRID["xend"], body_force=1, line_force=line_force, floors=1,
               params=dict(WIND, **params), char_limiting=char_limiting,
               shock_flattening=shock_flattening, entropy_switch=entropy_switch)
    if line_force:
        prm = dict(WIND, **params)
        o.set_flux(*synthetic_flux(o.grid(0), o.grid(1), o.ntot,
                                   l_uv=prm["l_star"] * prm["f_uv"], ngh=o.ngh[0],
                                   dense=dense_flux))
    if mfit:   # KRAD = ALPHARAD = 999: the tabulated force multiplier
        o.set_mfit(*synthetic_mfit(o.grid(0), o.grid(1), o.ntot, ngh=o.ngh[0]))
    o.init_wind()
    if initial is not None:
        g = o.ngh[0]
        init = np.asarray(initial)
        o.V[:init.shape[0], 0, g:-g, g:-g] = init
        lib().or_wind_reset(o.s)
    return o


def blondin_points(tuples, tx=5.6e7, mu=0.6):
    """BLONDIN T_new for rows (n_H, T, xi, dt_seconds) (or_blondin_point)."""
    L = lib()
    return np.array([L.or_blondin_point(float(r[0]), float(r[1]), float(r[2]), tx, float(r[3]), mu)
                     for r in np.asarray(tuples, dtype=np.float64)])
