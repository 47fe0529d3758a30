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
                ("cooling", ctypes.c_int)]


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
        L.or_grid.restype = DP
        L.or_grid.argtypes = [P, I, I]
        L.or_init_blast.argtypes = [P, D, D, D, D, ctypes.c_long]
        L.or_run.argtypes = [P, I]
        L.or_time.argtypes = [P, DP, DP, ctypes.POINTER(ctypes.c_long)]
        L.or_set_time.argtypes = [P, D, D, ctypes.c_long]
        L.or_history.argtypes = [P, DP, DP, I]
        _lib = L
    return _lib


class Oracle:
    def __init__(self, dims=2, nx=(64, 64, 1), nvar=5, limiter="mc", solver="hllc",
                 bc="outflow", gamma=5.0 / 3.0, cfl=0.4, cfl_max_var=1.1, tstop=10.0,
                 first_dt=1e-4, cooling=0):
        c = OrConfig()
        c.dims = dims
        n = list(nx) + [1] * (3 - len(nx))
        c.nx[:] = n[:3]
        c.nvar = nvar
        c.geometry = 0
        c.limiter = LIM[limiter]
        c.solver = SOLVER[solver]
        bcs = [bc] * 6 if isinstance(bc, str) else list(bc)
        c.bc[:] = [BC[b] for b in bcs]
        c.gridtype[:] = [0, 0, 0]
        c.xbeg[:] = [0.0, 0.0, 0.0]
        c.xend[:] = [1.0, 1.0, 1.0]
        c.ratio[:] = [1.0, 1.0, 1.0]
        c.gamma = gamma
        c.cfl = cfl
        c.cfl_max_var = cfl_max_var
        c.tstop = tstop
        c.first_dt = first_dt
        c.cooling = cooling
        self.cfg = c
        self.nvar = nvar
        self.dims = dims
        self.s = lib().or_create(ctypes.byref(c))
        self.ntot = [lib().or_ntot(self.s, d) for d in range(3)]

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
        g = [2 if d < self.dims else 0 for d in range(3)]
        a = V[:, g[2]:self.ntot[2] - g[2], g[1]:self.ntot[1] - g[1], g[0]:self.ntot[0] - g[0]]
        return a[:, 0] if self.dims == 2 else a
