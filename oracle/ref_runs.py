"""Runs of the reference's own serial CPU build (oracle/_ref/<cfg>/pluto,
built by oracle/ref.mk) on the synthetic configurations, with their step
loops timed.

TEST INFRASTRUCTURE ONLY: used by bench.py's reference arm (and the golden
generator's input files).  The product never imports it.

Each run gets a directory with its pluto.ini and, for the wind, the
directional_flux_*.dat files read_sirocco_fluxes reads (written by
liboracle's or_write_wind_flux from the oracle's own grid).  The binary runs
with `-maxsteps W+K-1 -no-write` and `log 1`, its standard output on a
pseudo-terminal so that the C library flushes every line: the "step:W;"
line that OutputLogPre prints when step W starts (Src/output_log.c:34) and
the "> Total allocated memory" line printed after the main loop
(Src/main.c:346-352) bracket the last K steps, i.e. the step loop without
the set-up (whose read_sirocco_fluxes matches every record against every
cell).
"""
import ctypes
import os
import select
import shutil
import subprocess
import threading
import time

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")

WIND_INI = """[Grid]

X1-grid    1    10.0   {nr}    l+   1000.0
X2-grid    1    0.0    {nt}    u    1.5707963267948966
X3-grid    1    0.0    1     u    1.0

[Time]

CFL              0.4
CFL_max_var      1.1
tstop            1.e10
first_dt         1.e-4

[Solver]

Solver         {solver}

[Boundary]

X1-beg        userdef
X1-end        outflow
X2-beg        axisymmetric
X2-end        reflective
X3-beg        outflow
X3-end        outflow

[Static Grid Output]

uservar    0
dbl       -1.0  {every}   single_file
flt       -1.0  -1   single_file
vtk       -1.0  -1   single_file
dbl.h5    -1.0  -1
flt.h5    -1.0  -1
tab       -1.0  -1
ppm       -1.0  -1
png       -1.0  -1
log        {log}
analysis  -1.0  -1

[Parameters]

MU                          0.6
RHO_0                       1.0e-9
R_0                         1.0e10
RHO_ALPHA                   1.5
CENT_MASS                   1.4e34
DISK_MDOT                   1.0e-8
T_ISO                       4.0e4
L_star                      {l_star}
f_x                         1.0
f_uv                        1.0
T_x                         5.6e7
KRAD                        {krad}
ALPHARAD                    {alpharad}
DFLOOR                      1.0e-20
GAMMA                       1.6666666666666667
"""

BLAST_INI = """[Grid]

X1-grid    1    0.0    {nx}    u    1.0
X2-grid    1    0.0    {ny}    u    1.0
X3-grid    1    0.0    {nz}    u    1.0

[Time]

CFL              {cfl}
CFL_max_var      1.1
tstop            {tstop}
first_dt         1.e-4

[Solver]

Solver         {solver}

[Boundary]

X1-beg        {bc}
X1-end        {bc}
X2-beg        {bc}
X2-end        {bc}
X3-beg        {bc}
X3-end        {bc}

[Static Grid Output]

uservar    0
dbl       -1.0  {every}   single_file
flt       -1.0  -1   single_file
vtk       -1.0  -1   single_file
dbl.h5    -1.0  -1
flt.h5    -1.0  -1
tab       -1.0  -1
ppm       -1.0  -1
png       -1.0  -1
log        {log}
analysis  -1.0  -1

[Parameters]

P_AMB                       0.1
P_IN                        10.0
R_IN                        0.1
NOISE                       0.01
"""


def binary(cfg):
    """Path of the reference's binary for a configuration, or None."""
    exe = os.path.join(REF_DIR, cfg, "pluto")
    return exe if os.access(exe, os.X_OK) else None


def _num(v):
    """A parameter as the ini file carries it: the shortest text that reads
    back as the same double."""
    return repr(float(v))


FLUX_FILES = ("directional_flux_r.dat", "directional_flux_theta.dat", "directional_flux_phi.dat")


def write_wind_flux(wd, nr, nt, l_star, axes=7):
    """The single-bin synthetic flux files of a wind grid (bit a of axes:
    the file of axis a), written by liboracle from the oracle's grid."""
    import numpy as np
    from oracle import WIND, WIND_GRID, NANGLES, Oracle, lib
    o = Oracle(dims=2, nx=(nr, nt, 1), nvar=6, geometry=3, gridtype=WIND_GRID["gridtype"],
               xbeg=WIND_GRID["xbeg"], xend=WIND_GRID["xend"])
    x1, x2 = (np.ascontiguousarray(o.grid(d)) for d in (0, 1))
    dp = ctypes.POINTER(ctypes.c_double)
    L = lib()
    L.or_write_wind_flux.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, dp, dp,
                                     ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                     ctypes.c_int, ctypes.c_int]
    rc = L.or_write_wind_flux(os.fsencode(wd), nr, nt, x1.ctypes.data_as(dp),
                              x2.ctypes.data_as(dp), o.ngh[0], float(l_star) * WIND["f_uv"],
                              WIND["unit_length"], NANGLES, axes)
    if rc:
        raise OSError("could not write the flux files in " + wd)


def prepare_wind(wd, nr, nt, l_star=1.0e37, krad=0.2, alpharad=-0.6, solver="hll",
                 every=-1, log=1, flux=True, shared=None):
    """pluto.ini (and the single-bin synthetic flux files) of one wind model.
    shared: a directory holding this grid's theta and phi files (all zero
    for the single-bin flux, whatever L_x), linked instead of written."""
    os.makedirs(wd, exist_ok=True)
    with open(os.path.join(wd, "pluto.ini"), "w") as f:
        f.write(WIND_INI.format(nr=nr, nt=nt, every=every, log=log, solver=solver,
                                l_star=_num(l_star), krad=_num(krad), alpharad=_num(alpharad)))
    if not flux:
        return
    if shared:
        # the radial file too when the shared directory holds one (replicas
        # of one model)
        own_r = not os.path.exists(os.path.join(shared, FLUX_FILES[0]))
        for name in FLUX_FILES[1 if own_r else 0:]:
            os.symlink(os.path.join(shared, name), os.path.join(wd, name))
        if own_r:
            write_wind_flux(wd, nr, nt, l_star, axes=1)
    else:
        write_wind_flux(wd, nr, nt, l_star)


def prepare_blast(wd, nx, ny, nz=1, solver="hllc", bc="outflow", cfl=0.4, tstop=10.0,
                  every=-1, log=1):
    os.makedirs(wd, exist_ok=True)
    with open(os.path.join(wd, "pluto.ini"), "w") as f:
        f.write(BLAST_INI.format(nx=nx, ny=ny, nz=nz, cfl=cfl, tstop=tstop, solver=solver,
                                 bc=bc, every=every, log=log))


def run_timed(exe, wd, steps, skip, timeout=3600.0):
    """Runs `steps` steps (0 .. steps-1) of the reference in wd and returns
    (seconds from the start of step `skip` to the end of the main loop,
    exit code, total wall seconds).  The process's standard output goes to a
    pseudo-terminal (line-buffered) and is read as it comes."""
    import pty
    master, slave = pty.openpty()
    t0 = time.perf_counter()
    p = subprocess.Popen([exe, "-maxsteps", str(steps - 1), "-no-write"], cwd=wd,
                         stdin=subprocess.DEVNULL, stdout=slave, stderr=slave, close_fds=True)
    os.close(slave)
    mark = ("step:%d;" % skip).encode()
    t_skip = t_end = None
    pending = b""
    log = open(os.path.join(wd, "run.log"), "wb")
    try:
        while True:
            if time.perf_counter() - t0 > timeout:
                p.kill()
                break
            r, _, _ = select.select([master], [], [], 0.5)
            if not r:
                if p.poll() is not None:
                    break
                continue
            try:
                chunk = os.read(master, 1 << 16)
            except OSError:   # the pty reports EIO once the child has closed it
                chunk = b""
            if not chunk:
                break
            now = time.perf_counter()
            log.write(chunk)
            pending += chunk
            while b"\n" in pending:
                line, pending = pending.split(b"\n", 1)
                line = line.strip()
                if t_skip is None and line.startswith(mark):
                    t_skip = now
                elif line.startswith(b"> Total allocated memory"):
                    t_end = now
    finally:
        rc = p.wait()
        os.close(master)
        log.close()
    wall = time.perf_counter() - t0
    if t_skip is None or t_end is None:
        return None, rc if rc else -1, wall
    return t_end - t_skip, rc, wall


def run_many(jobs, workers):
    """jobs: (prepare, exe, wd, steps, skip, cells) tuples; at most `workers`
    reference processes at a time, the largest first; each job's directory
    is made by prepare() just before its run and removed after it.  Returns
    the per-job (timed seconds, rc, wall) in the order given and the wall
    time of all."""
    order = sorted(range(len(jobs)), key=lambda k: -jobs[k][5])
    res = [None] * len(jobs)
    lock = threading.Lock()
    nxt = [0]

    def worker():
        while True:
            with lock:
                if nxt[0] >= len(order):
                    return
                k = order[nxt[0]]
                nxt[0] += 1
            prepare, exe, wd, steps, skip, _ = jobs[k]
            try:
                prepare()
                res[k] = run_timed(exe, wd, steps, skip)
            except Exception as e:   # reported as a failed run
                res[k] = (None, repr(e), 0.0)
            finally:
                clean(wd)

    t0 = time.perf_counter()
    th = [threading.Thread(target=worker) for _ in range(max(1, workers))]
    for t in th:
        t.start()
    for t in th:
        t.join()
    return res, time.perf_counter() - t0


def clean(wd):
    shutil.rmtree(wd, ignore_errors=True)
