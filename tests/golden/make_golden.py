"""Generate the golden vectors under tests/golden/ from the reference's own
serial CPU build (oracle/ref.mk -> oracle/_ref/<cfg>/pluto).

Runs only where the reference sources are present (they are read by
oracle/ref.mk); the resulting .npz/.json files are committed so that the
tests never need the reference at run time.

    python tests/golden/make_golden.py [--ref /path/to/reference]

Each case writes a pluto.ini (grid, solver, boundaries, output cadence),
runs `pluto -maxsteps N-1` (steps 0..N-1, i.e. N steps; the final snapshot
is written when the step counter reaches N), and stores the initial and
final primitive state as read from the .dbl files (raw little-endian
float64, one block per variable over the active cells).
"""
import argparse
import hashlib
import json
import os
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
ORACLE = os.path.join(ROOT, "oracle")

INI = """[Grid]

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
dbl       -1.0  {nsteps}   single_file
flt       -1.0  -1   single_file
vtk       -1.0  -1   single_file
dbl.h5    -1.0  -1
flt.h5    -1.0  -1
tab       -1.0  -1
ppm       -1.0  -1
png       -1.0  -1
log        {nsteps}
analysis  -1.0  -1

[Parameters]

P_AMB                       0.1
P_IN                        10.0
R_IN                        0.1
NOISE                       0.01
"""

# name, ref config dir, dims, (nx, ny, nz), solver, boundary, steps, store_full
CASES = [
    ("blast2d_mc_hllc_outflow_64x64", "blast2d", 2, (64, 64, 1), "hllc", "outflow", 50, True),
    ("blast2d_mc_hll_periodic_48x40", "blast2d", 2, (48, 40, 1), "hll", "periodic", 40, True),
    ("blast2d_vl_hllc_reflective_40x56", "blast2d_vl", 2, (40, 56, 1), "hllc", "reflective", 30, True),
    ("blast3d_mc_hllc_periodic_16x16x16", "blast3d", 3, (16, 16, 16), "hllc", "periodic", 20, True),
    ("blast3d_mc_hll_outflow_12x20x8", "blast3d", 3, (12, 20, 8), "hll", "outflow", 15, True),
    # full-size configuration: only a digest of the final state is stored
    ("blast2d_mc_hllc_outflow_256x256", "blast2d", 2, (256, 256, 1), "hllc", "outflow", 100, False),
]


def read_dbl(path, dims, n):
    nx, ny, nz = n
    a = np.fromfile(path, dtype="<f8")
    return a.reshape(5, nz, ny, nx) if dims == 3 else a.reshape(5, ny, nx)


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def run_case(ref, name, cfg, dims, n, solver, bc, steps, full):
    subprocess.run(["make", "-s", "-f", os.path.join(ORACLE, "ref.mk"), f"CFG={cfg}",
                    f"REF={ref}", "-j8"], check=True)
    exe = os.path.join(ORACLE, "_ref", cfg, "pluto")
    wd = os.path.join(ORACLE, "_ref", "runs", name)
    shutil.rmtree(wd, ignore_errors=True)
    os.makedirs(wd)
    with open(os.path.join(wd, "pluto.ini"), "w") as f:
        f.write(INI.format(nx=n[0], ny=n[1], nz=n[2], cfl=0.4 if dims == 2 else 0.3,
                           tstop=10.0, solver=solver, bc=bc, nsteps=steps))
    subprocess.run([exe, "-maxsteps", str(steps - 1)], cwd=wd, check=True,
                   stdout=subprocess.DEVNULL)
    v0 = read_dbl(os.path.join(wd, "data.0000.dbl"), dims, n)
    v1 = read_dbl(os.path.join(wd, "data.0001.dbl"), dims, n)
    lines = open(os.path.join(wd, "dbl.out")).read().split("\n")
    t_s, dt_s = lines[1].split()[1], lines[1].split()[2]
    meta = dict(name=name, ref_config=cfg, dims=dims, n=list(n), solver=solver, bc=bc,
                steps=steps, limiter="vl" if cfg.endswith("_vl") else "mc",
                cfl=0.4 if dims == 2 else 0.3, cfl_max_var=1.1, tstop=10.0, first_dt=1e-4,
                gamma="5/3", p_amb=0.1, p_in=10.0, r_in=0.1, noise=0.01, seed=1,
                t_final=t_s, dt_next=dt_s, ic_sha256=digest(v0), final_sha256=digest(v1),
                final_sums=[float(x) for x in v1.reshape(5, -1).sum(axis=1)])
    if full:
        np.savez_compressed(os.path.join(HERE, name + ".npz"), v0=v0, v1=v1)
    with open(os.path.join(HERE, name + ".json"), "w") as f:
        json.dump(meta, f, indent=1)
    print(name, "t =", t_s, "dt =", dt_s)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    args = ap.parse_args()
    if not os.path.isdir(os.path.join(args.ref, "Src")):
        sys.exit("reference sources not found at " + args.ref)
    for c in CASES:
        run_case(args.ref, *c)


if __name__ == "__main__":
    main()
