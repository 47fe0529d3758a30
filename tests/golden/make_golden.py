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
sys.path.insert(0, ORACLE)
sys.path.insert(0, os.path.join(ROOT, "pluto-sirocco_gb300"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

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
log        {every}
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


DBL_FIXTURES = ("blast2d_mc_hll_periodic_48x40",)


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
    if name in DBL_FIXTURES:
        # the reference's own output files, kept verbatim for the .dbl
        # reader/writer tests
        shutil.copyfile(os.path.join(wd, "data.0001.dbl"), os.path.join(HERE, name + ".dbl"))
        shutil.copyfile(os.path.join(wd, "dbl.out"), os.path.join(HERE, name + ".dbl.out"))
    with open(os.path.join(HERE, name + ".json"), "w") as f:
        json.dump(meta, f, indent=1)
    print(name, "t =", t_s, "dt =", dt_s)


def write_flux_files(wd, nr, nt, dense=False, l_uv=1.0e37):
    """directional_flux_{r,theta,phi}.dat in the format read by
    read_sirocco_fluxes (Src/LineDriven/line_connect.c:84-165): two header
    lines (the second holds the angle count as its third token), then one
    row per active cell: i j k r[cm] theta[rad] F_0 .. F_35.  dense: flux in
    every bin (oracle.dense_flux_bins).  l_uv = L_star f_uv."""
    import psgb
    from oracle import synthetic_flux, NANGLES, WIND
    x1 = psgb.build_grid(nr, 2, 10.0, 1000.0, "log")[0]
    x2 = psgb.build_grid(nt, 2, 0.0, 1.5707963267948966, "uniform")[0]
    fl = synthetic_flux(x1, x2, (nr + 4, nt + 4, 1), dense=dense, l_uv=l_uv)
    for ax, name in enumerate(("r", "theta", "phi")):
        with open(os.path.join(wd, f"directional_flux_{name}.dat"), "w") as f:
            f.write("# synthetic directional UV flux\n")
            f.write(f"# nangles {NANGLES}\n")
            for j in range(2, nt + 2):
                for i in range(2, nr + 2):
                    vals = " ".join("%.12e" % v for v in fl[ax][:, 0, j, i])
                    f.write(f"{i - 2} {j - 2} 0 {x1[i] * WIND['unit_length']:.12e} "
                            f"{x2[j]:.12e} {vals}\n")


def write_mfit_file(wd, nr, nt):
    """M_UV_data.dat in the layout read_sirocco_fluxes reads with KRAD =
    ALPHARAD = 999 (Src/LineDriven/line_connect.c:182-257): a header line
    whose second token is the number of points, a word followed by the t
    values, then one row per active cell: i j r[cm] theta[rad] M_0 .. M_n."""
    import psgb
    from oracle import synthetic_mfit, WIND
    x1 = psgb.build_grid(nr, 2, 10.0, 1000.0, "log")[0]
    x2 = psgb.build_grid(nt, 2, 0.0, 1.5707963267948966, "uniform")[0]
    t, m = synthetic_mfit(x1, x2, (nr + 4, nt + 4, 1))
    with open(os.path.join(wd, "M_UV_data.dat"), "w") as f:
        f.write(f"npoints {len(t)}\n")
        f.write("t " + " ".join("%.12e" % v for v in t) + "\n")
        for j in range(2, nt + 2):
            for i in range(2, nr + 2):
                vals = " ".join("%.12e" % v for v in m[:, 0, j, i])
                f.write(f"{i - 2} {j - 2} {x1[i] * WIND['unit_length']:.12e} {x2[j]:.12e} {vals}\n")


# The production disk-wind problem's own setup (cv_idl/init.c and
# definitions.h, compiled where they lie): its boundaries (X1-beg userdef,
# X1-end outflow, X2-beg userdef, X2-end reflective, as
# Test_Problems/LineDrivenWind/cv_idl/pluto_sirocco_sub.py:78-81 writes them)
# and an accretion rate that gives its Init a disk of 1e4..2e4 K.
CVIDL_INI = (WIND_INI.replace("X2-beg        axisymmetric", "X2-beg        userdef")
             .replace("DISK_MDOT                   1.0e-8", "DISK_MDOT                   1.0e17"))

# name, ref config, (nr, nt), steps, snapshot every, with flux files, and
# the numerics switches of the ref config's definitions.h / pluto.ini
WIND_CASES = [
    ("wind2d_full_64x32", "wind2d", (64, 32), 200, 20, True, {}),
    ("wind2d_hydro_64x32", "wind2d_hydro", (64, 32), 100, 20, False, {}),
    ("wind2d_char_64x32", "wind2d_char", (64, 32), 100, 20, False, dict(char_limiting=1)),
    ("wind2d_multid_64x32", "wind2d_multid", (64, 32), 100, 20, False,
     dict(char_limiting=1, shock_flattening=1)),
    ("wind2d_multid_hllc_64x32", "wind2d_multid_hllc", (64, 32), 100, 20, False,
     dict(shock_flattening=1, solver="hllc")),
    ("wind2d_entsel_64x32", "wind2d_entsel", (64, 32), 100, 20, False,
     dict(entropy_switch=1)),
    ("wind2d_idl_hydro_64x32", "wind2d_idl_hydro", (64, 32), 100, 20, False,
     dict(char_limiting=1, shock_flattening=1, entropy_switch=2)),
    ("wind2d_idl_64x32", "wind2d_idl", (64, 32), 200, 20, True,
     dict(char_limiting=1, shock_flattening=1, entropy_switch=2)),
    ("wind2d_mfit_64x32", "wind2d", (64, 32), 100, 20, True, dict(mfit=True)),
    ("wind2d_ode_64x32", "wind2d_ode", (64, 32), 100, 20, True, dict(ode_cooling=1)),
    ("wind2d_dense_64x32", "wind2d", (64, 32), 100, 20, True, dict(dense_flux=1)),
    ("wind2d_cvidl_64x32", "wind2d_cvidl", (64, 32), 100, 20, True,
     dict(char_limiting=1, shock_flattening=1, entropy_switch=2, cvidl=1)),
]


def run_wind_case(ref, name, cfg, n, steps, every, flux, opts):
    subprocess.run(["make", "-s", "-f", os.path.join(ORACLE, "ref.mk"), f"CFG={cfg}",
                    f"REF={ref}", "-j8"], check=True)
    exe = os.path.join(ORACLE, "_ref", cfg, "pluto")
    wd = os.path.join(ORACLE, "_ref", "runs", name)
    shutil.rmtree(wd, ignore_errors=True)
    os.makedirs(wd)
    with open(os.path.join(wd, "pluto.ini"), "w") as f:
        mfit = opts.get("mfit", False)
        f.write((CVIDL_INI if opts.get("cvidl") else WIND_INI).format(nr=n[0], nt=n[1], every=every,
                                solver=opts.get("solver", "hll"), l_star="1.0e37",
                                krad=999 if mfit else 0.2, alpharad=999 if mfit else -0.6))
    if flux:
        write_flux_files(wd, n[0], n[1], dense=bool(opts.get("dense_flux", 0)))
    if opts.get("mfit"):
        write_mfit_file(wd, n[0], n[1])
    subprocess.run([exe, "-maxsteps", str(steps - 1)], cwd=wd, check=True,
                   stdout=subprocess.DEVNULL)
    snaps = []
    for k in range(steps // every + 1):
        a = np.fromfile(os.path.join(wd, f"data.{k:04d}.dbl"), dtype="<f8")
        # the entropy variable of ENTROPY_SWITCH is not written (set_output.c:177-179)
        snaps.append(a.reshape(6, n[1], n[0]))
    lines = [l.split() for l in open(os.path.join(wd, "dbl.out")).read().split("\n") if l]
    keep = sorted({0, 1, len(snaps) // 2, len(snaps) - 1})
    meta = dict(name=name, ref_config=cfg, kind="wind", dims=2, n=[n[0], n[1], 1],
                steps=steps, snap_steps=[k * every for k in keep], cooling=int(flux),
                line_force=int(flux), char_limiting=opts.get("char_limiting", 0),
                shock_flattening=opts.get("shock_flattening", 0),
                entropy_switch=opts.get("entropy_switch", 0), mfit=int(opts.get("mfit", 0)),
                ode_cooling=opts.get("ode_cooling", 0), dense_flux=opts.get("dense_flux", 0),
                cvidl=opts.get("cvidl", 0),
                solver=opts.get("solver", "hll"),
                t=[lines[k][1] for k in keep],
                dt=[lines[k][2] for k in keep], final_sha256=digest(snaps[-1]))
    snaps = np.stack([snaps[k] for k in keep])
    np.savez_compressed(os.path.join(HERE, name + ".npz"), snaps=snaps)
    with open(os.path.join(HERE, name + ".json"), "w") as f:
        json.dump(meta, f, indent=1)
    print(name, "t =", meta["t"][-1])


def batch_probe_models():
    """The first model of each grid size in the 64-model batch (seed 4):
    (index, spec) pairs, smallest grid first."""
    import psgb
    specs = psgb.batch_models(64, seed=4)
    seen, out = set(), []
    for m, sp in enumerate(specs):
        if sp["grid"] not in seen:
            seen.add(sp["grid"])
            out.append((m, sp))
    return sorted(out, key=lambda e: e[1]["grid"][0])


def wind_full_cases():
    """Digest-only wind cases at full size: the 512 x 256 wind with every
    term on and hydro only (gravity, geometry, boundaries), 100 steps each,
    and one model of each grid size of the 64-model batch (its own L_x, k
    and alpha) for 20 steps."""
    prm = dict(l_star=1.0e37, krad=0.2, alpharad=-0.6)
    cases = [("wind2d_full_512x256", "wind2d", (512, 256), 100, prm, None),
             ("wind2d_hydro_512x256", "wind2d_hydro", (512, 256), 100, prm, None)]
    for m, sp in batch_probe_models():
        cases.append(("wind2d_batch_m%02d_%dx%d" % ((m,) + sp["grid"]), "wind2d", sp["grid"], 20,
                      dict(l_star=sp["l_star"], krad=sp["krad"], alpharad=sp["alpharad"]), m))
    return cases


def oracle_sensitivity(meta, seeds=(1, 2), eps=1e-15):
    """How far the reference's own algorithm (the oracle, bit-identical to
    it) moves when its initial state is perturbed by relative noise of
    1e-15: the relative L1 per variable between the perturbed and the
    unperturbed run after the case's steps, the largest over the seeds.
    Device results whose distance from the reference is of this size are
    indistinguishable from rounding."""
    from conftest import rel_l1
    from oracle import wind_oracle
    full = meta["ref_config"] == "wind2d"
    kw = dict(cooling=int(full), line_force=int(full), l_star=meta["l_star"], krad=meta["krad"],
              alpharad=meta["alpharad"])
    nr, nt = meta["n"][0], meta["n"][1]
    base = wind_oracle(nr, nt, **kw)
    base.run(meta["steps"])
    worst = np.zeros(6)
    for seed in seeds:
        o = wind_oracle(nr, nt, **kw)
        rng = np.random.default_rng(seed)
        V = o.V
        V[...] = V * (1.0 + eps * rng.standard_normal(V.shape))
        o.run(meta["steps"])
        worst = np.maximum(worst, rel_l1(o.active(), base.active()))
    return [float(x) for x in worst]


def run_wind_full_case(ref, name, cfg, n, steps, prm, model):
    """The reference on a full-size wind: only the digests, per-variable
    sums, t and dt of the initial and final states are kept (the states
    themselves come from the oracle, pinned by these digests, at test time),
    with the oracle's own sensitivity to 1e-15 perturbations."""
    flux = cfg == "wind2d"
    subprocess.run(["make", "-s", "-f", os.path.join(ORACLE, "ref.mk"), f"CFG={cfg}",
                    f"REF={ref}", "-j8"], check=True)
    exe = os.path.join(ORACLE, "_ref", cfg, "pluto")
    wd = os.path.join(ORACLE, "_ref", "runs", name)
    shutil.rmtree(wd, ignore_errors=True)
    os.makedirs(wd)
    with open(os.path.join(wd, "pluto.ini"), "w") as f:
        f.write(WIND_INI.format(nr=n[0], nt=n[1], every=steps, solver="hll",
                                l_star=repr(float(prm["l_star"])), krad=repr(float(prm["krad"])),
                                alpharad=repr(float(prm["alpharad"]))))
    if flux:
        write_flux_files(wd, n[0], n[1], l_uv=prm["l_star"])
    subprocess.run([exe, "-maxsteps", str(steps - 1)], cwd=wd, check=True,
                   stdout=subprocess.DEVNULL)
    v0 = np.fromfile(os.path.join(wd, "data.0000.dbl"), dtype="<f8").reshape(6, n[1], n[0])
    v1 = np.fromfile(os.path.join(wd, "data.0001.dbl"), dtype="<f8").reshape(6, n[1], n[0])
    lines = [l.split() for l in open(os.path.join(wd, "dbl.out")).read().split("\n") if l]
    meta = dict(name=name, ref_config=cfg, kind="wind_full", dims=2, n=[n[0], n[1], 1],
                steps=steps, batch_model=model, l_star=float(prm["l_star"]),
                krad=float(prm["krad"]), alpharad=float(prm["alpharad"]),
                cooling=int(flux), line_force=int(flux),
                t=[lines[0][1], lines[1][1]], dt=[lines[0][2], lines[1][2]],
                ic_sha256=digest(v0), final_sha256=digest(v1),
                final_sums=[float(x) for x in v1.reshape(6, -1).sum(axis=1)])
    meta["sensitivity_1e-15"] = oracle_sensitivity(meta)
    with open(os.path.join(HERE, name + ".json"), "w") as f:
        json.dump(meta, f, indent=1)
    print(name, "t =", meta["t"][-1], "sensitivity", meta["sensitivity_1e-15"])
    shutil.rmtree(wd, ignore_errors=True)   # the flux files of a full-size grid run to 0.3 GB


def add_sensitivity(name):
    """The oracle sensitivity of an existing full-size case (no reference run)."""
    path = os.path.join(HERE, name + ".json")
    meta = json.load(open(path))
    meta.setdefault("cooling", 1)
    meta.setdefault("line_force", 1)
    meta["sensitivity_1e-15"] = oracle_sensitivity(meta)
    with open(path, "w") as f:
        json.dump(meta, f, indent=1)
    print(name, "sensitivity", meta["sensitivity_1e-15"])


# SIROCCO hand-off data (per-cell xi, radiation temperature and rate
# prefactors) read by the reference at a restart, as the coupling loop hands
# them over (read_sirocco_heatcool with flag 1, Src/LineDriven/
# line_connect.c:307-497); BLONDIN uses them once g_time > 3
# (Src/Cooling/BLONDIN/cooling.c:73-108).
SIROCCO_T0 = 3.5


def sirocco_inputs(nr, nt, seed=2):
    """Seeded xi (1..1e6), T_r (1e6..1e8 K) and the six prefactors
    (0.5..2) of every cell of the total box ([j][i]), before the text
    rounding of the files."""
    n0, n1 = nr + 4, nt + 4
    rng = np.random.default_rng(seed)
    xi = 10 ** rng.uniform(0.0, 6.0, (n1, n0))
    tr = 10 ** rng.uniform(6.0, 8.0, (n1, n0))
    pre = rng.uniform(0.5, 2.0, (6, n1, n0))
    return xi, tr, pre


def sirocco_as_read(nr, nt, seed=2):
    """The data as the reference holds it after reading the files: xi and T_r
    through their 11-digit text with the floors xi >= 1, T_r >= 1e3 K, the
    prefactors through their 16-digit text ([j][i] over the total box)."""
    xi, tr, pre = sirocco_inputs(nr, nt, seed)
    rd = np.vectorize(lambda v, fmt: float(fmt % v))
    return (np.maximum(rd(xi, "%.10e"), 1.0), np.maximum(rd(tr, "%.10e"), 1e3),
            rd(pre, "%.15e"))


def write_sirocco_files(wd, nr, nt, rho, seed=2, unit_length=1e9, unit_density=1e-14):
    """py_heatcool.dat and prefactors.dat in the column layouts the reference
    parses (line_connect.c:336-339 and 428-431); rho: the active cells'
    density [j][i] in code units (the files' density column)."""
    import psgb
    xi, tr, pre = sirocco_inputs(nr, nt, seed)
    x1 = psgb.build_grid(nr, 2, 10.0, 1000.0, "log")[0]
    x2 = psgb.build_grid(nt, 2, 0.0, 1.5707963267948966, "uniform")[0]
    with open(os.path.join(wd, "py_heatcool.dat"), "w") as f:
        f.write("i j rcen thetacen vol temp t_r xi ne heat_xray heat_comp heat_lines heat_ff "
                "cool_comp cool_lines cool_ff rho n_h\n")
        for j in range(2, nt + 2):
            for i in range(2, nr + 2):
                f.write("%d %d %.10e %.10e 1.0 1e4 %.10e %.10e 1 0 0 0 0 0 0 0 %.10e 1e10\n"
                        % (i - 2, j - 2, x1[i] * unit_length, x2[j], tr[j, i], xi[j, i],
                           rho[j - 2, i - 2] * unit_density))
    with open(os.path.join(wd, "prefactors.dat"), "w") as f:
        f.write("i rcen j thetacen dens comp_h comp_c xray_h brem_c line_c xi_ion\n")
        for j in range(2, nt + 2):
            for i in range(2, nr + 2):
                f.write("%d %.10e %d %.10e %.10e %s\n"
                        % (i - 2, x1[i] * unit_length, j - 2, x2[j],
                           rho[j - 2, i - 2] * unit_density,
                           " ".join("%.15e" % v for v in pre[:, j, i])))


def run_sirocco_case(ref, name="wind2d_sirocco_64x32", n=(64, 32), steps=80, every=20, seed=2):
    """The wind restarted at t = 3.5 from its own initial dump with SIROCCO
    data files present: the restart record the reference wrote for the dump
    gets t = 3.5 (Restart, Src/structs.h:256-262: t at byte 72), then
    `pluto -restart 0` reads the files and BLONDIN uses them."""
    import struct
    cfg = "wind2d"
    subprocess.run(["make", "-s", "-f", os.path.join(ORACLE, "ref.mk"), f"CFG={cfg}",
                    f"REF={ref}", "-j8"], check=True)
    exe = os.path.join(ORACLE, "_ref", cfg, "pluto")
    wd = os.path.join(ORACLE, "_ref", "runs", name)
    shutil.rmtree(wd, ignore_errors=True)
    os.makedirs(wd)
    with open(os.path.join(wd, "pluto.ini"), "w") as f:
        f.write(WIND_INI.format(nr=n[0], nt=n[1], every=every, solver="hll", l_star="1.0e37",
                                krad=0.2, alpharad=-0.6))
    write_flux_files(wd, n[0], n[1])
    subprocess.run([exe, "-maxsteps", "0"], cwd=wd, check=True, stdout=subprocess.DEVNULL)
    rec = bytearray(open(os.path.join(wd, "restart.out"), "rb").read())
    assert len(rec) == 128 and struct.unpack("<i", rec[4:8])[0] == 0
    rec[72:80] = struct.pack("<d", SIROCCO_T0)
    open(os.path.join(wd, "restart.out"), "wb").write(bytes(rec))
    v0 = np.fromfile(os.path.join(wd, "data.0000.dbl"), dtype="<f8").reshape(6, n[1], n[0])
    write_sirocco_files(wd, n[0], n[1], v0[0], seed=seed)
    subprocess.run([exe, "-restart", "0", "-maxsteps", str(steps - 1)], cwd=wd, check=True,
                   stdout=subprocess.DEVNULL)
    snaps = [np.fromfile(os.path.join(wd, "data.%04d.dbl" % k), dtype="<f8").reshape(6, n[1], n[0])
             for k in range(steps // every + 1)]
    lines = [l.split() for l in open(os.path.join(wd, "dbl.out")).read().split("\n") if l]
    meta = dict(name=name, ref_config=cfg, kind="wind", dims=2, n=[n[0], n[1], 1], steps=steps,
                snap_steps=[k * every for k in range(len(snaps))], cooling=1, line_force=1,
                sirocco_seed=seed, t0=SIROCCO_T0, solver="hll",
                # the initial dump is the reference's at t = 0; the run restarts it at t0
                t=["%e" % SIROCCO_T0] + [l[1] for l in lines[1:]], dt=[l[2] for l in lines],
                final_sha256=digest(snaps[-1]))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), snaps=np.stack(snaps))
    with open(os.path.join(HERE, name + ".json"), "w") as f:
        json.dump(meta, f, indent=1)
    print(name, "t =", meta["t"][-1])
    shutil.rmtree(wd, ignore_errors=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("PLUTO_REF", "/root/reference"))
    ap.add_argument("--only", default=None)
    ap.add_argument("--sensitivity-only", action="store_true",
                    help="add the oracle's sensitivity to existing full-size cases")
    args = ap.parse_args()
    if args.sensitivity_only:
        for c in wind_full_cases():
            if (args.only is None or args.only in c[0]) and \
                    os.path.exists(os.path.join(HERE, c[0] + ".json")):
                add_sensitivity(c[0])
        return
    if not os.path.isdir(os.path.join(args.ref, "Src")):
        sys.exit("reference sources not found at " + args.ref)
    for c in CASES:
        if args.only is None or args.only in c[0]:
            run_case(args.ref, *c)
    for c in WIND_CASES:
        if args.only is None or args.only in c[0]:
            run_wind_case(args.ref, *c)
    for c in wind_full_cases():
        if args.only is None or args.only in c[0]:
            run_wind_full_case(args.ref, *c)
    if args.only is None or args.only in "wind2d_sirocco_64x32":
        run_sirocco_case(args.ref)


if __name__ == "__main__":
    main()
