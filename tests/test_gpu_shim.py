"""The drop-in on the GPU: the reference's own main loop (Src/main.c:
Integrate, NextTimeStep, output) with AdvanceStep and SplitSource taken
from pluto-sirocco_gb300/shim/ps_pluto_shim.c, i.e. computed by this
library (oracle/_ref/<cfg>/pluto_gb300, built by build()).  Its .dbl
output must match the reference's own output on the same case within the
hydro tolerance:

* the 2-D blast wave, 64x64, MC, HLLC, outflow, 50 steps;
* the 64x32 wind with the ODE cooling path (COOLING TABULATED), 100
  steps, snapshots every 20 steps: there the time step is limited by the
  cooling time, which reaches PLUTO's NextTimeStep only through the shim's
  Dts->dt_cool (ps_split_source_dt), so the dt column of dbl.out checks it;
* the 64x32 BLONDIN wind with the learned cooling step switched on through
  PS_LEARNED_COOLING (a network file written by ps_sg_save).
"""
import json
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import GOLDEN, HYDRO_REL_L1, rel_l1

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _shim_binary(cfg):
    import __graft_entry__ as g
    exe = os.path.join(ROOT, "oracle", "_ref", cfg, "pluto_gb300")
    if not os.access(exe, os.X_OK):
        ref = g.reference_tree()[0]
        assert ref, "neither the reference sources nor their staged copy are present"
        subprocess.run(["make", "-s", "-j8", "-f", os.path.join(ROOT, "oracle", "ref.mk"),
                        "CFG=" + cfg, "REF=" + ref, "shim"], check=True)
    return exe


def _dbl_out(wd):
    return [l.split() for l in open(os.path.join(wd, "dbl.out")).read().splitlines() if l]


def test_reference_main_loop_with_the_gpu_step_blast(built):
    import ref_runs
    exe = _shim_binary("blast2d")
    meta = json.load(open(os.path.join(GOLDEN, "blast2d_mc_hllc_outflow_64x64.json")))
    v1 = np.load(os.path.join(GOLDEN, "blast2d_mc_hllc_outflow_64x64.npz"))["v1"]
    wd = tempfile.mkdtemp(prefix="ps_shim_")
    try:
        ref_runs.prepare_blast(wd, 64, 64, solver="hllc", bc="outflow", cfl=0.4, tstop=10.0,
                               every=meta["steps"], log=meta["steps"])
        r = subprocess.run([exe, "-maxsteps", str(meta["steps"] - 1)], cwd=wd,
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
        a = np.fromfile(os.path.join(wd, "data.0001.dbl"), dtype="<f8").reshape(v1.shape)
        rl = rel_l1(a, v1)
        print("blast 64x64 through the shim, 50 steps: relative L1 per variable", rl)
        assert np.all(rl <= HYDRO_REL_L1), rl
        row = _dbl_out(wd)[1]
        assert abs(float(row[1]) - float(meta["t_final"])) <= 1e-6 * float(meta["t_final"])
    finally:
        shutil.rmtree(wd, ignore_errors=True)


def test_reference_main_loop_with_the_gpu_step_ode_wind(built):
    import ref_runs
    exe = _shim_binary("wind2d_ode")
    meta = json.load(open(os.path.join(GOLDEN, "wind2d_ode_64x32.json")))
    snaps = np.load(os.path.join(GOLDEN, "wind2d_ode_64x32.npz"))["snaps"]
    every = 20
    wd = tempfile.mkdtemp(prefix="ps_shim_")
    try:
        ref_runs.prepare_wind(wd, 64, 32, every=every, log=every)
        r = subprocess.run([exe, "-maxsteps", str(meta["steps"] - 1)], cwd=wd,
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
        rows = _dbl_out(wd)
        for k, step in enumerate(meta["snap_steps"]):
            a = np.fromfile(os.path.join(wd, "data.%04d.dbl" % (step // every)),
                            dtype="<f8").reshape(snaps[k].shape)
            rl = rel_l1(a, snaps[k])
            print("ODE wind through the shim, step", step, "relative L1 per variable", rl)
            assert np.all(rl <= HYDRO_REL_L1), (step, rl)
            row = rows[step // every]
            for col, key in ((1, "t"), (2, "dt")):
                want = float(meta[key][k])
                assert abs(float(row[col]) - want) <= 1e-6 * abs(want), (step, key, row, want)
    finally:
        shutil.rmtree(wd, ignore_errors=True)


def test_reference_main_loop_with_the_learned_cooling_step(built, tmp_path):
    """PS_LEARNED_COOLING names a network file (ps_sg_save): the drop-in
    then runs the learned BLONDIN step in SplitSource.  The reference's own
    main loop through the shim (64x32 BLONDIN wind, 20 steps) gives what
    the library's loop gives with the same network, and stays within the
    learned step's tolerance of the reference method's run.  The network is
    the library's default initialisation: the judge checks every cell and
    hands the ones it rejects to the reference method, so any network gives
    a valid step."""
    import psgb
    import ref_runs
    from test_gpu_wind import _wind_solver
    exe = _shim_binary("wind2d")
    lo, hi = [b[0] for b in psgb.SG_DRAW_BOX], [b[1] for b in psgb.SG_DRAW_BOX]
    sg = psgb.Surrogate(lo, hi)
    net = tmp_path / "net.psg"
    sg.save(net)
    again = psgb.Surrogate.load(net)
    assert np.array_equal(again.params(), sg.params())
    bad = tmp_path / "bad.psg"
    bad.write_bytes(open(net, "rb").read()[:-4])
    with pytest.raises(RuntimeError, match="not a network file"):
        psgb.Surrogate.load(bad)

    steps = 20
    lib_run = _wind_solver(64, 32, cooling=1, line_force=1)
    psgb.check(psgb.lib().ps_set_surrogate(lib_run.ctx, again.h, 1), "ps_set_surrogate")
    assert lib_run.run(steps) & ~0x2 == 0
    want = lib_run.get_state()[:6, 0, 2:-2, 2:-2]
    ref_run = _wind_solver(64, 32, cooling=1, line_force=1)      # the reference method
    assert ref_run.run(steps) & ~0x2 == 0
    exact = ref_run.get_state()[:6, 0, 2:-2, 2:-2]

    wd = tempfile.mkdtemp(prefix="ps_shim_")
    try:
        ref_runs.prepare_wind(wd, 64, 32, every=steps, log=steps)
        env = dict(os.environ, PS_LEARNED_COOLING=str(net))
        r = subprocess.run([exe, "-maxsteps", str(steps - 1)], cwd=wd, env=env,
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
        assert "learned cooling step" in r.stdout
        got = np.fromfile(os.path.join(wd, "data.0001.dbl"), dtype="<f8").reshape(want.shape)
        rl = rel_l1(got, want)
        print("learned step through the shim against the library's loop:", rl)
        assert np.all(rl <= 1e-9), rl
        rx = rel_l1(got, exact)
        print("learned step through the shim against the reference method:", rx)
        assert np.all(rx <= 1e-3), rx
    finally:
        shutil.rmtree(wd, ignore_errors=True)
