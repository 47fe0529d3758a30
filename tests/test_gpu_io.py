"""DBL snapshots of device state against the reference's own files: the
reader loads a .dbl that the reference wrote, the writer reproduces it byte
for byte together with its dbl.out lines, and a wind state survives a
write/read round trip exactly."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_cases, load_golden

pytestmark = pytest.mark.gpu

NAME = "blast2d_mc_hll_periodic_48x40"


def _ctx(meta):
    import psgb
    cfg = psgb.make_config(dims=meta["dims"], nx=meta["n"], limiter=meta["limiter"],
                           solver=meta["solver"], bc=meta["bc"], cfl=meta["cfl"],
                           cfl_max_var=meta["cfl_max_var"], tstop=meta["tstop"],
                           first_dt=meta["first_dt"])
    g = psgb.Grid(cfg)
    s = psgb.Solver(cfg, g)
    s.set_state(psgb.blast_state(cfg, g))
    return s


def test_dbl_reader_and_writer_match_the_reference_files(built, tmp_path):
    meta = [m for m in golden_cases() if m["name"] == NAME][0]
    ref_dbl = os.path.join(GOLDEN, NAME + ".dbl")
    ref_log = open(os.path.join(GOLDEN, NAME + ".dbl.out")).read().splitlines()
    s = _ctx(meta)
    s.read_dbl(ref_dbl)
    _, v1 = load_golden(meta)
    assert np.array_equal(s.get_state()[:, 0, 2:-2, 2:-2], v1)
    # the same snapshot written back: identical bytes and log lines
    f0 = ref_log[0].split()
    s.set_time(float(f0[1]), float(f0[2]), int(f0[3]))
    s.write_dbl(str(tmp_path), 0)
    f1 = ref_log[1].split()
    s.set_time(float(f1[1]), float(f1[2]), int(f1[3]))
    s.write_dbl(str(tmp_path), 1)
    assert open(tmp_path / "data.0001.dbl", "rb").read() == open(ref_dbl, "rb").read()
    assert open(tmp_path / "dbl.out").read().splitlines() == ref_log


def test_dbl_round_trip_of_a_wind_state(built, tmp_path):
    import psgb
    sp = dict(grid=(64, 32), l_star=1e37, krad=0.2, alpharad=-0.6)
    a = psgb.wind_model_solver(sp)
    a.write_dbl(str(tmp_path), 0)
    a.run(8)   # an even step: invDt_hyp starts afresh, as after a restart
    a.write_dbl(str(tmp_path), 3)
    b = psgb.wind_model_solver(sp)
    b.read_dbl(str(tmp_path / "data.0003.dbl"))
    va, vb = a.get_state(), b.get_state()
    assert np.array_equal(va[:, 0, 2:-2, 2:-2], vb[:, 0, 2:-2, 2:-2])
    # dbl.out keeps the lines before nfile (only one exists here)
    line = open(tmp_path / "dbl.out").read().splitlines()
    assert len(line) == 2 and line[1].split()[0] == "3" and line[1].split()[3] == "8"
    assert line[1].endswith("prs tr1 ")
    # b continues like a
    t, dt, step, _ = a.time()
    b.set_time(t, dt, step)
    a.run(4)
    b.run(4)
    assert np.array_equal(a.get_state()[:, 0, 2:-2, 2:-2], b.get_state()[:, 0, 2:-2, 2:-2])
    with pytest.raises(RuntimeError):
        c = psgb.wind_model_solver(dict(sp, grid=(32, 32)))
        c.read_dbl(str(tmp_path / "data.0003.dbl"))
