"""Failure detection without a GPU fault: what the path does when something
goes wrong is checked by making the failure on the host or by letting a
bounded wait run out, never by a trap, a bad address or an endless loop.

* The bounded mbarrier wait of the stage kernels' TMA loads and of the
  learned step's MMAs (ps_tma.cuh `mbar_wait_bounded`), on a barrier that
  nothing completes, gives up after its poll limit and reports; the
  context stays usable (the same probe then sees a completed barrier).
* A NaN planted in one model's state stops that model only: the batch
  reports PS_F_NAN, the failed model's step counter stops, and the other
  model's state is bit for bit its run alone (each model's `done` flag in
  its own scalars, as the reference's QUIT_PLUTO ends only that run).
* A truncated snapshot is refused with a message, and the context it was
  meant for still runs.
* Halo poisoning: NaN in every ghost cell of the state handed in never
  reaches the result (the ghost zones are refilled before every stage, as
  the reference's Boundary does), for the Cartesian blast and the wind.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SPEC = dict(grid=(64, 32), l_star=1e37, krad=0.2, alpharad=-0.6)


def test_bounded_wait_gives_up_and_reports(built):
    import ctypes
    import psgb
    P = psgb.probe()
    done = ctypes.c_int(-1)
    assert P.ps_probe_wait_timeout(64, 0, ctypes.byref(done)) == 0
    assert done.value == 0          # nothing completed the barrier: the wait gave up
    assert P.ps_probe_wait_timeout(64, 1, ctypes.byref(done)) == 0
    assert done.value == 1          # the context is still usable, and a completed wait is seen


def test_nan_in_one_model_stops_that_model_only(built):
    import psgb
    solo = psgb.wind_model_solver(SPEC)
    ok, bad = psgb.wind_model_solver(SPEC), psgb.wind_model_solver(SPEC)
    V = bad.get_state()
    V[4, 0, 12, 20] = np.nan         # the pressure of one active cell
    bad.set_state(V)
    batch = psgb.Batch([ok, bad])
    flags = batch.run(4)
    assert flags & 0x01              # PS_F_NAN
    assert solo.run(4) & 0x01 == 0
    assert np.array_equal(ok.get_state(), solo.get_state())
    assert ok.time()[2] == 4 and bad.time()[2] < 4
    assert ok.time()[:2] == solo.time()[:2]
    batch.close()


def test_truncated_snapshot_is_refused(built, tmp_path):
    import psgb
    s = psgb.wind_model_solver(SPEC)
    path = tmp_path / "data.0001.dbl"
    path.write_bytes(np.zeros(1000).tobytes())
    with pytest.raises(RuntimeError, match="does not hold"):
        s.read_dbl(path)
    assert s.run(2) & ~0x2 == 0      # still runs (PS_F_CONS2PRIM is a repaired cell)


def _poison_ghosts(V, g):
    """NaN in every ghost cell of a [nv][k][j][i] 2-D state with g ghost
    layers per side."""
    W = V.copy()
    W[:, :, :g, :] = np.nan
    W[:, :, -g:, :] = np.nan
    W[:, :, :, :g] = np.nan
    W[:, :, :, -g:] = np.nan
    return W


@pytest.mark.parametrize("case", ["blast", "wind"])
def test_poisoned_ghost_cells_never_reach_the_result(built, case):
    """The reference refills the ghost zones before every stage (Boundary),
    so what the host hands in there must not matter: a state whose ghost
    cells are all NaN gives, bit for bit, what the clean state gives."""
    import psgb
    if case == "blast":
        cfg = psgb.make_config(dims=2, nx=(48, 40, 1), limiter="mc", solver="hllc", bc="outflow")
        grid = psgb.Grid(cfg)
        V0 = psgb.blast_state(cfg, grid)
        runs = []
        for V in (V0, _poison_ghosts(V0, 2)):
            s = psgb.Solver(cfg, grid)
            s.set_state(V)
            s.set_time(0.0, 1e-4, 0)
            assert s.run(5) == 0
            runs.append(s.get_state()[:, 0, 2:-2, 2:-2])
    else:
        clean = psgb.wind_model_solver(SPEC)
        poisoned = psgb.wind_model_solver(SPEC)
        poisoned.set_state(_poison_ghosts(poisoned.get_state(), 2))
        runs = []
        for s in (clean, poisoned):
            assert s.run(5) & ~0x2 == 0
            runs.append(s.get_state()[:, 0, 2:-2, 2:-2])
    assert not np.isnan(runs[1]).any()
    assert np.array_equal(runs[0], runs[1])
