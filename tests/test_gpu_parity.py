"""CUDA path against the reference (golden vectors) and the oracle.

The device kernels keep the reference's operation order; they contract
multiplies and adds into FMAs, so the state is compared with the
tolerances of conftest (relative L1 1e-11 per variable, conserved totals
1e-12), the time-step sequence to 1e-12, and paths of the library against
each other bit for bit."""
import hashlib

import numpy as np
import pytest

from conftest import CONSERVED_REL, assert_hydro_close, golden_cases, load_golden

pytestmark = pytest.mark.gpu


def _digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def _active(V, dims):
    return V[:, 0, 2:-2, 2:-2] if dims == 2 else V[:, 2:-2, 2:-2, 2:-2]


def _solver(meta, **over):
    import psgb
    kw = dict(dims=meta["dims"], nx=meta["n"], limiter=meta["limiter"], solver=meta["solver"],
              bc=meta["bc"], cfl=meta["cfl"], cfl_max_var=meta["cfl_max_var"],
              tstop=meta["tstop"], first_dt=meta["first_dt"])
    kw.update(over)
    cfg = psgb.make_config(**kw)
    g = psgb.Grid(cfg)
    s = psgb.Solver(cfg, g)
    V = psgb.blast_state(cfg, g, meta["p_amb"], meta["p_in"], meta["r_in"], meta["noise"],
                         meta["seed"])
    s.set_state(V)
    s.set_time(0.0, meta["first_dt"], 0)
    return s, V


def _oracle(meta, **over):
    from oracle import Oracle
    kw = dict(dims=meta["dims"], nx=meta["n"], limiter=meta["limiter"], solver=meta["solver"],
              bc=meta["bc"], cfl=meta["cfl"], cfl_max_var=meta["cfl_max_var"],
              tstop=meta["tstop"], first_dt=meta["first_dt"])
    kw.update(over)
    o = Oracle(**kw)
    o.init_blast(meta["p_amb"], meta["p_in"], meta["r_in"], meta["noise"], meta["seed"])
    return o


@pytest.mark.parametrize("meta", golden_cases(), ids=lambda m: m["name"])
def test_gpu_matches_reference(built, meta):
    s, _ = _solver(meta)
    flags = s.run(meta["steps"])
    assert flags == 0
    a = _active(s.get_state(), meta["dims"])
    if meta["npz"]:
        _, ref = load_golden(meta)
    else:
        o = _oracle(meta)
        o.run(meta["steps"])
        ref = o.active().reshape(a.shape)
        assert _digest(ref) == meta["final_sha256"]   # the oracle is the reference here
    r = assert_hydro_close(a, ref, meta["name"])
    print(meta["name"], "relative L1 per variable", r)
    g = 5.0 / 3.0
    for k, (x, y) in enumerate(((a[0], ref[0]),
                                (0.5 * a[0] * (a[1] ** 2 + a[2] ** 2 + a[3] ** 2) + a[4] / (g - 1),
                                 0.5 * ref[0] * (ref[1] ** 2 + ref[2] ** 2 + ref[3] ** 2)
                                 + ref[4] / (g - 1)))):
        assert abs(x.sum() - y.sum()) <= CONSERVED_REL * abs(y.sum()), ("mass", "energy")[k]
    t, dt, step, _ = s.time()
    assert step == meta["steps"]
    # the golden files print t and dt with 7 significant digits
    assert abs(t - float(meta["t_final"])) <= 6e-7 * abs(t)
    assert abs(dt - float(meta["dt_next"])) <= 6e-7 * abs(dt)


@pytest.mark.parametrize("meta", golden_cases(full_only=True)[:3], ids=lambda m: m["name"])
def test_gpu_dt_sequence_matches_oracle(built, meta):
    s, _ = _solver(meta)
    s.run(meta["steps"])
    o = _oracle(meta)
    o.run(meta["steps"])
    dt_o, _ = o.history(meta["steps"])
    dt_g = s.dt_history(meta["steps"])
    assert len(dt_g) == len(dt_o)
    assert np.max(np.abs(dt_g - dt_o) / dt_o) <= 1e-12
    t_g, dt_g, _, _ = s.time()
    t_o, dt_o2, _ = o.time()
    assert abs(t_g - t_o) <= 1e-12 * t_o and abs(dt_g - dt_o2) <= 1e-12 * dt_o2


def test_advance_step_dropin_matches_run(built):
    """ps_advance_step (the AdvanceStep replacement driven by a host loop
    that does its own NextTimeStep) gives the same state as ps_run."""
    meta = golden_cases(full_only=True)[0]
    s, _ = _solver(meta)
    dt, t = meta["first_dt"], 0.0
    n = 12
    for _ in range(n):
        flags, inv = s.advance_step(dt, 0.0)
        assert flags == 0
        t += dt
        dt_hyp = 1.0 / inv
        dt_hyp *= meta["cfl"]
        dt = min(dt_hyp, meta["cfl_max_var"] * dt)
    a = s.get_state()
    s2, _ = _solver(meta)
    s2.run(n)
    assert np.array_equal(a, s2.get_state()) or np.array_equal(
        _active(a, meta["dims"]), _active(s2.get_state(), meta["dims"]))
    t2, dt2, _, _ = s2.time()
    assert t2 == t and dt2 == dt


def test_tstop_clamp_matches_oracle(built):
    meta = dict(golden_cases(full_only=True)[0])
    s, _ = _solver(meta, tstop=0.01)
    s.run(40)  # more steps than needed: the ones after tstop are no-ops
    o = _oracle(meta, tstop=0.01)
    o.run(40)
    t, _, step, _ = s.time()
    assert step == o.time()[2]
    assert abs(t - 0.01) < 1e-15 and abs(o.time()[0] - 0.01) < 1e-15
    assert_hydro_close(_active(s.get_state(), 2), o.active(), "tstop")


def test_periodic_conservation(built):
    meta = [m for m in golden_cases() if m["bc"] == "periodic" and m["dims"] == 2][0]
    s, V0 = _solver(meta)
    s.run(meta["steps"])
    V1 = s.get_state()
    g = 5.0 / 3.0

    def totals(V):
        a = _active(V, 2)
        rho, vx, vy, vz, p = a
        e = 0.5 * rho * (vx * vx + vy * vy + vz * vz) + p / (g - 1)
        return rho.sum(), e.sum()

    m0, e0 = totals(V0)
    m1, e1 = totals(V1)
    assert abs(m1 - m0) / m0 < 1e-12
    assert abs(e1 - e0) / e0 < 1e-12


def test_nan_in_input_is_flagged(built):
    meta = golden_cases(full_only=True)[0]
    import psgb
    cfg = psgb.make_config(dims=2, nx=meta["n"])
    g = psgb.Grid(cfg)
    s = psgb.Solver(cfg, g)
    V = psgb.blast_state(cfg, g)
    V[4, 0, 20, 20] = np.nan
    s.set_state(V)
    s.set_time(0.0, 1e-4, 0)
    flags = s.run(1)
    assert flags & 0x01


def test_launch_count_is_three_per_step(built):
    meta = golden_cases(full_only=True)[0]
    s, _ = _solver(meta)
    before = s.launches()
    s.run(20)
    assert s.launches() - before == 60
