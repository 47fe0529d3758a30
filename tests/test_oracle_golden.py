"""The CPU oracle against golden vectors produced by the reference's own
serial build (tests/golden/make_golden.py).  Bit-exact: every variable of
every active cell, plus the reference's printed time and next dt."""
import hashlib

import numpy as np
import pytest

from conftest import golden_cases, load_golden


def _digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def _oracle_for(meta):
    from oracle import Oracle
    o = Oracle(dims=meta["dims"], nx=meta["n"], limiter=meta["limiter"], solver=meta["solver"],
               bc=meta["bc"], cfl=meta["cfl"], cfl_max_var=meta["cfl_max_var"],
               tstop=meta["tstop"], first_dt=meta["first_dt"])
    o.init_blast(meta["p_amb"], meta["p_in"], meta["r_in"], meta["noise"], meta["seed"])
    return o


@pytest.mark.parametrize("meta", golden_cases(), ids=lambda m: m["name"])
def test_oracle_matches_reference(built, meta):
    o = _oracle_for(meta)
    assert _digest(o.active()) == meta["ic_sha256"], "initial condition differs"
    if meta["npz"]:
        v0, v1 = load_golden(meta)
        assert np.array_equal(o.active(), v0)
    assert o.run(meta["steps"]) == 0
    a = o.active()
    if meta["npz"]:
        assert np.array_equal(a, v1), f"max |diff| = {np.abs(a - v1).max()}"
    assert _digest(a) == meta["final_sha256"]
    t, dt, step = o.time()
    assert step == meta["steps"]
    assert float(f"{t:e}") == float(meta["t_final"])
    assert float(f"{dt:e}") == float(meta["dt_next"])


def test_oracle_detects_planted_error(built):
    """A deliberately perturbed initial cell must break bit-exactness (the
    comparison is not vacuous)."""
    meta = [m for m in golden_cases(full_only=True) if m["dims"] == 2][0]
    o = _oracle_for(meta)
    V = o.V
    V[0, 0, 10, 10] = np.nextafter(V[0, 0, 10, 10], 2.0)
    o.run(meta["steps"])
    _, v1 = load_golden(meta)
    assert not np.array_equal(o.active(), v1)


@pytest.mark.parametrize("meta", golden_cases(kind="wind"), ids=lambda m: m["name"])
def test_wind_oracle_matches_reference(built, meta):
    """2-D spherical line-driven disk wind: geometry, general-grid PLM, HLL,
    tracer, userdef boundary and floors, gravity and (full case) BLONDIN
    cooling with the Strang alternation and the line force: bit-exact at
    every stored snapshot."""
    from oracle import CVIDL_BC, wind_oracle
    snaps = np.load(meta["npz"])["snaps"]
    nr, nt = meta["n"][0], meta["n"][1]
    # the production problem starts from the reference's own first snapshot
    # (its Init is not restated); its boundaries are its user sides
    cvidl = bool(meta.get("cvidl", 0))
    o = wind_oracle(nr, nt, cooling=meta["cooling"], line_force=meta["line_force"],
                    bc=CVIDL_BC if cvidl else None, initial=snaps[0] if cvidl else None,
                    char_limiting=meta.get("char_limiting", 0),
                    shock_flattening=meta.get("shock_flattening", 0),
                    solver=meta.get("solver", "hll"),
                    entropy_switch=meta.get("entropy_switch", 0), mfit=bool(meta.get("mfit", 0)),
                    ode_cooling=meta.get("ode_cooling", 0),
                    dense_flux=bool(meta.get("dense_flux", 0)))
    if "sirocco_seed" in meta:
        # restarted at t0 with the SIROCCO data files (make_golden.run_sirocco_case)
        from make_golden import sirocco_as_read
        from oracle import lib as olib
        xi, tr, pre = sirocco_as_read(nr, nt, meta["sirocco_seed"])
        o.set_sirocco(xi[None], tr[None], pre[:, None])
        olib().or_set_time(o.s, meta["t0"], 1e-4, 0)
    done = 0
    for k, step in enumerate(meta["snap_steps"]):
        if step > done:
            o.run(step - done)
            done = step
        a = o.active()[:snaps.shape[1]]   # the dumped variables
        assert np.array_equal(a, snaps[k]), f"step {step}: max |diff| {np.abs(a - snaps[k]).max()}"
        t, dt, _ = o.time()
        assert float(f"{t:e}") == float(meta["t"][k])
        assert float(f"{dt:e}") == float(meta["dt"][k])
    assert _digest(o.active()[:snaps.shape[1]]) == meta["final_sha256"]


def test_production_wind_sensitivity(built):
    """The production numerics (characteristic limiting, MULTID, entropy
    switch) with BLONDIN cooling and the line force are sensitive to the
    last bit: a 1e-15 relative perturbation of the initial state stays at
    1e-15 for 100 steps and has grown to 1e-10 .. 1e-7 (relative L1) by
    step 200, where a shock flag or limiter branch flips.  This bounds how
    close any implementation that rounds differently (the FMA-contracted
    device code) can stay to the reference at that step."""
    from oracle import wind_oracle
    meta = [m for m in golden_cases(kind="wind") if m["name"].startswith("wind2d_idl_64")][0]
    snaps = np.load(meta["npz"])["snaps"]
    o = wind_oracle(64, 32, cooling=1, line_force=1, char_limiting=1, shock_flattening=1,
                    entropy_switch=2)
    rng = np.random.default_rng(1)
    o.V[:5] *= 1 + 1e-15 * rng.standard_normal(o.V[:5].shape)

    def rel(a, b):
        return (np.abs(a - b).sum(axis=(1, 2)) / np.abs(b).sum(axis=(1, 2))).max()

    o.run(100)
    assert rel(o.active()[:6], snaps[2]) < 1e-13
    o.run(100)
    r = rel(o.active()[:6], snaps[3])
    assert 1e-10 < r < 1e-7, r
