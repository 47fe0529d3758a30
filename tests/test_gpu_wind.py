"""CUDA path of the 2-D spherical line-driven disk wind against the
reference (golden snapshots) and the oracle.

* hydro part (geometry, general-grid PLM, HLL, tracer, userdef boundary,
  floors, gravity): relative L1 within 1e-11 per variable (the device code
  contracts multiplies and adds into FMAs; the measured difference after
  100 steps is about 5e-13);
* full physics (plus BLONDIN cooling and the line force): the device
  exp/pow/log10 are CUDA's, not glibc's, so results differ in the last
  bits and the differences are bounded by the tolerances below."""
import numpy as np
import pytest

from conftest import assert_hydro_close, golden_cases

pytestmark = pytest.mark.gpu


def _wind_solver(nr, nt, cooling, line_force, char_limiting=0, shock_flattening=0, solver="hll",
                 entropy_switch=0):
    import psgb
    cfg = psgb.make_wind_config(nr, nt, cooling=cooling, char_limiting=char_limiting,
                                shock_flattening=shock_flattening, solver=solver,
                                entropy_switch=entropy_switch)
    w = psgb.make_wind(line_force=line_force)
    g = psgb.WindGrid(cfg)
    s = psgb.Solver(cfg, g)
    s.set_state(psgb.wind_state(cfg, w, g))
    s.set_time(0.0, 1e-4, 0)
    s.set_wind(w, psgb.wind_flux(cfg, w, g) if line_force else None)
    return s


def _active(V, g=2):
    """Active cells of the variables written to .dbl files (the entropy of
    ENTROPY_SWITCH contexts is not written); g ghost zones per side."""
    return V[:6, 0, g:-g, g:-g]


def _case(name):
    return [m for m in golden_cases(kind="wind") if m["name"].startswith(name)][0]


def test_wind_hydro_matches_reference(built):
    meta = _case("wind2d_hydro")
    snaps = np.load(meta["npz"])["snaps"]
    s = _wind_solver(meta["n"][0], meta["n"][1], cooling=0, line_force=0)
    done = 0
    for k, step in enumerate(meta["snap_steps"]):
        if step > done:
            s.run(step - done)
            done = step
        a = _active(s.get_state())
        r = assert_hydro_close(a, snaps[k], f"step {step}")
        print("step", step, "relative L1 per variable", r)
        t, dt, _, _ = s.time()
        assert abs(t - float(meta["t"][k])) <= 6e-7 * abs(t)


def test_wind_char_limiting_matches_reference(built):
    """CHAR_LIMITING YES (PLM on characteristic variables, as the production
    cv_idl configuration uses it), hydro part of the wind."""
    meta = _case("wind2d_char")
    snaps = np.load(meta["npz"])["snaps"]
    s = _wind_solver(meta["n"][0], meta["n"][1], cooling=0, line_force=0, char_limiting=1)
    done = 0
    for k, step in enumerate(meta["snap_steps"]):
        if step > done:
            s.run(step - done)
            done = step
        r = assert_hydro_close(_active(s.get_state()), snaps[k], f"step {step}")
        print("char limiting, step", step, "relative L1 per variable", r)
    # and it is not the primitive-variable limiter
    h = _wind_solver(meta["n"][0], meta["n"][1], cooling=0, line_force=0)
    h.run(meta["snap_steps"][-1])
    assert not np.allclose(_active(h.get_state()), snaps[-1], rtol=1e-6)


@pytest.mark.parametrize("name", ["wind2d_multid_64", "wind2d_multid_hllc"])
def test_wind_multid_matches_reference(built, name):
    """SHOCK_FLATTENING MULTID (FlagShock once per step, minmod slopes in
    and next to the shocked zones), hydro part of the wind: with
    CHAR_LIMITING YES and HLL as in the production cv_idl configuration,
    and with primitive limiting and HLLC, whose faces next to a shocked
    zone take the HLL flux."""
    meta = _case(name)
    snaps = np.load(meta["npz"])["snaps"]
    char, solver = meta["char_limiting"], meta.get("solver", "hll")
    s = _wind_solver(meta["n"][0], meta["n"][1], cooling=0, line_force=0, char_limiting=char,
                     shock_flattening=1, solver=solver)
    done = 0
    for k, step in enumerate(meta["snap_steps"]):
        if step > done:
            s.run(step - done)
            done = step
        r = assert_hydro_close(_active(s.get_state(), 3), snaps[k], f"step {step}")
        print("MULTID, step", step, "relative L1 per variable", r)
        t, dt, _, _ = s.time()
        assert abs(t - float(meta["t"][k])) <= 6e-7 * abs(t)
    # the flattening is switched on: without it the result is another one
    h = _wind_solver(meta["n"][0], meta["n"][1], cooling=0, line_force=0, char_limiting=char,
                     solver=solver)
    h.run(meta["snap_steps"][-1])
    assert not np.allclose(_active(h.get_state()), snaps[-1], rtol=1e-6)


@pytest.mark.parametrize("name", ["wind2d_entsel", "wind2d_idl_hydro", "wind2d_idl_64"])
def test_wind_entropy_switch_matches_reference(built, name):
    """ENTROPY_SWITCH: pressure recovered from the advected entropy rho s
    (s = p / rho^gamma recomputed after every Boundary) -- SELECTIVE with
    primitive limiting, and ALWAYS with characteristic limiting and MULTID
    flattening (the numerics of the production cv_idl configuration), hydro
    only and with BLONDIN cooling and the line force."""
    meta = _case(name)
    snaps = np.load(meta["npz"])["snaps"]
    g = 3 if meta["shock_flattening"] else 2
    s = _wind_solver(meta["n"][0], meta["n"][1], cooling=meta["cooling"],
                     line_force=meta["line_force"], char_limiting=meta["char_limiting"],
                     shock_flattening=meta["shock_flattening"], solver=meta["solver"],
                     entropy_switch=meta["entropy_switch"])
    done = 0
    for k, step in enumerate(meta["snap_steps"]):
        if step > done:
            s.run(step - done)
            done = step
        # with cooling and the line force the reference's own solution moves
        # by ~3e-9 (relative L1) at step 200 when its initial state is
        # perturbed by 1e-15 (a shock flag or limiter branch flips between
        # steps 100 and 200; test_production_wind_sensitivity), so the last
        # snapshot of that case is held to 1e-7
        tol = 1e-7 if (meta["cooling"] and step > 100) else None
        if tol is None:
            r = assert_hydro_close(_active(s.get_state(), g), snaps[k], f"step {step}")
        else:
            r = _rel_l1(_active(s.get_state(), g), snaps[k])
            assert np.all(r < tol), (step, r)
        print(name, "step", step, "relative L1 per variable", r)
        t, dt, _, _ = s.time()
        assert abs(t - float(meta["t"][k])) <= 6e-7 * abs(t)
    if meta["cooling"]:
        return   # the split cooling step changes p after the stage, not s
    # the entropy (last variable) is p / rho^gamma up to the stage's rounding
    V = s.get_state()
    ent = V[6, 0, g:-g, g:-g]
    ref = V[4, 0, g:-g, g:-g] / V[0, 0, g:-g, g:-g] ** 1.6666666666666667
    assert np.max(np.abs(ent / ref - 1.0)) < 1e-9


def test_wind_tabulated_force_multiplier_matches_reference(built, tmp_path):
    """KRAD = ALPHARAD = 999: the line force interpolates each cell's
    tabulated M(t) (M_UV_data.dat, read here by the C reader from the file
    the reference read) instead of k t^alpha; full physics, 100 steps."""
    import psgb
    from make_golden import write_mfit_file
    meta = _case("wind2d_mfit")
    snaps = np.load(meta["npz"])["snaps"]
    nr, nt = meta["n"][0], meta["n"][1]
    cfg = psgb.make_wind_config(nr, nt, cooling=1)
    w = psgb.make_wind(line_force=1, krad=999.0, alpharad=999.0)
    g = psgb.WindGrid(cfg)
    s = psgb.Solver(cfg, g)
    s.set_state(psgb.wind_state(cfg, w, g))
    s.set_time(0.0, 1e-4, 0)
    s.set_wind(w, psgb.wind_flux(cfg, w, g))
    with pytest.raises(RuntimeError):        # the table is required
        s.run(1)
    write_mfit_file(str(tmp_path), nr, nt)
    t, m, matched = psgb.read_m_uv_fit(cfg, g, str(tmp_path / "M_UV_data.dat"))
    assert matched == nr * nt
    s.set_mfit(t, m)
    done = 0
    for k, step in enumerate(meta["snap_steps"]):
        if step > done:
            s.run(step - done)
            done = step
        r = assert_hydro_close(_active(s.get_state()), snaps[k], f"step {step}")
        print("tabulated M, step", step, "relative L1 per variable", r)
    # and it is not the power law
    h = _wind_solver(nr, nt, cooling=1, line_force=1)
    h.run(meta["snap_steps"][-1])
    assert not np.allclose(_active(h.get_state()), snaps[-1], rtol=1e-6)


def test_wind_dense_flux_matches_reference(built):
    """Flux in every one of the 36 bins (the shape of SIROCCO's fluxes): the
    line force takes its factored form (one power of rho p per sweep and a
    product per bin) and matches the reference run on the same flux files."""
    import psgb
    meta = _case("wind2d_dense")
    snaps = np.load(meta["npz"])["snaps"]
    nr, nt = meta["n"][0], meta["n"][1]
    cfg = psgb.make_wind_config(nr, nt, cooling=1)
    w = psgb.make_wind(line_force=1)
    g = psgb.WindGrid(cfg)
    s = psgb.Solver(cfg, g)
    s.set_state(psgb.wind_state(cfg, w, g))
    s.set_time(0.0, 1e-4, 0)
    s.set_wind(w, psgb.wind_flux(cfg, w, g, dense=True))
    done = 0
    for k, step in enumerate(meta["snap_steps"]):
        if step > done:
            s.run(step - done)
            done = step
        r = assert_hydro_close(_active(s.get_state()), snaps[k], f"step {step}")
        print("dense flux, step", step, "relative L1 per variable", r)


def test_wind_ode_cooling_matches_reference(built):
    """The ODE cooling path (cooling = 2: COOLING TABULATED with the
    production problem's CoolingSource and Radiat, RKF12 or adaptive
    Cash-Karp per cell, dt_cool limiting the step), with the line force,
    against the reference run: state and the time step at every snapshot."""
    import psgb
    meta = _case("wind2d_ode")
    snaps = np.load(meta["npz"])["snaps"]
    s = _wind_solver(meta["n"][0], meta["n"][1], cooling=2, line_force=1)
    done = 0
    for k, step in enumerate(meta["snap_steps"]):
        if step > done:
            assert s.run(step - done) & 0x20 == 0   # PS_F_COOLING
            done = step
        r = assert_hydro_close(_active(s.get_state()), snaps[k], f"step {step}")
        print("ODE cooling, step", step, "relative L1 per variable", r)
        t, dt, _, _ = s.time()
        assert abs(t - float(meta["t"][k])) <= 6e-7 * abs(t)
        assert abs(dt - float(meta["dt"][k])) <= 6e-7 * abs(dt)
    # dt_cool is what limits the step here: the BLONDIN run's dt differs
    h = _wind_solver(meta["n"][0], meta["n"][1], cooling=1, line_force=1)
    h.run(20)
    assert abs(h.time()[1] - float(meta["dt"][1])) > 1e-3 * h.time()[1]
    # the learned step is for BLONDIN's implicit solve only
    sg = psgb.Surrogate(psgb.SG_DRAW_BOX and [b[0] for b in psgb.SG_DRAW_BOX],
                        [b[1] for b in psgb.SG_DRAW_BOX])
    assert psgb.lib().ps_set_surrogate(s.ctx, sg.h, 1) < 0
    sg.close()


def _rel_l1(a, b):
    return np.abs(a - b).sum(axis=(1, 2)) / np.maximum(np.abs(b).sum(axis=(1, 2)), 1e-300)


def test_wind_full_physics_close_to_reference(built):
    meta = _case("wind2d_full")
    snaps = np.load(meta["npz"])["snaps"]
    s = _wind_solver(meta["n"][0], meta["n"][1], cooling=1, line_force=1)
    done = 0
    report = []
    for k, step in enumerate(meta["snap_steps"]):
        if step > done:
            s.run(step - done)
            done = step
        a = _active(s.get_state())
        rl1 = _rel_l1(a, snaps[k])
        report.append((step, rl1))
        print("step", step, "rel L1 per variable", rl1)
    # every snapshot (steps 20, 100, 200) within 1e-11 of the reference:
    # measured 4e-13, 2.4e-13 and 8e-13; at this size the flow is not
    # sensitive (the oracle perturbed by 1e-15 moves 1.4e-12 by step 200)
    for step, rl1 in report:
        assert np.all(rl1 <= 1e-11), (step, rl1)


def test_production_problem_hooks_match_reference(built):
    """The production disk-wind problem's own hooks (cv_idl/init.c compiled by
    the reference build: floors, X1-beg inflow copy, X2-beg hybrid condition
    -- reflected velocities, density and pressure copied -- and gravity) with
    its numerics (characteristic PLM, MULTID, entropy switch, BLONDIN, line
    force), started from the reference's own first snapshot: every snapshot
    through step 100 within 1e-11 (the oracle perturbed by 1e-15 moves 2e-15
    by then)."""
    import psgb
    meta = _case("wind2d_cvidl")
    snaps = np.load(meta["npz"])["snaps"]
    nr, nt = meta["n"][0], meta["n"][1]
    cfg = psgb.make_wind_config(nr, nt, cooling=1, char_limiting=1, shock_flattening=1,
                                entropy_switch=2, bc=psgb.CVIDL_BC)
    w = psgb.make_wind(line_force=1)
    g = psgb.WindGrid(cfg)
    ng = psgb.nghost(cfg)
    V = np.zeros((cfg.nvar, 1, g.ntot[1], g.ntot[0]))
    V[:6, 0, ng:-ng, ng:-ng] = snaps[0]     # ghosts come from the first Boundary
    s = psgb.Solver(cfg, g)
    s.set_state(V)
    s.set_time(0.0, 1e-4, 0)
    s.set_wind(w, psgb.wind_flux(cfg, w, g))
    done = 0
    for k, step in enumerate(meta["snap_steps"]):
        if step > done:
            s.run(step - done)
            done = step
        a = _active(s.get_state(), ng)
        r = assert_hydro_close(a, snaps[k], f"step {step}")
        print("production hooks, step", step, "relative L1 per variable", r)
        t, dt, _, _ = s.time()
        assert abs(t - float(meta["t"][k])) <= 6e-7 * max(t, 1e-300)
        assert abs(dt - float(meta["dt"][k])) <= 6e-7 * dt
    # the X2-beg user side differs from the axisymmetric one of the test
    # problem: run with that instead and the state moves
    cfg2 = psgb.make_wind_config(nr, nt, cooling=1, char_limiting=1, shock_flattening=1,
                                 entropy_switch=2)
    s2 = psgb.Solver(cfg2, g)
    s2.set_state(V)
    s2.set_time(0.0, 1e-4, 0)
    s2.set_wind(w, psgb.wind_flux(cfg2, w, g))
    s2.run(20)
    assert not np.allclose(_active(s2.get_state(), ng), snaps[1], rtol=1e-9, atol=0)
