"""C-ABI library checks that need no GPU: it loads, exports every entry
point declared in include/ps_gb300.h, its host helpers reproduce the
reference's grid and initial condition, and bad configurations are
rejected before any device work."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, golden_cases


def _declared():
    src = open(os.path.join(ROOT, "include", "ps_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(ps_[a-z_0-9]+)\s*\(", src)))


def test_exports_every_declared_symbol(built):
    import psgb
    L = psgb.lib()
    names = _declared()
    assert len(names) >= 15
    for n in names:
        assert hasattr(L, n), f"{n} declared but not exported"
    assert sorted(psgb.EXPORTS) == names


@pytest.mark.parametrize("kind,n,xb,xe,ratio", [("uniform", 256, 0.0, 1.0, 1.0),
                                                ("uniform", 37, -0.5, 0.75, 1.0),
                                                ("log", 512, 1.0, 100.0, 1.0),
                                                ("ratio", 96, 1.0, 50.0, 1.03)])
def test_grid_matches_oracle(built, kind, n, xb, xe, ratio):
    import psgb
    from oracle import Oracle, OrConfig, lib as olib
    x, xl, xr, dx = psgb.build_grid(n, 2, xb, xe, kind, ratio)
    c = OrConfig()
    c.dims = 1
    c.nx[:] = [n, 1, 1]
    c.nvar = 5
    c.gridtype[:] = [{"uniform": 0, "log": 1, "ratio": 2}[kind], 0, 0]
    c.xbeg[:] = [xb, 0, 0]
    c.xend[:] = [xe, 1, 1]
    c.ratio[:] = [ratio, 1, 1]
    c.gamma, c.cfl, c.cfl_max_var, c.tstop, c.first_dt = 5 / 3, 0.4, 1.1, 1.0, 1e-4
    s = olib().or_create(ctypes.byref(c))
    try:
        for which, arr in enumerate((x, xl, xr, dx)):
            ref = np.ctypeslib.as_array(olib().or_grid(s, 0, which), shape=(n + 4,))
            assert np.array_equal(arr, ref)
    finally:
        olib().or_destroy(s)


def test_uniform_grid_matches_reference_spacing(built):
    import psgb
    x, xl, xr, dx = psgb.build_grid(256, 2)
    assert x[2] == 0.5 / 256 and xl[2] == 0.0 and xr[-3] == 1.0
    assert np.all(dx == 1.0 / 256)


@pytest.mark.parametrize("meta", [m for m in golden_cases() if m["npz"]], ids=lambda m: m["name"])
def test_blast_ic_matches_reference(built, meta):
    import psgb
    from conftest import load_golden
    cfg = psgb.make_config(dims=meta["dims"], nx=meta["n"])
    g = psgb.Grid(cfg)
    V = psgb.blast_state(cfg, g, meta["p_amb"], meta["p_in"], meta["r_in"], meta["noise"],
                         meta["seed"])
    v0, _ = load_golden(meta)
    if meta["dims"] == 2:
        act = V[:, 0, 2:-2, 2:-2]
    else:
        act = V[:, 2:-2, 2:-2, 2:-2]
    assert np.array_equal(act, v0)


@pytest.mark.parametrize("bad", [dict(dims=1), dict(nvar=7), dict(limiter="mc", nx=(3, 64, 1)),
                                 dict(nx=(0, 64, 1)), dict(nx=(64, -4, 1)),
                                 dict(bc=["periodic", "outflow", "outflow", "outflow",
                                          "outflow", "outflow"])])
def test_bad_config_rejected_without_gpu(built, bad):
    import psgb
    kw = dict(dims=2, nx=(64, 64, 1))
    kw.update(bad)
    if kw["dims"] == 1:
        kw["nx"] = (64, 1, 1)
    cfg = psgb.make_config(**kw)
    ctx = ctypes.c_void_p()
    rc = psgb.lib().ps_create(ctypes.byref(cfg), ctypes.byref(ctx))
    assert rc == -1
    assert psgb.lib().ps_last_error()
    assert not ctx.value


def test_wind_host_helpers_match_oracle(built):
    """ps_init_wind (Init() at the volume centroids) and the synthetic
    flux-file values equal the oracle's, which equal the reference's."""
    import psgb
    from oracle import wind_oracle, synthetic_flux
    cfg = psgb.make_wind_config(48, 24)
    w = psgb.make_wind()
    g = psgb.WindGrid(cfg)
    V = psgb.wind_state(cfg, w, g)
    o = wind_oracle(48, 24)
    assert np.array_equal(V, o.V)
    fr, ft, fp = psgb.wind_flux(cfg, w, g)
    ofr, oft, ofp = synthetic_flux(o.grid(0), o.grid(1), o.ntot)
    assert np.array_equal(fr, ofr) and np.array_equal(ft, oft) and np.array_equal(fp, ofp)
    assert np.count_nonzero(fr) == 48 * 24  # one bin per active cell


def test_wind_requires_spherical_nvar6(built):
    import psgb
    cfg = psgb.make_config(dims=2, nx=(32, 32, 1), nvar=5)
    cfg.geometry = psgb.SPHERICAL
    ctx = ctypes.c_void_p()
    assert psgb.lib().ps_create(ctypes.byref(cfg), ctypes.byref(ctx)) == -1


@pytest.mark.parametrize("case", ["entropy_cartesian", "nvar7_without_entropy", "nvar6_with_entropy",
                                  "char_cartesian", "multid_cartesian", "ode_cartesian",
                                  "entropy_out_of_range", "cooling_out_of_range"])
def test_numerics_switches_rejected_without_gpu(built, case):
    """The production numerics and the ODE cooling path are built for the
    spherical wind: other combinations are refused before any device work."""
    import psgb
    if case in ("entropy_cartesian", "char_cartesian", "multid_cartesian", "ode_cartesian"):
        cfg = psgb.make_config(dims=2, nx=(32, 32, 1), nvar=7 if case == "entropy_cartesian" else 5)
    else:
        cfg = psgb.make_wind_config(32, 16)
    if case == "entropy_cartesian":
        cfg.entropy_switch = 2
    elif case == "nvar7_without_entropy":
        cfg.nvar = 7
    elif case == "nvar6_with_entropy":
        cfg.entropy_switch = 2
        cfg.nvar = 6
    elif case == "char_cartesian":
        cfg.char_limiting = 1
    elif case == "multid_cartesian":
        cfg.shock_flattening = 1
    elif case == "ode_cartesian":
        cfg.cooling = 2
    elif case == "entropy_out_of_range":
        cfg.entropy_switch = 3
    else:
        cfg.cooling = 3
    ctx = ctypes.c_void_p()
    assert psgb.lib().ps_create(ctypes.byref(cfg), ctypes.byref(ctx)) == -1
    assert psgb.lib().ps_last_error()
    assert not ctx.value


def test_wind_host_helpers_with_three_ghost_zones_and_entropy(built):
    """MULTID contexts carry 3 ghost zones per side (GetNghost): the host
    grid, initial state (with the entropy s = p / rho^gamma of the entropy
    switch) and flux arrays follow, matching the oracle's."""
    import psgb
    from oracle import wind_oracle, synthetic_flux
    cfg = psgb.make_wind_config(40, 20, char_limiting=1, shock_flattening=1, entropy_switch=2)
    assert psgb.nghost(cfg) == 3 and cfg.nvar == 7
    w = psgb.make_wind()
    g = psgb.WindGrid(cfg)
    assert g.ntot[:2] == [46, 26]
    V = psgb.wind_state(cfg, w, g)
    o = wind_oracle(40, 20, char_limiting=1, shock_flattening=1, entropy_switch=2)
    assert o.ngh[:2] == [3, 3]
    assert np.array_equal(V[:6], o.V[:6])
    act = (slice(3, -3), slice(3, -3))
    assert np.allclose(V[6, 0][act], o.V[6, 0][act], rtol=1e-15, atol=0)
    fr, ft, fp = psgb.wind_flux(cfg, w, g)
    ofr, oft, ofp = synthetic_flux(o.grid(0), o.grid(1), o.ntot, ngh=3)
    assert np.array_equal(fr, ofr) and np.array_equal(ft, oft)
