"""Readers of the SIROCCO hand-off files (host C, no GPU): the directional
flux files the reference read in the golden wind run, and py_heatcool.dat /
prefactors.dat written here in the reference's column formats
(Src/LineDriven/line_connect.c:43-497)."""
import os

import numpy as np
import pytest


def _grid(nr=24, nt=16):
    import psgb
    cfg = psgb.make_wind_config(nr, nt)
    return cfg, psgb.WindGrid(cfg)


def test_flux_files_round_trip(built, tmp_path):
    import psgb
    from make_golden import write_flux_files
    cfg, g = _grid()
    write_flux_files(str(tmp_path), cfg.nx[0], cfg.nx[1])
    fr, ft, fp, matched = psgb.read_sirocco_fluxes(cfg, g, str(tmp_path))
    w = psgb.make_wind()
    er, et, ep = psgb.wind_flux(cfg, w, g)
    assert matched == cfg.nx[0] * cfg.nx[1]
    assert fr.shape == er.shape
    assert np.array_equal(fr, er) and np.array_equal(ft, et) and np.array_equal(fp, ep)


def _write_heatcool(path, g, cfg, xi, tr, skip=()):
    with open(path, "w") as f:
        f.write("i j rcen thetacen vol temp t_r xi ne heat_xray heat_comp heat_lines heat_ff "
                "cool_comp cool_lines cool_ff rho n_h\n")
        for j in range(2, cfg.nx[1] + 2):
            for i in range(2, cfg.nx[0] + 2):
                if (i, j) in skip:
                    continue
                f.write("%d %d %.10e %.10e 1.0 1e4 %.10e %.10e 1 0 0 0 0 0 0 0 1e-14 1e10\n"
                        % (i - 2, j - 2, g.x(0)[i] * 1e9, g.x(1)[j], tr[j, i], xi[j, i]))


def test_heatcool_and_prefactor_files(built, tmp_path):
    import psgb
    cfg, g = _grid()
    n0, n1 = cfg.nx[0] + 4, cfg.nx[1] + 4
    rng = np.random.default_rng(1)
    xi_f = 10 ** rng.uniform(-0.5, 5, (n1, n0))
    tr_f = 10 ** rng.uniform(2.5, 8, (n1, n0))
    _write_heatcool(tmp_path / "py_heatcool.dat", g, cfg, xi_f, tr_f, skip={(5, 7)})
    xi = np.full((n1, n0), -1.0)
    tr = np.full((n1, n0), -1.0)
    m = psgb.read_sirocco_heatcool(cfg, g, str(tmp_path / "py_heatcool.dat"), xi, tr)
    assert m == cfg.nx[0] * cfg.nx[1] - 1
    act = (slice(2, -2), slice(2, -2))
    want_xi = np.maximum(np.array(["%.10e" % v for v in xi_f.ravel()], float).reshape(xi_f.shape), 1.0)
    want_tr = np.maximum(np.array(["%.10e" % v for v in tr_f.ravel()], float).reshape(tr_f.shape), 1e3)
    mask = np.ones((n1, n0), bool)
    mask[7, 5] = False
    sel = np.zeros((n1, n0), bool)
    sel[act] = True
    assert np.array_equal(xi[sel & mask], want_xi[sel & mask])
    assert np.array_equal(tr[sel & mask], want_tr[sel & mask])
    assert xi[7, 5] == -1.0 and np.all(xi[~sel] == -1.0)
    # prefactors.dat: i rcen j thetacen dens comp_h comp_c xray_h brem_c line_c xi_ion
    pre_f = rng.uniform(0.5, 2.0, (6, n1, n0))
    with open(tmp_path / "prefactors.dat", "w") as f:
        f.write("i rcen j thetacen dens comp_h comp_c xray_h brem_c line_c xi_ion\n")
        for j in range(2, cfg.nx[1] + 2):
            for i in range(2, cfg.nx[0] + 2):
                f.write("%d %.10e %d %.10e 1e-14 %s\n" % (i - 2, g.x(0)[i] * 1e9, j - 2, g.x(1)[j],
                                                          " ".join("%.15e" % v for v in pre_f[:, j, i])))
    pre = np.ones((6, n1, n0))
    m = psgb.read_sirocco_prefactors(cfg, g, str(tmp_path / "prefactors.dat"), pre)
    assert m == cfg.nx[0] * cfg.nx[1]
    want = np.array(["%.15e" % v for v in pre_f.ravel()], float).reshape(pre_f.shape)
    assert np.array_equal(pre[:, sel], want[:, sel])
    assert np.all(pre[:, ~sel] == 1.0)


def test_bad_files_are_rejected(built, tmp_path):
    import psgb
    cfg, g = _grid()
    with pytest.raises(RuntimeError):
        psgb.read_sirocco_fluxes(cfg, g, str(tmp_path))          # no files
    (tmp_path / "py_heatcool.dat").write_text("header\n1 2 3\n")
    with pytest.raises(RuntimeError):
        psgb.read_sirocco_heatcool(cfg, g, str(tmp_path / "py_heatcool.dat"),
                                   np.zeros((20, 28)), np.zeros((20, 28)))


def test_force_multiplier_table_file(built, tmp_path):
    """M_UV_data.dat (read with KRAD = ALPHARAD = 999) in the layout the
    golden generator writes for the reference: the reader places every row
    and returns the table's t values and each cell's M as written."""
    import psgb
    from make_golden import write_mfit_file
    from oracle import synthetic_mfit
    cfg, g = _grid()
    write_mfit_file(str(tmp_path), cfg.nx[0], cfg.nx[1])
    t, m, matched = psgb.read_m_uv_fit(cfg, g, str(tmp_path / "M_UV_data.dat"))
    et, em = synthetic_mfit(g.x(0), g.x(1), (cfg.nx[0] + 4, cfg.nx[1] + 4, 1))
    assert matched == cfg.nx[0] * cfg.nx[1]
    assert np.array_equal(t, et)
    assert np.array_equal(m[:, 2:-2, 2:-2], em[:, 0, 2:-2, 2:-2])
    assert np.all(m[:, :2] == 1.0)          # ghost rows keep the caller's values
    with pytest.raises(RuntimeError):       # more points than room for them
        psgb.read_m_uv_fit(cfg, g, str(tmp_path / "M_UV_data.dat"), max_points=4)


def test_dense_flux_matches_the_golden_generator(built):
    """The dense synthetic flux of the library (every bin filled) is the one
    the golden reference run read from its flux files."""
    import psgb
    from oracle import synthetic_flux
    cfg, g = _grid()
    w = psgb.make_wind()
    fr, ft, fp = psgb.wind_flux(cfg, w, g, dense=True)
    er, et, ep = synthetic_flux(g.x(0), g.x(1), g.ntot, l_uv=w.l_star * w.f_uv, dense=True)
    assert np.array_equal(fr, er) and np.array_equal(ft, et) and np.array_equal(fp, ep)
    assert np.count_nonzero(fr[:, 0, 2:-2, 2:-2]) > 30 * cfg.nx[0] * cfg.nx[1]
