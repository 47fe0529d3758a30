"""The wind with SIROCCO hand-off data (per-cell xi, radiation temperature
and rate prefactors, as read_sirocco_heatcool provides them) on the GPU
against the oracle; the learned cooling step leaves such cells to the
reference method, so its run is identical to the plain one."""
import numpy as np
import pytest

from conftest import rel_l1

pytestmark = pytest.mark.gpu

NR, NT = 64, 32


def _data(seed=2):
    import psgb
    cfg = psgb.make_wind_config(NR, NT)
    n0, n1 = NR + 4, NT + 4
    rng = np.random.default_rng(seed)
    xi = 10 ** rng.uniform(0.0, 6.0, (1, n1, n0))
    tr = 10 ** rng.uniform(6.0, 8.0, (1, n1, n0))
    pre = rng.uniform(0.5, 2.0, (6, 1, n1, n0))
    return cfg, xi, tr, pre


def _gpu(xi, tr, pre):
    import psgb
    s = psgb.wind_model_solver(dict(grid=(NR, NT), l_star=1e37, krad=0.2, alpharad=-0.6))
    s.set_sirocco(xi, tr, pre)
    return s


def test_sirocco_data_matches_oracle(built):
    from oracle import wind_oracle
    _, xi, tr, pre = _data()
    from oracle import lib as olib
    s = _gpu(xi, tr, pre)
    o = wind_oracle(NR, NT)
    o.set_sirocco(xi, tr, pre)
    # start past t = 3, where BLONDIN takes xi and T_r from the per-cell data
    s.set_time(3.5, 1e-4, 0)
    olib().or_set_time(o.s, 3.5, 1e-4, 0)
    done = 0
    for step in (2, 20, 80):
        s.run(step - done)
        o.run(step - done)
        done = step
        r = rel_l1(s.get_state()[:, 0, 2:-2, 2:-2], o.active())
        print("step", step, "t", s.time()[0], "relative L1 per variable", r)
        assert np.all(r <= 1e-8), r
    # the data matter: without prefactors the state differs
    plain = psgb_plain = None
    import psgb
    plain = psgb.wind_model_solver(dict(grid=(NR, NT), l_star=1e37, krad=0.2, alpharad=-0.6))
    plain.set_sirocco(xi, tr, None)
    plain.set_time(3.5, 1e-4, 0)
    plain.run(80)
    assert np.max(rel_l1(plain.get_state(), s.get_state())) > 1e-6


def test_surrogate_leaves_prefactor_cells_to_the_reference(built):
    import psgb
    cfg, xi, tr, pre = _data(3)
    a = _gpu(xi, tr, pre)
    b = _gpu(xi, tr, pre)
    sg = psgb.Surrogate((-2, 4, -1, -5), (16, 9, 14, 0))
    psgb.lib().ps_set_surrogate(b.ctx, sg.h, 1)
    a.run(30)
    b.run(30)
    assert np.array_equal(a.get_state(), b.get_state())
    st = sg.stats()
    assert st[0] == 0 and st[2] > 0
