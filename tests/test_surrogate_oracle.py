"""CPU checks of the surrogate's oracles: the numpy network's gradient
formulas against central finite differences, its bfloat16 rounding, and
the BLONDIN point solve against the whole-grid cooling step of the oracle."""
import numpy as np
import pytest

import mlp_oracle as M


def _params(seed=0):
    rng = np.random.default_rng(seed)
    p = np.concatenate([rng.uniform(-0.5, 0.5, 256), rng.uniform(-0.5, 0.5, 64),
                        rng.uniform(-0.125, 0.125, 4096), rng.uniform(-0.125, 0.125, 64),
                        rng.uniform(-0.125, 0.125, 64), [0.01]])
    assert len(p) == M.N_PARAMS
    return p


def test_bf16_rounding():
    # bfloat16 keeps 8 significant bits: the spacing above 1 is 2^-7
    x = np.array([1.0, 1.00390625, 1.001953125, 1.005859375, 1.01171875, -3.14159, 0.0])
    r = M.bf16(x)
    # 1 + 2^-8 and 1 + 1.5 * 2^-7 are ties: they go to the even neighbour
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 and r[3] == 1.0078125
    assert r[4] == 1.015625
    assert abs(r[5] + 3.140625) < 1e-12 and r[6] == 0.0


def test_gradient_formulas_finite_differences():
    rng = np.random.default_rng(1)
    p = _params(1)
    u = rng.uniform(-1, 1, (37, 4))
    t = rng.uniform(-0.3, 0.3, 37)
    loss, g = M.loss_grad(p, u, t, exact=True)
    idx = np.concatenate([rng.choice(256, 6), 256 + rng.choice(64, 4), 320 + rng.choice(4096, 8),
                          4416 + rng.choice(64, 4), 4480 + rng.choice(64, 4), [4544]])
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (M.loss_grad(pp, u, t, exact=True)[0] - M.loss_grad(pm, u, t, exact=True)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_rounded_gradient_close_to_exact():
    rng = np.random.default_rng(2)
    p = _params(2)
    u = rng.uniform(-1, 1, (256, 4))
    t = rng.uniform(-0.3, 0.3, 256)
    _, g0 = M.loss_grad(p, u, t, exact=True)
    _, g1 = M.loss_grad(p, u, t)
    assert np.linalg.norm(g1 - g0) < 0.05 * np.linalg.norm(g0)


def test_blondin_point_matches_grid_cooling(built):
    from oracle import wind_oracle, blondin_points, WIND
    o = wind_oracle(32, 16)
    o.run(41)
    V0 = o.active().copy()
    t, dt, _ = o.time()
    rho = V0[0] * WIND["unit_density"]
    prs = V0[4] * WIND["unit_density"] * WIND["unit_velocity"] ** 2
    kMP, kKB = 1.67262171e-24, 1.3806505e-16
    nH = rho / (1.43 * kMP)
    n = rho / (WIND["mu"] * kMP)
    T = (prs / (2.0 / 3.0)) * (2.0 / 3.0) / (n * kKB)
    r = o.grid(0)[2:-2] * WIND["unit_length"]
    xi = WIND["l_star"] * WIND["f_x"] / nH / r[None, :] ** 2
    tup = np.stack([nH.ravel(), T.ravel(), (xi * np.ones_like(T)).ravel(),
                    np.full(T.size, dt)], axis=1)
    Tp = blondin_points(tup, tx=WIND["t_x"], mu=WIND["mu"])
    o.cooling(dt, t)
    V1 = o.active()
    n1 = V1[0] * WIND["unit_density"] / (WIND["mu"] * kMP)
    T1 = V1[4] * WIND["unit_density"] * WIND["unit_velocity"] ** 2 / (n1 * kKB)
    rel = np.abs(Tp - T1.ravel()) / T1.ravel()
    assert rel.max() < 1e-4, rel.max()


def test_constant_xi_cooling_matches_point_solve(built):
    """The oracle's cooling step at constant xi (3-D Cartesian) against the
    point solve of every cell."""
    from oracle import Oracle, blondin_points
    import psgb
    cp = psgb.COOL_PARAMS
    cfg = psgb.cube_config((8, 6, 4))
    V = psgb.cube_state(cfg, psgb.Grid(cfg), seed=7)
    o = Oracle(dims=3, nx=(8, 6, 4), nvar=5, limiter="mc", solver="hllc", bc="periodic",
               cooling=1, params=dict(unit_density=cp["unit_density"],
                                      unit_length=cp["unit_length"],
                                      unit_velocity=cp["unit_velocity"], mu=cp["mu"],
                                      t_x=cp["t_x"], xi_const=cp["xi"]))
    o.V[...] = V
    a = o.active().copy()
    kMP, kKB = 1.67262171e-24, 1.3806505e-16
    rho = a[0] * cp["unit_density"]
    prs = a[4] * cp["unit_density"] * cp["unit_velocity"] ** 2
    n = rho / (cp["mu"] * kMP)
    T = (prs / (2.0 / 3.0)) * (2.0 / 3.0) / (n * kKB)
    dt = 1e-2
    tup = np.stack([(rho / (1.43 * kMP)).ravel(), T.ravel(), np.full(T.size, cp["xi"]),
                    np.full(T.size, dt * cp["unit_length"] / cp["unit_velocity"])], axis=1)
    Tp = blondin_points(tup, tx=cp["t_x"], mu=cp["mu"])
    o.cooling(dt, 10.0)
    b = o.active()
    T1 = b[4] * cp["unit_density"] * cp["unit_velocity"] ** 2 / (n * kKB)
    rel = np.abs(Tp - T1.ravel()) / T1.ravel()
    assert rel.max() < 1e-4, rel.max()
    assert np.any(np.abs(T1 - T) > 1e-3 * T)
