"""The binary64 product on the integer pipes (csrc/ps_dmul.cuh) that the
stage kernels use in place of the FP64 unit, its exact scalings by 1/4,
1/2, 2 and 4 and the product's sign test, against the hardware multiply,
bit for bit.

Five kinds of operand pairs (ps_probe.cu dm_pair): exponents near the
middle of the range; short significands, whose products are exact or exact
ties (round half to even); any bit pattern (subnormals, infinities, NaNs);
products near either end of the normal range; zeros, powers of two and
sign mixes.  Pairs the integer form hands back (`bad`: operands or results
outside the normal range) are counted, not compared: the kernels take the
hardware multiply for them.  On the CPU the same code, compiled for the
host, is held to the host's IEEE multiply.
"""
import ctypes

import pytest


def _check(on_gpu, seed, n):
    import psgb
    out = (ctypes.c_ulonglong * 4)()
    assert psgb.probe().ps_probe_dmul_check(on_gpu, seed, n, out) == 0
    return out[0], out[1], (out[2], out[3])


def test_integer_product_matches_host_multiply(built):
    n = 4_000_000
    mism, bad, first = _check(0, 17, n)
    assert mism == 0, f"first differing pair {first[0]:016x} {first[1]:016x}"
    # the edge kinds hand back (subnormal, infinite, NaN operands; results
    # out of range), the ordinary ones never do
    assert 0.05 * n < bad < 0.4 * n


@pytest.mark.gpu
def test_integer_product_matches_gpu_multiply(built):
    n = 1 << 28
    mism, bad, first = _check(1, 23, n)
    assert mism == 0, f"first differing pair {first[0]:016x} {first[1]:016x}"
    assert 0.05 * n < bad < 0.4 * n


@pytest.mark.gpu
def test_subnormal_state_takes_the_fp64_path_and_matches_oracle(built):
    """Subnormal velocities planted in a fifth of a 64x32 wind's cells make
    the integer products of the stage kernel hand back in the cells that
    read them, which are done again on the FP64 unit; after 10 steps the
    run is within 1e-11 of the oracle started from the same state (the
    planted values change the run: it differs from the unplanted one)."""
    import numpy as np
    import psgb
    from conftest import assert_hydro_close
    from oracle import wind_oracle
    nr, nt, ng = 64, 32, 2
    cfg = psgb.make_wind_config(nr, nt, cooling=0)
    w = psgb.make_wind(line_force=0)
    g = psgb.WindGrid(cfg)
    V = psgb.wind_state(cfg, w, g)
    act = V[:, 0, ng:-ng, ng:-ng].copy()
    rng = np.random.default_rng(3)
    mask = rng.random(act.shape[1:]) < 0.2
    act[2][mask] = np.where(rng.random(mask.sum()) < 0.5, -3e-310, 3e-310)
    act[3][mask] = np.where(rng.random(mask.sum()) < 0.5, -1e-315, 7e-312)
    V[:, 0, ng:-ng, ng:-ng] = act
    runs = {}
    for name, state in (("planted", V), ("plain", psgb.wind_state(cfg, w, g))):
        s = psgb.Solver(cfg, g)
        s.set_state(state)
        s.set_time(0.0, 1e-4, 0)
        s.set_wind(w, None)
        assert s.run(10) & ~0x2 == 0
        runs[name] = s.get_state()[:6, 0, ng:-ng, ng:-ng]
    o = wind_oracle(nr, nt, cooling=0, line_force=0, initial=act)
    o.run(10)
    r = assert_hydro_close(runs["planted"], np.asarray(o.active()), "planted subnormals")
    print("relative L1 per variable against the oracle", r)
    assert not np.array_equal(runs["planted"], runs["plain"])


@pytest.mark.gpu
def test_subnormal_blast_takes_the_fp64_path_and_matches_oracle(built):
    """The same for the Cartesian stage kernels (the blast, MC limiter,
    HLLC): subnormal velocities in a fifth of a 64x64 blast's cells make
    the integer products and the limiter's sign test hand back, and after
    10 steps the run is within 1e-11 of the oracle from the same state."""
    import numpy as np
    import psgb
    from conftest import assert_hydro_close
    from oracle import Oracle
    o = Oracle(dims=2, nx=(64, 64, 1), limiter="mc", solver="hllc", bc="outflow")
    o.init_blast(0.1, 10.0, 0.1, 0.01, 1)
    act = o.active()                     # a view of the oracle's state
    rng = np.random.default_rng(5)
    mask = rng.random(act.shape[1:]) < 0.2
    act[1][mask] = np.where(rng.random(mask.sum()) < 0.5, -3e-310, 3e-310)
    act[2][mask] = np.where(rng.random(mask.sum()) < 0.5, -1e-315, 7e-312)
    cfg = psgb.make_config(dims=2, nx=(64, 64, 1), limiter="mc", solver="hllc", bc="outflow")
    s = psgb.Solver(cfg, psgb.Grid(cfg))
    s.set_state(o.V.copy())
    s.set_time(0.0, 1e-4, 0)
    assert s.run(10) == 0
    o.run(10)
    r = assert_hydro_close(s.get_state()[:, 0, 2:-2, 2:-2], np.asarray(o.active()),
                           "planted subnormals, blast")
    print("relative L1 per variable against the oracle", r)
