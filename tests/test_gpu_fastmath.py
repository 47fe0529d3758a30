"""The table-driven exp and log of the stage kernels and the learned step's
judge (csrc/ps_fastmath.cuh) against numpy's (glibc) and CUDA's on the
same arguments: within 2 ulp of each everywhere, and equal to the
correctly rounded value on almost every argument (numpy's exp and log are
within 1 ulp of it, so two results 2 ulp apart are the most two correct
implementations can differ)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ulps(a, b):
    ia, ib = a.view(np.int64), b.view(np.int64)
    return np.abs(ia - ib)


def _run(op, x):
    import psgb
    fast, ref = np.empty_like(x), np.empty_like(x)
    P = psgb.probe()
    dp = lambda a: a.ctypes.data_as(psgb.ctypes.POINTER(psgb.ctypes.c_double))
    assert P.ps_probe_fastmath(op, dp(x), dp(fast), dp(ref), len(x)) == 0
    return fast, ref


def test_fast_exp_within_an_ulp(built):
    rng = np.random.default_rng(11)
    x = np.concatenate([rng.uniform(-700.0, 700.0, 1 << 20),
                        rng.uniform(-1.0, 1.0, 1 << 18),
                        rng.uniform(-1e-6, 1e-6, 1 << 16),
                        [0.0, -0.0, 1e-300, -1e-300, 700.0, -700.0]])
    fast, cuda = _run(0, x)
    want = np.exp(x)
    assert _ulps(fast, want).max() <= 2
    assert _ulps(fast, cuda).max() <= 2
    assert np.mean(_ulps(fast, want) == 0) > 0.99
    # outside |x| <= 700 the function is CUDA's
    y = np.array([701.0, -701.0, 710.0, -745.0, -760.0, np.inf, -np.inf, np.nan])
    fast, cuda = _run(0, y)
    assert np.array_equal(fast, cuda, equal_nan=True)


def test_fast_log_within_an_ulp(built):
    rng = np.random.default_rng(12)
    x = np.concatenate([10.0 ** rng.uniform(-300.0, 300.0, 1 << 20),
                        1.0 + rng.uniform(-1e-3, 1e-3, 1 << 18),
                        1.0 + rng.uniform(-1e-9, 1e-9, 1 << 16),
                        rng.uniform(1.0, 2.0, 1 << 18),
                        [1.0, 2.0, 0.5, np.nextafter(1.0, 2.0), np.nextafter(1.0, 0.0),
                         np.finfo(float).tiny, np.finfo(float).max]])
    fast, cuda = _run(1, x)
    want = np.log(x)
    assert _ulps(fast, want).max() <= 2
    assert _ulps(fast, cuda).max() <= 2
    assert np.mean(_ulps(fast, want) == 0) > 0.99
    # zero, subnormal, negative, infinite and NaN arguments are CUDA's
    y = np.array([0.0, -0.0, 1e-310, -1.0, np.inf, -np.inf, np.nan])
    fast, cuda = _run(1, y)
    assert np.array_equal(fast, cuda, equal_nan=True)
