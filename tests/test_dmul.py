"""The binary64 product on the integer pipes (csrc/ps_dmul.cuh) that the
wind stage kernels use in place of the FP64 unit, and its exact halving
and quartering, against the hardware multiply, bit for bit.

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
