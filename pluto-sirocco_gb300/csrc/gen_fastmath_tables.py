"""Writes ps_fastmath_tables.cuh: the tables of the table-driven exp and
log in ps_fastmath.cuh, computed with mpmath at 120 bits and rounded to
double (round to nearest).

    python pluto-sirocco_gb300/csrc/gen_fastmath_tables.py

exp (after P. T. P. Tang, "Table-driven implementation of the exponential
function in IEEE floating-point arithmetic", ACM TOMS 15(2), 1989):
  x = (256 m + j) ln2/256 + r,  exp(x) = 2^m 2^(j/256) e^r
  kExpHi[j] = RN(2^(j/256)),  kExpLo[j] = RN(2^(j/256) - kExpHi[j])
  kExpL1 + kExpL2 = ln2/256 (Cody-Waite split, kExpL1 = RN(ln2/256)).

log (after P. T. P. Tang, "Table-driven implementation of the logarithm
function in IEEE floating-point arithmetic", ACM TOMS 16(4), 1990):
  x = 2^e m,  F_j = 1 + j/256 nearest to m,  r = (m - F_j) / F_j,
  log(x) = e ln2 + log(F_j) + log1p(r)
  kLogInv[j] = RN(1/F_j); kLogHi[j] = log(F_j) rounded to a multiple of
  2^-42 (so that e ln2_hi + kLogHi[j] is exact for |e| < 2^11);
  kLogLo[j] = RN(log(F_j) - kLogHi[j]); the same split for ln2.

The polynomials are the Taylor series of e^r - 1 and log1p(r) truncated
where the remainder falls below 2^-60 on the reduced interval.
"""
import os

import mpmath

mpmath.mp.prec = 120
HERE = os.path.dirname(os.path.abspath(__file__))


def rn(v):
    """Round an mpf to the nearest double."""
    return float(mpmath.mpf(v))


def on_grid(v, bits):
    """v rounded to a multiple of 2^-bits."""
    s = mpmath.mpf(2) ** bits
    return rn(mpmath.nint(v * s) / s)


def lit(x):
    return x.hex()


def main():
    out = []
    out.append("// ps_fastmath_tables.cuh -- generated by gen_fastmath_tables.py; do not edit.")
    out.append("// Tables of the table-driven exp and log of ps_fastmath.cuh (values in")
    out.append("// hexadecimal floating point, rounded to nearest from 120-bit mpmath).")
    out.append("#pragma once")
    out.append("")
    out.append("namespace ps {")
    out.append("namespace fm {")
    ln2 = mpmath.log(2)
    l1 = rn(ln2 / 256)
    l2 = rn(ln2 / 256 - mpmath.mpf(l1))
    out.append(f"constexpr double kExpInvL = {lit(rn(256 / ln2))};  // 256 / ln 2")
    out.append(f"constexpr double kExpL1 = {lit(l1)};  // ln2 / 256, leading part")
    out.append(f"constexpr double kExpL2 = {lit(l2)};  // ln2 / 256 - kExpL1")
    ln2_hi = on_grid(ln2, 42)
    ln2_lo = rn(ln2 - mpmath.mpf(ln2_hi))
    out.append(f"constexpr double kLn2Hi = {lit(ln2_hi)};  // ln 2 on the 2^-42 grid")
    out.append(f"constexpr double kLn2Lo = {lit(ln2_lo)};  // ln 2 - kLn2Hi")
    hi, lo = [], []
    for j in range(256):
        v = mpmath.mpf(2) ** (mpmath.mpf(j) / 256)
        h = rn(v)
        hi.append(h)
        lo.append(rn(v - mpmath.mpf(h)))
    inv, lhi, llo = [], [], []
    for j in range(257):
        F = 1 + mpmath.mpf(j) / 256
        inv.append(rn(1 / F))
        lf = mpmath.log(F)
        h = on_grid(lf, 42)
        lhi.append(h)
        llo.append(rn(lf - mpmath.mpf(h)))

    def table(name, vals, what):
        out.append(f"// {what}")
        out.append(f"static __device__ const double {name}[{len(vals)}] = {{")
        for k in range(0, len(vals), 3):
            out.append("    " + ", ".join(lit(v) for v in vals[k:k + 3]) + ",")
        out.append("};")

    table("kExpHi", hi, "2^(j/256), rounded")
    table("kExpLo", lo, "2^(j/256) - kExpHi[j], rounded")
    table("kLogInv", inv, "1 / (1 + j/256), rounded")
    table("kLogHi", lhi, "log(1 + j/256) on the 2^-42 grid")
    table("kLogLo", llo, "log(1 + j/256) - kLogHi[j], rounded")
    out.append("")
    out.append("}  // namespace fm")
    out.append("}  // namespace ps")
    with open(os.path.join(HERE, "ps_fastmath_tables.cuh"), "w") as f:
        f.write("\n".join(out) + "\n")


if __name__ == "__main__":
    main()
