"""Generates crpow_tables.inc, the tables of the correctly rounded pow (crpow.cuh).

Run with mpmath (200-bit arithmetic); the generated file is committed, so building the
library does not need mpmath.

Log table, 256 entries indexed by the top 8 fraction bits of x's significand m in [1, 2):
  entries i < 106 (m < 1.4140625): c_i = 1/(1 + (i + 1/2)/256) rounded to 9 significant
  bits, applied to m itself;
  entries i >= 106: the significand is halved (m' = m/2 in [0.707, 1), exponent + 1) and
  c_i = 1/((1 + (i + 1/2)/256)/2) rounded to 9 significant bits.
  With 9-bit c_i the reduced argument r = m'*c_i - 1 is exact in binary64 (checked
  below over every interval), |r| < 2^-8.
  T_i = -log(c_i) as a double-double (hi, lo).
Exp table, 128 entries: 2^(j/128) as a double-double (hi, lo).
Splitting constants of ln 2 and ln 2 / 128 for exact Cody-Waite products, and
double-double values of 1/3, 1/5, 1/6, 1/24 and 1/120 for the accurate polynomials.
"""
import os
from fractions import Fraction

import mpmath as mp

mp.mp.prec = 200
HERE = os.path.dirname(os.path.abspath(__file__))


def round_bits(v, bits):
    """v (mpf > 0) rounded to `bits` significant bits, as a Python float."""
    e = int(mp.floor(mp.log(v, 2)))
    scale = mp.mpf(2) ** (bits - 1 - e)
    return float(mp.nint(v * scale) / scale)


def dd(v):
    hi = float(v)
    lo = float(v - mp.mpf(hi))
    return hi, lo


def split_hi(v, bits):
    """v rounded to `bits` significant bits (so that small integer multiples stay exact)."""
    return round_bits(v, bits) if v > 0 else -round_bits(-v, bits)


def check_exact(lo, hi, c, ulp_m):
    """r = m*c - 1 exact in binary64 for every m in [lo, hi) on the grid ulp_m."""
    cf = Fraction(c)
    m, e = mp.frexp(c)
    ulp_c = Fraction(2) ** (int(e) - 9)         # c has at most 9 significant bits
    assert Fraction(c) / ulp_c == int(Fraction(c) / ulp_c)
    g = ulp_m * ulp_c
    rmax = max(abs(Fraction(lo) * cf - 1), abs(Fraction(hi) * cf - 1))
    assert rmax <= Fraction(2) ** 53 * g, (lo, hi, c)
    return float(rmax)


def main():
    lines = ["// Generated by gen_crpow_tables.py (mpmath, 200-bit arithmetic). Do not edit.", ""]
    invc, thi, tlo = [], [], []
    rmax_all = 0.0
    for i in range(256):
        mid = 1 + (mp.mpf(i) + mp.mpf(0.5)) / 256
        lo, hi = Fraction(256 + i, 256), Fraction(256 + i + 1, 256)
        if i < 106:
            c = round_bits(1 / mid, 9)
            rmax_all = max(rmax_all, check_exact(lo, hi, c, Fraction(1, 2 ** 52)))
        else:
            c = round_bits(2 / mid, 9)
            rmax_all = max(rmax_all, check_exact(lo / 2, hi / 2, c, Fraction(1, 2 ** 53)))
        t = -mp.log(mp.mpf(c))
        h, l = dd(t)
        invc.append(c)
        thi.append(h)
        tlo.append(l)
    assert rmax_all < 2.0 ** -8, rmax_all
    e2hi, e2lo = [], []
    for j in range(128):
        h, l = dd(mp.mpf(2) ** (mp.mpf(j) / 128))
        e2hi.append(h)
        e2lo.append(l)

    def arr(name, vals):
        out = [f"DXG_CRPOW_TABLE double {name}[{len(vals)}] = {{"]
        for k in range(0, len(vals), 4):
            out.append("    " + ", ".join(v.hex() for v in vals[k:k + 4]) + ",")
        out.append("};")
        return out

    ln2 = mp.log(2)
    # E * LN2_HI exact for |E| < 2^11; LN2_LO / LN2_LL the rest of ln 2
    ln2_hi = split_hi(ln2, 42)
    ln2_lo = float(ln2 - ln2_hi)
    ln2_ll = float(ln2 - ln2_hi - ln2_lo)
    # ln2/128 for the exp reduction: n * L1 exact for |n| < 2^19
    l1 = split_hi(ln2 / 128, 34)
    l2 = float(ln2 / 128 - l1)
    l3 = float(ln2 / 128 - l1 - l2)
    inv_l = float(128 / ln2)
    consts = {"kLn2Hi": ln2_hi, "kLn2Lo": ln2_lo, "kLn2Ll": ln2_ll, "kL1": l1, "kL2": l2, "kL3": l3,
              "kInvL": inv_l}
    for name, den in (("Inv3", 3), ("Inv5", 5), ("Inv6", 6), ("Inv24", 24), ("Inv120", 120)):
        h, l = dd(mp.mpf(1) / den)
        consts[f"k{name}Hi"] = h
        consts[f"k{name}Lo"] = l
    for k, v in consts.items():
        lines.append(f"constexpr double {k} = {v.hex()};  // {v!r}")
    lines.append(f"// largest |r| of the log reduction: {rmax_all!r}")
    lines.append("")
    lines += arr("kLogInvC", invc)
    lines += arr("kLogTHi", thi)
    lines += arr("kLogTLo", tlo)
    lines += arr("kExp2Hi", e2hi)
    lines += arr("kExp2Lo", e2lo)
    with open(os.path.join(HERE, "crpow_tables.inc"), "w") as f:
        f.write("\n".join(lines) + "\n")
    print("rmax", rmax_all, "-> written")


if __name__ == "__main__":
    main()
