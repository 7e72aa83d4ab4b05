"""The correctly rounded pow of the material laws (dumux_gb300/csrc/crpow.cuh), host build.

The oracle library compiles the same header for the host; these tests check it against
exact rational arithmetic, against 200-bit arithmetic (mpmath, where installed) and
against the host C library's pow, which the reference's laws call (std::pow).
"""
from fractions import Fraction

import numpy as np
import pytest

import oracle

CR, LIBM = oracle.POW_CORRECTLY_ROUNDED, oracle.POW_LIBM


def test_exact_midpoints_round_to_even():
    # odd x with 18 significant bits: x^3 has exactly 54 bits, a binary64 rounding midpoint
    xs = np.array([220001, 220003, 233333, 240001, 250001, 262141], dtype=np.float64)
    got = oracle.pow_batch(xs, 3.0, CR)
    want = [float(Fraction(int(v)) ** 3) for v in xs]   # Fraction -> float rounds to even
    assert list(got) == want
    # x^(3/2) with x = t^2: t^3 is the same kind of midpoint
    got = oracle.pow_batch(xs * xs, 1.5, CR)
    assert list(got) == want


@pytest.mark.parametrize("y", [2.0, 3.0, 4.0, 5.0, -2.0, -3.0, -4.0])
def test_integer_powers_of_short_significands_are_exact_roundings(y):
    rng = np.random.default_rng(int(abs(y) * 10))
    x = rng.integers(1, 2 ** 20, 4000).astype(np.float64) * 2.0 ** rng.integers(-30, 30, 4000)
    got = oracle.pow_batch(x, y, CR)
    k = int(y)
    want = [float(Fraction(v) ** k) for v in x]
    assert np.array_equal(got, np.array(want))


def test_special_values_follow_c99():
    sv = [0.0, -0.0, 1.0, -1.0, np.inf, -np.inf, np.nan, 2.0, -2.0, 0.5, -0.5, 3.0, -3.0, 1e-310, 5e-324,
          1.7e308, 0.25, -0.25]
    xs, ys = (a.ravel() for a in np.meshgrid(sv, sv))
    a = oracle.pow_batch(xs, ys, CR)
    b = oracle.pow_batch(xs, ys, LIBM)
    same = ((a == b) & (np.signbit(a) == np.signbit(b))) | (np.isnan(a) & np.isnan(b))
    assert same.all(), [(x, y, u, v) for x, y, u, v, s in zip(xs, ys, a, b, same) if not s]


def test_agrees_with_200_bit_arithmetic():
    mp = pytest.importorskip("mpmath")
    mp.mp.prec = 200
    rng = np.random.default_rng(0)
    n = 6000
    x = np.exp(rng.uniform(-30, 30, n))
    y = rng.uniform(-12, 12, n)
    x[:2000] = rng.uniform(0, 1, 2000)                    # saturations
    y[:1000] = rng.choice([-0.5, 4.0, 2.0, 3.0, -1.5, 1.0 / 2.7, 2.7], 1000)
    got = oracle.pow_batch(x, y, CR)
    want = np.array([float(mp.power(mp.mpf(a), mp.mpf(b))) for a, b in zip(x, y)])
    assert np.array_equal(got, want)


def test_c_library_pow_differs_only_where_it_misrounds():
    """The host C library's pow is not correctly rounded in binary64: on the laws' domain
    it differs from the correctly rounded value in ~0.1% of the arguments, by one ulp.
    Each difference is checked against 200-bit arithmetic where mpmath is installed."""
    rng = np.random.default_rng(1)
    sw = rng.uniform(0, 1, 200000)
    for y in (-0.5, 4.0, 2.0, -1.5, 3.0, 1.0 / 2.7, 1.0 - 1.0 / 2.7):
        a = oracle.pow_batch(sw, y, CR)
        b = oracle.pow_batch(sw, y, LIBM)
        diff = np.nonzero(a != b)[0]
        assert len(diff) <= 0.005 * len(sw)
        ulps = np.abs(a[diff].view(np.int64) - b[diff].view(np.int64))
        assert np.all(ulps <= 1)
        try:
            import mpmath as mp
        except ImportError:
            continue
        mp.mp.prec = 200
        for i in diff[:40]:
            assert a[i] == float(mp.power(mp.mpf(sw[i]), mp.mpf(y)))
