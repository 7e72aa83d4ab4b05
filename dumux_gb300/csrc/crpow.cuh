// crpow.cuh -- correctly rounded binary64 pow(x, y), one source for host and device.
//
// The material laws (Brooks-Corey, Van Genuchten) raise saturations to real powers.  The
// reference evaluates them with the host C library's pow, which for binary64 returns the
// correctly rounded result except in rare hard cases; CUDA's pow is accurate to a few ulp
// only.  A numeric-difference Jacobian divides residual differences by ~1e-10, so a single
// ulp of a capillary pressure becomes a 1e-7 relative Jacobian difference.  This pow returns
// the correctly rounded result on host and device alike, so both follow the reference's
// values bit for bit wherever the C library is itself correctly rounded.
//
// Method (written from the published algorithms):
//   * table-driven logarithm after P. T. P. Tang, "Table-driven implementation of the
//     logarithm function in IEEE floating-point arithmetic", ACM TOMS 16(4), 1990:
//     x = 2^E m, r = m c_i - 1 exact (c_i of 9 significant bits, |r| < 2^-8.4),
//     log x = E ln2 - log c_i + log1p(r);
//   * table-driven exponential after Tang, "Table-driven implementation of the exponential
//     function in IEEE floating-point arithmetic", ACM TOMS 15(2), 1989:
//     Y = (128 k + j) ln2/128 + s, exp Y = 2^k 2^(j/128) exp(s), |s| < 2^-8.5;
//   * double-double arithmetic (T. J. Dekker, "A floating-point technique for extending the
//     available precision", Numer. Math. 18, 1971; Knuth's TwoSum) for y log x and the
//     polynomial heads;
//   * Ziv's rounding test (A. Ziv, "Fast evaluation of elementary mathematical functions
//     with correctly rounded last bit", ACM TOMS 17(3), 1991): a fast phase (relative error
//     below 2^-72 for |y| <= 16, tested against 2^-69 + |y| 2^-74) whose result is returned
//     when no rounding boundary lies within its error bound, else an accurate phase
//     (relative error below 2^-100 for moderate |y| log x).  A result that the accurate
//     phase still cannot separate from a rounding midpoint is taken as the exact midpoint
//     and rounded to even (the exact midpoint cases of pow, e.g. x^3 or x^(3/2) of short
//     significands, land there).
// Results in the subnormal range (below 2^-1022) are not guaranteed correctly rounded.
// Special values follow C99 Annex F.  Every operation is written out (explicit fma, and
// __dadd_rn / __dmul_rn on the device), so contraction flags do not change the result.
//
// Tables: crpow_tables.inc, generated by gen_crpow_tables.py with 200-bit arithmetic.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define DXG_CR_HD __host__ __device__ __forceinline__
#define DXG_CR_CALL static __host__ __device__ __noinline__
#else
#define DXG_CR_HD inline
#define DXG_CR_CALL inline
#endif

namespace dxg {
namespace crpow {

#if defined(__CUDACC__)
namespace dev {
#define DXG_CRPOW_TABLE __device__ static const
#include "crpow_tables.inc"
#undef DXG_CRPOW_TABLE
}  // namespace dev
#endif
namespace host {
#define DXG_CRPOW_TABLE static const
#include "crpow_tables.inc"
#undef DXG_CRPOW_TABLE
}  // namespace host

#if defined(__CUDA_ARCH__)
#define DXG_CR(name) ::dxg::crpow::dev::name
#else
#define DXG_CR(name) ::dxg::crpow::host::name
#endif

struct DD {
    double hi, lo;
};

DXG_CR_HD double add(double a, double b)
{
#if defined(__CUDA_ARCH__)
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
}
DXG_CR_HD double mul(double a, double b)
{
#if defined(__CUDA_ARCH__)
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
DXG_CR_HD double sub(double a, double b) { return add(a, -b); }
DXG_CR_HD uint64_t bitsOf(double x)
{
    uint64_t u;
    memcpy(&u, &x, sizeof u);
    return u;
}
DXG_CR_HD double fromBits(uint64_t u)
{
    double x;
    memcpy(&x, &u, sizeof x);
    return x;
}

// a + b = s + e exactly
DXG_CR_HD DD twoSum(double a, double b)
{
    const double s = add(a, b);
    const double bb = sub(s, a);
    const double e = add(sub(a, sub(s, bb)), sub(b, bb));
    return {s, e};
}
// a + b = s + e exactly, |a| >= |b| or a == 0
DXG_CR_HD DD fastTwoSum(double a, double b)
{
    const double s = add(a, b);
    return {s, sub(b, sub(s, a))};
}
// a * b = p + e exactly
DXG_CR_HD DD twoProd(double a, double b)
{
    const double p = mul(a, b);
    return {p, fma(a, b, -p)};
}
// double-double + double-double (absolute error ~2^-105 max(|a|, |b|))
DXG_CR_HD DD ddAdd(DD a, DD b)
{
    const DD s = twoSum(a.hi, b.hi);
    return fastTwoSum(s.hi, add(s.lo, add(a.lo, b.lo)));
}
// double-double * double
DXG_CR_HD DD ddMulD(DD a, double b)
{
    const DD p = twoProd(a.hi, b);
    return fastTwoSum(p.hi, fma(a.lo, b, p.lo));
}
// double-double * double-double
DXG_CR_HD DD ddMul(DD a, DD b)
{
    const DD p = twoProd(a.hi, b.hi);
    return fastTwoSum(p.hi, add(p.lo, add(mul(a.hi, b.lo), mul(a.lo, b.hi))));
}
DXG_CR_HD double scale2(double v, int k)
{
    if (k >= -1022 && k <= 1023) return mul(v, fromBits((uint64_t)(k + 1023) << 52));
    if (k > 1023) return mul(mul(v, 0x1p1000), fromBits((uint64_t)(k - 1000 + 1023) << 52));
    return mul(mul(v, 0x1p-600), fromBits((uint64_t)(k + 600 + 1023) << 52));
}

// x > 0 finite: x = 2^E m', r = m' c_i - 1 (exact), table index i
DXG_CR_HD void reduceLog(double x, int& E, double& r, int& i)
{
    uint64_t u = bitsOf(x);
    E = 0;
    if (u < (1ull << 52)) {   // subnormal
        x = mul(x, 0x1p64);
        u = bitsOf(x);
        E = -64;
    }
    E += (int)(u >> 52) - 1023;
    i = (int)((u >> 44) & 0xFF);
    const uint64_t frac = u & ((1ull << 52) - 1);
    uint64_t mb = frac | (1023ull << 52);   // m in [1, 2)
    if (i >= 106) {                         // m/2 in [0.707, 1), exponent + 1
        mb = frac | (1022ull << 52);
        E += 1;
    }
    r = fma(fromBits(mb), DXG_CR(kLogInvC)[i], -1.0);
}

// E ln2 + T_i + l1p
DXG_CR_HD DD logAssemble(int E, int i, DD l1p, bool accurate)
{
    const double Ed = (double)E;
    if (!accurate) {
        const DD s1 = twoSum(mul(Ed, DXG_CR(kLn2Hi)), DXG_CR(kLogTHi)[i]);
        const DD s2 = twoSum(s1.hi, l1p.hi);
        const double lo =
            add(add(s1.lo, s2.lo), add(fma(Ed, DXG_CR(kLn2Lo), DXG_CR(kLogTLo)[i]), l1p.lo));
        return fastTwoSum(s2.hi, lo);
    }
    const DD e2 = twoProd(Ed, DXG_CR(kLn2Lo));
    const DD eln2 = fastTwoSum(mul(Ed, DXG_CR(kLn2Hi)), e2.hi);
    const DD el = fastTwoSum(eln2.hi, add(eln2.lo, fma(Ed, DXG_CR(kLn2Ll), e2.lo)));
    const DD t = {DXG_CR(kLogTHi)[i], DXG_CR(kLogTLo)[i]};
    return ddAdd(ddAdd(el, t), l1p);
}

// log x as a double-double.  Fast: absolute error below 2^-76; accurate: below 2^-103.
DXG_CR_HD DD logDD(double x, bool accurate)
{
    int E, i;
    double r;
    reduceLog(x, E, r, i);
    if (!accurate) {
        // log1p(r) = r - r^2/2 + r^3 P(r), P = 1/3 - r/4 + ... - r^7/10
        const DD sq = twoProd(r, r);
        const DD a = fastTwoSum(r, mul(-0.5, sq.hi));
        double P = -0.1;
        P = fma(P, r, 1.0 / 9.0);
        P = fma(P, r, -0.125);
        P = fma(P, r, 1.0 / 7.0);
        P = fma(P, r, -1.0 / 6.0);
        P = fma(P, r, 0.2);
        P = fma(P, r, -0.25);
        P = fma(P, r, 1.0 / 3.0);
        const double tail = fma(mul(r, sq.hi), P, mul(-0.5, sq.lo));
        return logAssemble(E, i, fastTwoSum(a.hi, add(a.lo, tail)), false);
    }
    // log1p(r) = r (1 - r/2 + r^2/3 - ... + r^12/13): terms from r^7 on in double
    double q = 1.0 / 13.0;
    q = fma(q, r, -1.0 / 12.0);
    q = fma(q, r, 1.0 / 11.0);
    q = fma(q, r, -0.1);
    q = fma(q, r, 1.0 / 9.0);
    q = fma(q, r, -0.125);
    q = fma(q, r, 1.0 / 7.0);
    DD t = {q, 0.0};
    t = ddAdd(ddMulD(t, r), DD{-DXG_CR(kInv6Hi), -DXG_CR(kInv6Lo)});
    t = ddAdd(ddMulD(t, r), DD{DXG_CR(kInv5Hi), DXG_CR(kInv5Lo)});
    t = ddAdd(ddMulD(t, r), DD{-0.25, 0.0});
    t = ddAdd(ddMulD(t, r), DD{DXG_CR(kInv3Hi), DXG_CR(kInv3Lo)});
    t = ddAdd(ddMulD(t, r), DD{-0.5, 0.0});
    t = ddAdd(ddMulD(t, r), DD{1.0, 0.0});
    return logAssemble(E, i, ddMulD(t, r), true);
}

// exp(Y) = 2^k R, R a double-double in [0.99, 2.02].  Fast: relative error below 2^-78
// (plus the error of Y); accurate: below 2^-103.
DXG_CR_HD DD expDD(DD Y, int& k, bool accurate)
{
    const double nd = rint(mul(Y.hi, DXG_CR(kInvL)));
    const int n = (int)nd;
    const int j = n & 127;
    k = (n - j) / 128;
    const double s1 = fma(-nd, DXG_CR(kL1), Y.hi);   // exact
    const DD t = twoProd(nd, DXG_CR(kL2));
    const DD u = twoSum(s1, -t.hi);
    const double slo = fma(-nd, DXG_CR(kL3), add(sub(u.lo, t.lo), Y.lo));
    const DD S = fastTwoSum(u.hi, slo);
    const DD T2 = {DXG_CR(kExp2Hi)[j], DXG_CR(kExp2Lo)[j]};
    DD em1;
    if (!accurate) {
        // expm1(s) = s + s^2/2 + s^3 (1/6 + s/24 + ... + s^4/5040)
        const DD sq = twoProd(S.hi, S.hi);
        double p = 1.0 / 5040.0;
        p = fma(p, S.hi, 1.0 / 720.0);
        p = fma(p, S.hi, 1.0 / 120.0);
        p = fma(p, S.hi, 1.0 / 24.0);
        p = fma(p, S.hi, 1.0 / 6.0);
        const double c3 = mul(mul(sq.hi, S.hi), p);
        const DD a = fastTwoSum(S.hi, mul(0.5, sq.hi));
        const double rest = add(add(add(a.lo, S.lo), fma(0.5, sq.lo, c3)), mul(S.hi, S.lo));
        em1 = fastTwoSum(a.hi, rest);
        const DD P = twoProd(T2.hi, em1.hi);
        const DD a2 = twoSum(T2.hi, P.hi);
        const double rest2 =
            add(add(a2.lo, P.lo), add(fma(T2.lo, em1.hi, T2.lo), mul(T2.hi, em1.lo)));
        return fastTwoSum(a2.hi, rest2);
    }
    // expm1(s) = s (1 + s/2 + s^2/6 + ... + s^10/11!): terms from s^5/6! on in double
    double q = 1.0 / 39916800.0;
    q = fma(q, S.hi, 1.0 / 3628800.0);
    q = fma(q, S.hi, 1.0 / 362880.0);
    q = fma(q, S.hi, 1.0 / 40320.0);
    q = fma(q, S.hi, 1.0 / 5040.0);
    q = fma(q, S.hi, 1.0 / 720.0);
    DD e = {q, 0.0};
    e = ddAdd(ddMulD(e, S.hi), DD{DXG_CR(kInv120Hi), DXG_CR(kInv120Lo)});
    e = ddAdd(ddMulD(e, S.hi), DD{DXG_CR(kInv24Hi), DXG_CR(kInv24Lo)});
    e = ddAdd(ddMulD(e, S.hi), DD{DXG_CR(kInv6Hi), DXG_CR(kInv6Lo)});
    e = ddAdd(ddMulD(e, S.hi), DD{0.5, 0.0});
    e = ddAdd(ddMulD(e, S.hi), DD{1.0, 0.0});
    em1 = ddMulD(e, S.hi);
    // exp(s_hi + s_lo) - 1 = em1 + s_lo (1 + em1) (s_lo^2 below 2^-120)
    em1 = fastTwoSum(em1.hi, add(em1.lo, fma(S.lo, em1.hi, S.lo)));
    const DD one = fastTwoSum(1.0, em1.hi);
    return ddMul(T2, DD{one.hi, add(one.lo, em1.lo)});
}

// RN(R) when no rounding boundary lies within rel * |R| of R
DXG_CR_HD bool roundsUnambiguously(DD R, double rel, double& out)
{
    const double e = mul(rel, fabs(R.hi));
    const double u1 = add(R.hi, add(R.lo, e));
    const double u2 = add(R.hi, sub(R.lo, e));
    out = u1;
    return u1 == u2;
}

// x > 0 finite, y finite and nonzero (one out-of-line body per translation unit keeps the
// many inlined material-law instantiations small)
DXG_CR_CALL double powPositive(double x, double y)
{
    for (int phase = 0; phase < 2; ++phase) {
        const bool acc = phase == 1;
        const DD L = logDD(x, acc);
        const double yl = mul(y, L.hi);
        if (yl > 709.8) return INFINITY;
        if (yl < -745.2) return 0.0;
        const DD p = twoProd(y, L.hi);
        const DD Y = fastTwoSum(p.hi, fma(y, L.lo, p.lo));
        int k;
        const DD R = expDD(Y, k, acc);
        if (k < -1021) return scale2(add(R.hi, R.lo), k);   // subnormal range
        const double ay = fabs(y);
        const double rel = acc ? fma(fabs(Y.hi), 0x1p-102, fma(ay, 0x1p-101, 0x1p-98))
                               : fma(ay, 0x1p-74, 0x1p-69);
        double out;
        if (roundsUnambiguously(R, rel, out)) return scale2(out, k);
        if (acc) {
            // indistinguishable from a midpoint: round to even
            const double nb = fromBits(bitsOf(R.hi) + ((R.lo > 0) == (R.hi > 0) ? 1 : -1));
            return scale2((bitsOf(R.hi) & 1) ? nb : R.hi, k);
        }
    }
    return 0.0;   // not reached
}

}  // namespace crpow

// Correctly rounded pow (see above).
DXG_CR_HD double crPow(double x, double y)
{
    using namespace crpow;
    if (y == 0.0 || x == 1.0) return 1.0;
    if (x != x || y != y) return add(x, y);   // NaN
    const bool yInt = floor(y) == y;
    const bool yOdd = yInt && fabs(y) < 0x1p53 && fmod(y, 2.0) != 0.0;
    if (fabs(y) == INFINITY) {
        const double ax = fabs(x);
        if (ax == 1.0) return 1.0;
        return ((ax < 1.0) == (y < 0.0)) ? INFINITY : 0.0;
    }
    if (x == 0.0) {
        if (y < 0.0) return yOdd ? copysign(INFINITY, x) : INFINITY;
        return yOdd ? x : 0.0;
    }
    if (fabs(x) == INFINITY) {
        if (x > 0.0) return y > 0.0 ? INFINITY : 0.0;
        if (y > 0.0) return yOdd ? -INFINITY : INFINITY;
        return yOdd ? -0.0 : 0.0;
    }
    double sign = 1.0;
    if (x < 0.0) {
        if (!yInt) return NAN;
        if (yOdd) sign = -1.0;
        x = -x;
        if (x == 1.0) return sign;
    }
    // exact shortcuts: each is a single correctly rounded IEEE operation
    if (y == 1.0) return sign * x;
    if (y == 2.0) return mul(x, x);
    if (y == -1.0) return sign / x;
    if (y == 0.5) return sqrt(x);
    return sign * powPositive(x, y);
}

}  // namespace dxg
