// materiallaw.cuh -- regularised two-phase material laws, one source for host and device.
//
// TwoPMaterialLaw<BaseLaw, Regularization, TwoPEffToAbsDefaultPolicy>
// (dumux/material/fluidmatrixinteractions/2p/materiallaw.hh:103-223): the absolute
// saturation is mapped to the effective one, swe = (sw - Swr)/(1 - Swr - Snr)
// (efftoabsdefaultpolicy.hh:106-151); the regularisation answers outside its thresholds,
// the base law inside.  Derivatives w.r.t. sw are those w.r.t. swe times dswe/dsw.
//   kind 0: BrooksCoreyDefault  (brookscorey.hh:99-306 base law, 315-503 regularisation)
//   kind 1: VanGenuchtenDefault (vangenuchten.hh:30-300 base law, 304-620 regularisation
//           with two-point cubic splines, common/spline.hh and common/splinecommon_.hh)
// The device compiles these without FMA contraction (assemble.cu, --fmad=false) and the
// host with -ffp-contract=off, so both evaluate the reference's operation sequence.  The
// reference's std::pow is replaced by the correctly rounded crPow (crpow.cuh) on host and
// device alike.
#pragma once

#include <cmath>

#include "common.cuh"
#include "crpow.cuh"

namespace dxg {

__host__ __device__ inline double clamp01(double x) { return fmin(fmax(x, 0.0), 1.0); }

// ---------------------------------------------------------------- two-point spline
// Spline<Scalar, 2>::eval_ / evalDerivative_ on its only segment (splinecommon_.hh:478-523)
__host__ __device__ inline double splineEval(const Spline2& s, double x)
{
    const double h_i1 = s.x1 - s.x0;
    const double x_i = x - s.x0;
    const double x_i1 = s.x1 - x;
    const double A_i = (s.y1 - s.y0) / h_i1 - h_i1 / 6 * (s.M1 - s.M0);
    const double B_i = s.y0 - s.M0 * (h_i1 * h_i1) / 6;
    return s.M0 * x_i1 * x_i1 * x_i1 / (6 * h_i1) + s.M1 * x_i * x_i * x_i / (6 * h_i1) + A_i * x_i + B_i;
}
__host__ __device__ inline double splineDerivative(const Spline2& s, double x)
{
    const double h_i1 = s.x1 - s.x0;
    const double x_i = x - s.x0;
    const double x_i1 = s.x1 - x;
    const double A_i = (s.y1 - s.y0) / h_i1 - h_i1 / 6 * (s.M1 - s.M0);
    return -s.M0 * x_i1 * x_i1 / (2 * h_i1) + s.M1 * x_i * x_i / (2 * h_i1) + A_i;
}

// ---------------------------------------------------------------- Van Genuchten base law
__host__ __device__ inline double vgPcBase(const MaterialLaw& m, double swe)
{
    swe = clamp01(swe);
    return crPow(crPow(swe, m.vgNegInvM) - 1, m.vgInvN) / m.vgAlpha;
}
__host__ __device__ inline double vgDpcDsweBase(const MaterialLaw& m, double swe)
{
    swe = clamp01(swe);
    const double powSwe = crPow(swe, -1 / m.vgM);
    return -1.0 / m.vgAlpha * crPow(powSwe - 1, 1.0 / m.vgN - 1) / m.vgN * powSwe / swe / m.vgM;
}
__host__ __device__ inline double vgKrwBase(const MaterialLaw& m, double swe)
{
    swe = clamp01(swe);
    const double r = 1.0 - crPow(1.0 - crPow(swe, m.vgInvM), m.vgM);
    return crPow(swe, m.vgL) * r * r;
}
__host__ __device__ inline double vgDkrwDsweBase(const MaterialLaw& m, double swe)
{
    swe = clamp01(swe);
    const double x = 1.0 - crPow(swe, 1.0 / m.vgM);
    const double xToM = crPow(x, m.vgM);
    return (1.0 - xToM) * crPow(swe, m.vgL - 1) * ((1.0 - xToM) * m.vgL + 2 * xToM * (1.0 - x) / x);
}
__host__ __device__ inline double vgKrnBase(const MaterialLaw& m, double swe)
{
    swe = clamp01(swe);
    return crPow(1 - swe, m.vgL) * crPow(1 - crPow(swe, m.vgInvM), 2 * m.vgM);
}
__host__ __device__ inline double vgDkrnDsweBase(const MaterialLaw& m, double swe)
{
    swe = clamp01(swe);
    const double sne = 1.0 - swe;
    const double x = 1.0 - crPow(swe, 1.0 / m.vgM);
    return -crPow(sne, m.vgL - 1.0) * crPow(x, 2 * m.vgM - 1.0) * (m.vgL * x + 2.0 * sne / swe * (1.0 - x));
}

// ---------------------------------------------------------------- regularised laws
__host__ __device__ inline double lawSwe(const MaterialLaw& m, double sw) { return (sw - m.swr) / m.denom; }

__host__ __device__ inline double lawPc(const MaterialLaw& m, double sw)
{
    const double swe = lawSwe(m, sw);
    if (m.kind == 0) {
        if (swe <= m.pcLowSwe) return m.pcLowSwePcValue + m.pcDerivativeLowSw * (swe - m.pcLowSwe);
        else if (swe >= 1.0) return m.pcDerivativeHighSwEnd * (swe - 1.0) + m.entryPressure;
        return m.pe * crPow(clamp01(swe), m.expPc);
    }
    if (swe <= m.pcLowSwe) return m.pcLowSwePcValue + m.pcDerivativeLowSw * (swe - m.pcLowSwe);
    else if (swe >= 1.0) return m.pcDerivativeHighSwEnd * (swe - 1.0);
    else if (swe > m.pcHighSwe) return splineEval(m.pcSpline, swe);
    return vgPcBase(m, swe);
}
__host__ __device__ inline double lawKrw(const MaterialLaw& m, double sw)
{
    const double swe = lawSwe(m, sw);
    if (swe <= 0.0) return 0.0;
    else if (swe >= 1.0) return 1.0;
    if (m.kind == 0) return crPow(clamp01(swe), m.expKrw);
    if (swe >= m.krwHighSwe) return splineEval(m.krwSpline, swe);
    return vgKrwBase(m, swe);
}
__host__ __device__ inline double lawKrn(const MaterialLaw& m, double sw)
{
    const double swe = lawSwe(m, sw);
    if (swe <= 0.0) return 1.0;
    else if (swe >= 1.0) return 0.0;
    if (m.kind == 0) {
        const double s = clamp01(swe);
        const double sne = 1.0 - s;
        return sne * sne * (1.0 - crPow(s, m.expKrn));
    }
    if (swe <= m.krnLowSwe) return splineEval(m.krnSpline, swe);
    return vgKrnBase(m, swe);
}
__host__ __device__ inline double lawDpcDsw(const MaterialLaw& m, double sw)
{
    const double swe = lawSwe(m, sw);
    if (swe <= m.pcLowSwe) return m.pcDerivativeLowSw * m.dsweDsw;
    else if (swe >= 1.0) return m.pcDerivativeHighSwEnd * m.dsweDsw;
    if (m.kind == 0) return m.dpcCoef * crPow(clamp01(swe), m.dpcExp) * m.dsweDsw;
    if (swe > m.pcHighSwe) return splineDerivative(m.pcSpline, swe) * m.dsweDsw;
    return vgDpcDsweBase(m, swe) * m.dsweDsw;
}
__host__ __device__ inline double lawDkrwDsw(const MaterialLaw& m, double sw)
{
    const double swe = lawSwe(m, sw);
    if (swe <= 0.0 || swe >= 1.0) return 0.0 * m.dsweDsw;
    if (m.kind == 0) return m.dkrwCoef * crPow(clamp01(swe), m.dkrwExp) * m.dsweDsw;
    if (swe >= m.krwHighSwe) return splineDerivative(m.krwSpline, swe) * m.dsweDsw;
    return vgDkrwDsweBase(m, swe) * m.dsweDsw;
}
__host__ __device__ inline double lawDkrnDsw(const MaterialLaw& m, double sw)
{
    const double swe = lawSwe(m, sw);
    if (swe <= 0.0 || swe >= 1.0) return 0.0 * m.dsweDsw;
    if (m.kind == 0) {
        const double s = clamp01(swe);
        const double swePow = crPow(s, m.dkrnExp);
        return 2.0 * (s - 1.0) * (1.0 + (0.5 + m.lambdaInv) * swePow - (1.5 + m.lambdaInv) * swePow * s) *
               m.dsweDsw;
    }
    if (swe <= m.krnLowSwe) return splineDerivative(m.krnSpline, swe) * m.dsweDsw;
    return vgDkrnDsweBase(m, swe) * m.dsweDsw;
}

// ---------------------------------------------------------------- set-up (host)
// Spline<Scalar, 2>::set: moments of the clamped two-point spline from the 2x2 system
// [[2, 1], [1, 2]] M = d (splinecommon_.hh:419-470), solved by the closed form for 2x2
// dense matrices (inverse determinant times the adjugate).
inline Spline2 makeSpline2(double x0, double x1, double y0, double y1, double m0, double m1)
{
    Spline2 s{x0, x1, y0, y1, 0.0, 0.0};
    const double h = x1 - x0;
    const double d0 = 6 / h * ((y1 - y0) / h - m0);
    const double d1 = 6 / h * (m1 - (y1 - y0) / h);
    const double a00 = 2, a01 = 1, a10 = 1, a11 = 2;
    double detinv = a00 * a11 - a01 * a10;
    detinv = 1.0 / detinv;
    s.M0 = detinv * (a11 * d0 - a01 * d1);
    s.M1 = detinv * (a00 * d1 - a10 * d0);
    return s;
}

// Parameter set of one material: 5 doubles (Brooks-Corey: pcEntry, lambda, Swr, Snr,
// pcLowSwe) or 9 doubles (Van Genuchten: alpha, n, l, Swr, Snr, pcLowSwe, pcHighSwe,
// krnLowSwe, krwHighSwe); derived constants as the regularisations' init functions
// compute them (brookscorey.hh:477-486, vangenuchten.hh:553-598).
inline MaterialLaw makeMaterialLaw(int kind, const double* prm)
{
    MaterialLaw m{};
    m.kind = kind;
    auto sweToSw = [&](double swe) { return swe * (1.0 - m.swr - m.snr) + m.swr; };
    if (kind == 0) {
        m.pe = prm[0];
        m.lambda = prm[1];
        m.swr = prm[2];
        m.snr = prm[3];
        m.pcLowSwe = prm[4];
        m.denom = 1.0 - m.swr - m.snr;
        m.expPc = -1.0 / m.lambda;
        m.expKrw = 2.0 / m.lambda + 3.0;
        m.expKrn = 2.0 / m.lambda + 1.0;
        auto swToSwe = [&](double sw) { return (sw - m.swr) / (1.0 - m.swr - m.snr); };
        auto dpc_dswe = [&](double swe) {
            swe = clamp01(swe);
            return -m.pe / m.lambda * crPow(swe, -1.0 / m.lambda - 1.0);
        };
        const double dswe_dsw = 1.0 / (1.0 - m.swr - m.snr);
        const double dsw_dswe = 1.0 - m.swr - m.snr;
        const double lowSw = sweToSw(m.pcLowSwe);
        const double highSw = sweToSw(1.0);
        m.entryPressure = m.pe;
        m.pcDerivativeLowSw = dpc_dswe(swToSwe(lowSw)) * dswe_dsw * dsw_dswe;
        m.pcDerivativeHighSwEnd = dpc_dswe(swToSwe(highSw)) * dswe_dsw * dsw_dswe;
        m.pcLowSwePcValue = m.pe * crPow(clamp01(swToSwe(lowSw)), -1.0 / m.lambda);
        m.dsweDsw = 1.0 / (1.0 - m.swr - m.snr);
        m.dpcCoef = -m.pe / m.lambda;
        m.dpcExp = -1.0 / m.lambda - 1.0;
        m.dkrwCoef = 2.0 / m.lambda + 3.0;
        m.dkrwExp = 2.0 / m.lambda + 2.0;
        m.lambdaInv = 1.0 / m.lambda;
        m.dkrnExp = 2 * m.lambdaInv;
        return m;
    }
    // VanGenuchten::Params (alpha, n, l): m = 1 - 1/n
    m.vgAlpha = prm[0];
    m.vgN = prm[1];
    m.vgM = 1.0 - 1.0 / m.vgN;
    m.vgL = prm[2];
    m.swr = prm[3];
    m.snr = prm[4];
    m.pcLowSwe = prm[5];
    m.pcHighSwe = prm[6];
    m.krnLowSwe = prm[7];
    m.krwHighSwe = prm[8];
    m.denom = 1.0 - m.swr - m.snr;
    m.vgNegInvM = -1.0 / m.vgM;
    m.vgInvN = 1.0 / m.vgN;
    m.vgInvM = 1.0 / m.vgM;
    m.dsweDsw = 1.0 / (1.0 - m.swr - m.snr);
    auto swToSwe = [&](double sw) { return (sw - m.swr) / (1.0 - m.swr - m.snr); };
    const double dswe_dsw = 1.0 / (1.0 - m.swr - m.snr);
    const double dsw_dswe = 1.0 - m.swr - m.snr;
    // unregularised pc, krw, krn and their sw-derivatives (TwoPMaterialLaw::<fn><false>)
    auto pcNoReg = [&](double sw) { return vgPcBase(m, swToSwe(sw)); };
    auto dpcNoReg = [&](double sw) { return vgDpcDsweBase(m, swToSwe(sw)) * dswe_dsw; };
    // initPcParameters_(lowSwe, highSwe)
    {
        const double lowSw = sweToSw(m.pcLowSwe);
        const double highSw = sweToSw(m.pcHighSwe);
        m.pcDerivativeLowSw = dpcNoReg(lowSw) * dsw_dswe;
        const double pcDerivativeHighSweThreshold = dpcNoReg(highSw) * dsw_dswe;
        m.pcDerivativeHighSwEnd = 2.0 * (0.0 - pcNoReg(highSw)) / (1.0 - m.pcHighSwe);
        m.pcLowSwePcValue = pcNoReg(lowSw);
        const double pcHighSwePcValue = pcNoReg(highSw);
        if (m.pcHighSwe < 1.0)
            m.pcSpline = makeSpline2(m.pcHighSwe, 1.0, pcHighSwePcValue, 0, pcDerivativeHighSweThreshold,
                                     m.pcDerivativeHighSwEnd);
    }
    // initKrParameters_(krnLowSwe, krwHighSwe)
    {
        const double lowSw = sweToSw(m.krnLowSwe);
        const double highSw = sweToSw(m.krwHighSwe);
        const double krwHighSw = vgKrwBase(m, swToSwe(highSw));
        const double dkrwHighSw = vgDkrwDsweBase(m, swToSwe(highSw)) * dswe_dsw * dsw_dswe;
        const double krnLowSw = vgKrnBase(m, swToSwe(lowSw));
        const double dkrnLowSw = vgDkrnDsweBase(m, swToSwe(lowSw)) * dswe_dsw * dsw_dswe;
        if (m.krwHighSwe < 1.0) m.krwSpline = makeSpline2(m.krwHighSwe, 1.0, krwHighSw, 1.0, dkrwHighSw, 0.0);
        if (m.krnLowSwe > 0.0) m.krnSpline = makeSpline2(0.0, m.krnLowSwe, 1.0, krnLowSw, 0.0, dkrnLowSw);
    }
    return m;
}

}  // namespace dxg
