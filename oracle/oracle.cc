// oracle.cc -- CPU oracle for the cc-TPFA hot path.  TEST INFRASTRUCTURE ONLY:
// the checker for the product's CUDA path (tests, smoke check, CPU baseline of
// bench.py).  Never linked into the product.
//
// A faithful FP64 restatement of the reference's element-wise algorithm:
//   * element loop and numeric-difference Jacobian: dumux/assembly/fvassembler.hh:461-510,
//     dumux/assembly/cclocalassembler.hh:164-348 (column-wise scatter, neighbour fluxes
//     evaluated with the neighbour as inside element);
//   * local residual: dumux/assembly/fvlocalresidual.hh:132-333,
//     dumux/assembly/cclocalresidual.hh:49-105,
//     dumux/porousmediumflow/immiscible/localresidual.hh:64-126;
//   * TPFA Darcy flux with gravity and upwinding: dumux/flux/cctpfa/darcyslaw.hh:153-259,
//     dumux/discretization/cellcentered/tpfa/computetransmissibility.hh:66-80,
//     dumux/flux/upwindscheme.hh:35-54;
//   * element volume variables incl. Dirichlet ghosts built with the inside cell's
//     spatial parameters: dumux/discretization/cellcentered/tpfa/elementvolumevariables.hh:277-342,
//     dumux/porousmediumflow/2p/volumevariables.hh:74-191, 1p/volumevariables.hh:65-179;
//   * regularised Brooks-Corey: dumux/material/fluidmatrixinteractions/2p/brookscorey.hh:99-503,
//     materiallaw.hh:103-223, efftoabsdefaultpolicy.hh:106-151;
//   * numeric differentiation: dumux/common/numericdifferentiation.hh:36-123,
//     dumux/assembly/numericepsilon.hh:37-53;
//   * Newton driver: dumux/nonlinear/newtonsolver.hh:110-128, 309-382, 428-701, 784-798,
//     917-1072, 1138-1178, 1213-1254;
//   * linear solver: dune-istl >= 2.10 (not vendored in the reference) SeqILU(n=0, w=1) and
//     BiCGSTABSolver as bound by dumux/linear/istlsolvers.hh:535-568, 635-642 with the
//     defaults of dumux/linear/linearsolverparameters.hh:56-73.  ILU(0) follows the
//     published block ILU(0) algorithm (Saad 2003, Alg. 10.4, row-wise "IKJ" variant,
//     pivots stored inverted); BiCGSTAB follows van der Vorst (1992) with dune-istl's
//     half-step convergence tests (def < reduction*def0 or def < 1e-30) and breakdown
//     threshold 1e-80.
// Compiled with -ffp-contract=off so x86 and Arm hosts give identical bits.
#include "oracle.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../dumux_gb300/csrc/crpow.cuh"

namespace orc {

// pow of the material laws.  Mode 0 (default): the C library's pow, which the reference
// calls (std::pow); for binary64 it is not correctly rounded in ~0.1% of arguments, and
// its rounding may differ between C libraries.  Mode 1: the correctly rounded pow
// (crpow.cuh, checked against 200-bit arithmetic in tests/test_crpow.py), which takes
// the libm out of a comparison with the device, whose pow is correctly rounded.
static int g_pow_mode = 0;
static inline double lawPow(double x, double y) { return g_pow_mode == 1 ? dxg::crPow(x, y) : std::pow(x, y); }

struct NumericalProblem : std::runtime_error { using std::runtime_error::runtime_error; };
struct SolverAbort : std::runtime_error { using std::runtime_error::runtime_error; };

static int g_threads = 0;
}  // namespace orc
extern "C" int orc_get_threads(void);
namespace orc {

// ---------------------------------------------------------------- Brooks-Corey
struct BrooksCoreyDefault {
    double pe, lambda, swr, snr, pcLowSwe;
    double pcLowSwePcValue = 0, pcDerivativeLowSw = 0, pcDerivativeHighSwEnd = 0, entryPressure = 0;

    explicit BrooksCoreyDefault(const double* prm)
        : pe(prm[0]), lambda(prm[1]), swr(prm[2]), snr(prm[3]), pcLowSwe(prm[4])
    {
        // BrooksCoreyRegularization::init / initPcParameters_ (brookscorey.hh:347-354, 477-486)
        entryPressure = pe;
        const double lowSw = sweToSw(pcLowSwe);
        const double highSw = sweToSw(1.0);
        const double dsw_dswe = 1.0 - swr - snr;
        pcDerivativeLowSw = dpc_dsw_noreg(lowSw) * dsw_dswe;
        pcDerivativeHighSwEnd = dpc_dsw_noreg(highSw) * dsw_dswe;
        pcLowSwePcValue = pc_noreg(lowSw);
    }
    double swToSwe(double sw) const { return (sw - swr) / (1.0 - swr - snr); }
    double sweToSw(double swe) const { return swe * (1.0 - swr - snr) + swr; }
    double dswe_dsw() const { return 1.0 / (1.0 - swr - snr); }
    static double clamp01(double x) { return std::clamp(x, 0.0, 1.0); }
    double base_pc(double swe) const { swe = clamp01(swe); return pe * lawPow(swe, -1.0 / lambda); }
    double base_dpc_dswe(double swe) const
    {
        swe = clamp01(swe);
        return -pe / lambda * lawPow(swe, -1.0 / lambda - 1.0);
    }
    double pc_noreg(double sw) const { return base_pc(swToSwe(sw)); }
    double dpc_dsw_noreg(double sw) const { return base_dpc_dswe(swToSwe(sw)) * dswe_dsw(); }

    double pc(double sw) const
    {
        const double swe = swToSwe(sw);
        if (swe <= pcLowSwe) return pcLowSwePcValue + pcDerivativeLowSw * (swe - pcLowSwe);
        else if (swe >= 1.0) return pcDerivativeHighSwEnd * (swe - 1.0) + entryPressure;
        return base_pc(swe);
    }
    double krw(double sw) const
    {
        const double swe = swToSwe(sw);
        if (swe <= 0.0) return 0.0;
        else if (swe >= 1.0) return 1.0;
        return lawPow(clamp01(swe), 2.0 / lambda + 3.0);
    }
    double krn(double sw) const
    {
        const double swe = swToSwe(sw);
        if (swe <= 0.0) return 1.0;
        else if (swe >= 1.0) return 0.0;
        const double s = clamp01(swe);
        const double exponent = 2.0 / lambda + 1.0;
        const double sne = 1.0 - s;
        return sne * sne * (1.0 - lawPow(s, exponent));
    }
    // TwoPMaterialLaw::dpc_dsw / dkrw_dsw / dkrn_dsw (materiallaw.hh:121-239): the
    // regularised slope (BrooksCoreyRegularization::dpc_dswe, dkrw_dswe, dkrn_dswe,
    // brookscorey.hh:385-475) or the Brooks-Corey derivative (brookscorey.hh:166-305),
    // times dswe/dsw (efftoabsdefaultpolicy.hh:135-138)
    double dpc_dsw(double sw) const
    {
        const double swe = swToSwe(sw);
        if (swe <= pcLowSwe) return pcDerivativeLowSw * dswe_dsw();
        else if (swe >= 1.0) return pcDerivativeHighSwEnd * dswe_dsw();
        return base_dpc_dswe(swe) * dswe_dsw();
    }
    double dkrw_dsw(double sw) const
    {
        const double swe = swToSwe(sw);
        if (swe <= 0.0 || swe >= 1.0) return 0.0 * dswe_dsw();
        const double s = clamp01(swe);
        return (2.0 / lambda + 3.0) * lawPow(s, 2.0 / lambda + 2.0) * dswe_dsw();
    }
    double dkrn_dsw(double sw) const
    {
        const double swe = swToSwe(sw);
        if (swe <= 0.0 || swe >= 1.0) return 0.0 * dswe_dsw();
        const double s = clamp01(swe);
        const double lambdaInv = 1.0 / lambda;
        const double swePow = lawPow(s, 2 * lambdaInv);
        return 2.0 * (s - 1.0) * (1.0 + (0.5 + lambdaInv) * swePow - (1.5 + lambdaInv) * swePow * s) * dswe_dsw();
    }
};

// ---------------------------------------------------------------- grid / geometry
// VanGenuchtenDefault = TwoPMaterialLaw<VanGenuchten, VanGenuchtenRegularization,
// TwoPEffToAbsDefaultPolicy> (material/fluidmatrixinteractions/2p/vangenuchten.hh:30-620,
// materiallaw.hh:103-239): base law on the clamped effective saturation; regularisation by
// linear extensions and clamped two-point cubic splines (common/spline.hh:310-345,
// common/splinecommon_.hh:419-523) outside [pcLowSwe, pcHighSwe] for pc, above krwHighSwe
// for krw and below krnLowSwe for krn.
struct Spline2Point {
    double x0 = 0, x1 = 1, y0 = 0, y1 = 0, M0 = 0, M1 = 0;
    Spline2Point() = default;
    Spline2Point(double a0, double a1, double b0, double b1, double m0, double m1)
        : x0(a0), x1(a1), y0(b0), y1(b1)
    {
        // moments of the clamped spline: [[2,1],[1,2]] M = d, closed-form 2x2 solve
        const double h = x1 - x0;
        const double d0 = 6 / h * ((y1 - y0) / h - m0);
        const double d1 = 6 / h * (m1 - (y1 - y0) / h);
        double detinv = 2.0 * 2.0 - 1.0 * 1.0;
        detinv = 1.0 / detinv;
        M0 = detinv * (2.0 * d0 - 1.0 * d1);
        M1 = detinv * (2.0 * d1 - 1.0 * d0);
    }
    double eval(double x) const
    {
        const double h = x1 - x0, xi = x - x0, xi1 = x1 - x;
        const double A = (y1 - y0) / h - h / 6 * (M1 - M0);
        const double B = y0 - M0 * (h * h) / 6;
        return M0 * xi1 * xi1 * xi1 / (6 * h) + M1 * xi * xi * xi / (6 * h) + A * xi + B;
    }
    double derivative(double x) const
    {
        const double h = x1 - x0, xi = x - x0, xi1 = x1 - x;
        const double A = (y1 - y0) / h - h / 6 * (M1 - M0);
        return -M0 * xi1 * xi1 / (2 * h) + M1 * xi * xi / (2 * h) + A;
    }
};

struct VanGenuchtenDefault {
    double alpha, n, m, l, swr, snr;
    double pcLowSwe, pcHighSwe, krnLowSwe, krwHighSwe;
    double pcLowSwePcValue = 0, pcDerivativeLowSw = 0, pcDerivativeHighSweEnd = 0;
    Spline2Point pcSpline, krwSpline, krnSpline;

    explicit VanGenuchtenDefault(const double* prm)
        : alpha(prm[0]), n(prm[1]), m(1.0 - 1.0 / prm[1]), l(prm[2]), swr(prm[3]), snr(prm[4]),
          pcLowSwe(prm[5]), pcHighSwe(prm[6]), krnLowSwe(prm[7]), krwHighSwe(prm[8])
    {
        const double dsw_dswe = 1.0 - swr - snr;
        // initPcParameters_ (vangenuchten.hh:553-574)
        const double lowSw = sweToSw(pcLowSwe), highSw = sweToSw(pcHighSwe);
        pcDerivativeLowSw = base_dpc_dswe(swToSwe(lowSw)) * dswe_dsw() * dsw_dswe;
        const double pcDerivativeHighSweThreshold = base_dpc_dswe(swToSwe(highSw)) * dswe_dsw() * dsw_dswe;
        pcDerivativeHighSweEnd = 2.0 * (0.0 - base_pc(swToSwe(highSw))) / (1.0 - pcHighSwe);
        pcLowSwePcValue = base_pc(swToSwe(lowSw));
        const double pcHighSwePcValue = base_pc(swToSwe(highSw));
        if (pcHighSwe < 1.0)
            pcSpline = Spline2Point(pcHighSwe, 1.0, pcHighSwePcValue, 0, pcDerivativeHighSweThreshold,
                                    pcDerivativeHighSweEnd);
        // initKrParameters_ (vangenuchten.hh:576-598)
        const double krLowSw = sweToSw(krnLowSwe), krHighSw = sweToSw(krwHighSwe);
        const double krwHighSw = base_krw(swToSwe(krHighSw));
        const double dkrwHighSw = base_dkrw_dswe(swToSwe(krHighSw)) * dswe_dsw() * dsw_dswe;
        const double krnLowSw = base_krn(swToSwe(krLowSw));
        const double dkrnLowSw = base_dkrn_dswe(swToSwe(krLowSw)) * dswe_dsw() * dsw_dswe;
        if (krwHighSwe < 1.0) krwSpline = Spline2Point(krwHighSwe, 1.0, krwHighSw, 1.0, dkrwHighSw, 0.0);
        if (krnLowSwe > 0.0) krnSpline = Spline2Point(0.0, krnLowSwe, 1.0, krnLowSw, 0.0, dkrnLowSw);
    }
    double swToSwe(double sw) const { return (sw - swr) / (1.0 - swr - snr); }
    double sweToSw(double swe) const { return swe * (1.0 - swr - snr) + swr; }
    double dswe_dsw() const { return 1.0 / (1.0 - swr - snr); }
    static double c01(double x) { return std::clamp(x, 0.0, 1.0); }
    double base_pc(double swe) const { swe = c01(swe); return lawPow(lawPow(swe, -1.0 / m) - 1, 1.0 / n) / alpha; }
    double base_dpc_dswe(double swe) const
    {
        swe = c01(swe);
        const double powSwe = lawPow(swe, -1 / m);
        return -1.0 / alpha * lawPow(powSwe - 1, 1.0 / n - 1) / n * powSwe / swe / m;
    }
    double base_krw(double swe) const
    {
        swe = c01(swe);
        const double r = 1.0 - lawPow(1.0 - lawPow(swe, 1.0 / m), m);
        return lawPow(swe, l) * r * r;
    }
    double base_dkrw_dswe(double swe) const
    {
        swe = c01(swe);
        const double x = 1.0 - lawPow(swe, 1.0 / m);
        const double xToM = lawPow(x, m);
        return (1.0 - xToM) * lawPow(swe, l - 1) * ((1.0 - xToM) * l + 2 * xToM * (1.0 - x) / x);
    }
    double base_krn(double swe) const
    {
        swe = c01(swe);
        return lawPow(1 - swe, l) * lawPow(1 - lawPow(swe, 1.0 / m), 2 * m);
    }
    double base_dkrn_dswe(double swe) const
    {
        swe = c01(swe);
        const double sne = 1.0 - swe;
        const double x = 1.0 - lawPow(swe, 1.0 / m);
        return -lawPow(sne, l - 1.0) * lawPow(x, 2 * m - 1.0) * (l * x + 2.0 * sne / swe * (1.0 - x));
    }
    double pc(double sw) const
    {
        const double swe = swToSwe(sw);
        if (swe <= pcLowSwe) return pcLowSwePcValue + pcDerivativeLowSw * (swe - pcLowSwe);
        else if (swe >= 1.0) return pcDerivativeHighSweEnd * (swe - 1.0);
        else if (swe > pcHighSwe) return pcSpline.eval(swe);
        return base_pc(swe);
    }
    double krw(double sw) const
    {
        const double swe = swToSwe(sw);
        if (swe <= 0.0) return 0.0;
        else if (swe >= 1.0) return 1.0;
        else if (swe >= krwHighSwe) return krwSpline.eval(swe);
        return base_krw(swe);
    }
    double krn(double sw) const
    {
        const double swe = swToSwe(sw);
        if (swe <= 0.0) return 1.0;
        else if (swe >= 1.0) return 0.0;
        else if (swe <= krnLowSwe) return krnSpline.eval(swe);
        return base_krn(swe);
    }
    double dpc_dsw(double sw) const
    {
        const double swe = swToSwe(sw);
        if (swe <= pcLowSwe) return pcDerivativeLowSw * dswe_dsw();
        else if (swe >= 1.0) return pcDerivativeHighSweEnd * dswe_dsw();
        else if (swe > pcHighSwe) return pcSpline.derivative(swe) * dswe_dsw();
        return base_dpc_dswe(swe) * dswe_dsw();
    }
    double dkrw_dsw(double sw) const
    {
        const double swe = swToSwe(sw);
        if (swe <= 0.0 || swe >= 1.0) return 0.0 * dswe_dsw();
        else if (swe >= krwHighSwe) return krwSpline.derivative(swe) * dswe_dsw();
        return base_dkrw_dswe(swe) * dswe_dsw();
    }
    double dkrn_dsw(double sw) const
    {
        const double swe = swToSwe(sw);
        if (swe <= 0.0 || swe >= 1.0) return 0.0 * dswe_dsw();
        else if (swe <= krnLowSwe) return krnSpline.derivative(swe) * dswe_dsw();
        return base_dkrn_dswe(swe) * dswe_dsw();
    }
};

// The 2p material law of one parameter set: Brooks-Corey or Van Genuchten.
struct TwoPLaw {
    int kind;
    BrooksCoreyDefault bc;
    VanGenuchtenDefault vg;
    static const double* zeros() { static const double z[9] = {1, 2, 0, 0, 0, 0.01, 0.99, 0.1, 0.9}; return z; }
    TwoPLaw(int k, const double* prm)
        : kind(k), bc(k == 0 ? prm : zeros()), vg(k == 1 ? prm : zeros()) {}
    double pc(double sw) const { return kind == 0 ? bc.pc(sw) : vg.pc(sw); }
    double krw(double sw) const { return kind == 0 ? bc.krw(sw) : vg.krw(sw); }
    double krn(double sw) const { return kind == 0 ? bc.krn(sw) : vg.krn(sw); }
    double dpc_dsw(double sw) const { return kind == 0 ? bc.dpc_dsw(sw) : vg.dpc_dsw(sw); }
    double dkrw_dsw(double sw) const { return kind == 0 ? bc.dkrw_dsw(sw) : vg.dkrw_dsw(sw); }
    double dkrn_dsw(double sw) const { return kind == 0 ? bc.dkrn_dsw(sw) : vg.dkrn_dsw(sw); }
};

struct Face {
    int axis, side;            // local face f = 2*axis + side
    bool boundary;
    int64_t outside;           // neighbour cell (interior faces)
    int64_t bidx;              // boundary face index (boundary faces)
    double ip[3], n[3], area;
};

struct Problem {
    const dxg_problem_desc& d;
    int dim, b;
    int64_t n[3], N;
    int64_t side_offset[7];
    std::vector<TwoPLaw> laws;
    double g[3] = {0, 0, 0};

    explicit Problem(const dxg_problem_desc& desc) : d(desc)
    {
        dim = d.dim;
        b = d.num_eq;
        if (dim < 2 || dim > 3 || (b != 1 && b != 2)) throw std::invalid_argument("unsupported dim/num_eq");
        for (int a = 0; a < 3; ++a) n[a] = (a < dim) ? d.cells[a] : 1;
        N = n[0] * n[1] * n[2];
        side_offset[0] = 0;
        for (int f = 0; f < 2 * dim; ++f) {
            const int a = f / 2;
            int64_t cnt = 1;
            for (int c = 0; c < dim; ++c) if (c != a) cnt *= n[c];
            side_offset[f + 1] = side_offset[f] + cnt;
        }
        if (b == 2) {
            const int width = d.material_law == 1 ? 9 : 5;
            for (int m = 0; m < d.num_materials; ++m) laws.emplace_back(d.material_law, d.material_params + width * m);
        }
        if (d.enable_gravity) for (int a = 0; a < dim; ++a) g[a] = d.gravity[a];
    }
    void ijk(int64_t c, int64_t* id) const { id[0] = c % n[0]; id[1] = (c / n[0]) % n[1]; id[2] = c / (n[0] * n[1]); }
    double lo(int a, int64_t i) const { return d.coords[a][i]; }
    double hi(int a, int64_t i) const { return d.coords[a][i + 1]; }
    void center(int64_t c, double* x) const
    {
        int64_t id[3]; ijk(c, id);
        for (int a = 0; a < 3; ++a) x[a] = 0.0;
        for (int a = 0; a < dim; ++a) x[a] = 0.5 * (lo(a, id[a]) + hi(a, id[a]));
    }
    double volume(int64_t c) const
    {
        int64_t id[3]; ijk(c, id);
        double v = 1.0;
        for (int a = 0; a < dim; ++a) v *= hi(a, id[a]) - lo(a, id[a]);
        return v;
    }
    Face face(int64_t c, int f) const
    {
        Face fc{};
        int64_t id[3]; ijk(c, id);
        fc.axis = f / 2; fc.side = f % 2;
        const int a = fc.axis;
        center(c, fc.ip);
        fc.ip[a] = fc.side == 0 ? lo(a, id[a]) : hi(a, id[a]);
        for (int k = 0; k < 3; ++k) fc.n[k] = 0.0;
        fc.n[a] = fc.side == 0 ? -1.0 : 1.0;
        fc.area = 1.0;
        for (int k = 0; k < dim; ++k) if (k != a) fc.area *= hi(k, id[k]) - lo(k, id[k]);
        const bool bnd = fc.side == 0 ? id[a] == 0 : id[a] == n[a] - 1;
        fc.boundary = bnd;
        if (!bnd) {
            int64_t stride = 1;
            for (int k = 0; k < a; ++k) stride *= n[k];
            fc.outside = c + (fc.side == 0 ? -stride : stride);
            fc.bidx = -1;
        } else {
            fc.outside = -1;
            int64_t pos = 0, mul = 1;
            for (int k = 0; k < dim; ++k) if (k != a) { pos += id[k] * mul; mul *= n[k]; }
            fc.bidx = side_offset[f] + pos;
        }
        return fc;
    }
    double perm(int64_t c) const { return d.permeability[c]; }
    double poro(int64_t c) const { return d.porosity[c]; }
    double extr(int64_t c) const { return d.extrusion ? d.extrusion[c] : 1.0; }
    const TwoPLaw& law(int64_t c) const { return laws[d.material ? d.material[c] : 0]; }
};

struct VolVars {
    double p[2], rho[2], mob[2], S[2];
    double phi, extr, K;
};

// OnePVolumeVariables::update / TwoPVolumeVariables::update + completeFluidState (p0s1,
// water wetting).  Spatial parameters are those of cell c.
static VolVars volVars(const Problem& P, const double* pv, int64_t c)
{
    VolVars v{};
    v.phi = P.poro(c);
    v.extr = P.extr(c);
    v.K = P.perm(c);
    if (P.b == 1) {
        v.p[0] = pv[0];
        v.rho[0] = P.d.density[0];
        v.mob[0] = 1.0 / P.d.viscosity[0];
        v.S[0] = 1.0;
    } else {
        const auto& law = P.law(c);
        const double Sn = pv[1];
        v.S[1] = Sn;
        v.S[0] = 1 - Sn;
        const double pc = law.pc(v.S[0]);
        v.p[0] = pv[0];
        v.p[1] = pv[0] + pc;
        v.rho[0] = P.d.density[0];
        v.rho[1] = P.d.density[1];
        v.mob[0] = law.krw(v.S[0]) / P.d.viscosity[0];
        v.mob[1] = law.krn(v.S[0]) / P.d.viscosity[1];
    }
    return v;
}

// computeTpfaTransmissibility for a scalar permeability
static double tpfaT(const Problem& P, const Face& f, int64_t scvCell, double K, double extr)
{
    double c[3]; P.center(scvCell, c);
    double dv[3];
    for (int i = 0; i < P.dim; ++i) dv[i] = f.ip[i] - c[i];
    double n2 = 0.0;
    for (int i = 0; i < P.dim; ++i) n2 += dv[i] * dv[i];
    for (int i = 0; i < P.dim; ++i) dv[i] /= n2;
    double dot = 0.0;
    for (int i = 0; i < P.dim; ++i) dot += dv[i] * f.n[i];
    return K * extr * dot;
}

static double nDotG(const Problem& P, const Face& f)
{
    double s = 0.0;
    for (int i = 0; i < P.dim; ++i) s += f.n[i] * P.g[i];
    return s;
}

// ImmiscibleLocalResidual::computeFlux for the face f of cell `inside`
static void computeFlux(const Problem& P, int64_t inside, const Face& f,
                        const VolVars& vin, const VolVars& vout, double* F)
{
    // flux variables cache: TPFA transmissibility (darcyslaw.hh:217-259)
    const double ti = tpfaT(P, f, inside, vin.K, vin.extr);
    double tij;
    if (f.boundary)
        tij = f.area * ti;
    else {
        const double tj = -1.0 * tpfaT(P, f, f.outside, vout.K, vout.extr);
        if (ti * tj <= 0.0) tij = 0;
        else tij = f.area * (ti * tj) / (ti + tj);
    }
    const double w = P.d.upwind_weight;
    for (int ph = 0; ph < P.b; ++ph) {
        double flux;
        if (P.d.enable_gravity) {
            const double rho = f.boundary ? vout.rho[ph] : (vin.rho[ph] + vout.rho[ph]) * 0.5;
            const double alpha_inside = vin.K * nDotG(P, f) * vin.extr;
            flux = tij * (vin.p[ph] - vout.p[ph]) + rho * f.area * alpha_inside;
            if (!f.boundary) {
                const double outsideTi = -1.0 * tpfaT(P, f, f.outside, vout.K, vout.extr);
                const double alpha_outside = vout.K * nDotG(P, f) * vout.extr;
                flux -= rho * tij / outsideTi * (alpha_inside - alpha_outside);
            }
        } else {
            flux = tij * (vin.p[ph] - vout.p[ph]);
        }
        const double upIn = vin.rho[ph] * vin.mob[ph];
        const double upOut = vout.rho[ph] * vout.mob[ph];
        double mult;
        if (std::signbit(flux)) mult = w * upOut + (1.0 - w) * upIn;
        else mult = w * upIn + (1.0 - w) * upOut;
        F[ph] = flux * mult;
    }
}

// PorousMediumFluxVariables advective Darcy flux of phase ph without the upwinded
// mobility (AdvectionType::flux, darcyslaw.hh:153-213) and the face transmissibility
static double darcyFlux(const Problem& P, int64_t inside, const Face& f, const VolVars& vin, const VolVars& vout,
                        int ph, double* tijOut)
{
    const double ti = tpfaT(P, f, inside, vin.K, vin.extr);
    double tij;
    if (f.boundary)
        tij = f.area * ti;
    else {
        const double tj = -1.0 * tpfaT(P, f, f.outside, vout.K, vout.extr);
        if (ti * tj <= 0.0) tij = 0;
        else tij = f.area * (ti * tj) / (ti + tj);
    }
    *tijOut = tij;
    if (!P.d.enable_gravity) return tij * (vin.p[ph] - vout.p[ph]);
    const double rho = f.boundary ? vout.rho[ph] : (vin.rho[ph] + vout.rho[ph]) * 0.5;
    const double alpha_inside = vin.K * nDotG(P, f) * vin.extr;
    double flux = tij * (vin.p[ph] - vout.p[ph]) + rho * f.area * alpha_inside;
    if (!f.boundary) {
        const double outsideTi = -1.0 * tpfaT(P, f, f.outside, vout.K, vout.extr);
        const double alpha_outside = vout.K * nDotG(P, f) * vout.extr;
        flux -= rho * tij / outsideTi * (alpha_inside - alpha_outside);
    }
    return flux;
}

// element-local view: volume variables of the element, its neighbours and the
// Dirichlet ghosts, bound at the current solution
struct ElemView {
    int64_t I;
    VolVars vI;
    VolVars vOut[6];           // per local face: neighbour vv or Dirichlet ghost
    Face faces[6];
    VolVars vPrev;
    bool transient;
    double dt;
};

// CCLocalResidual::evalFlux (boundary handling, cclocalresidual.hh:58-101)
static void evalFlux(const Problem& P, int64_t inside, const Face& f, const VolVars& vin,
                     const VolVars& vout, double* out)
{
    double flux[2] = {0.0, 0.0};
    if (!f.boundary) {
        double F[2]; computeFlux(P, inside, f, vin, vout, F);
        for (int e = 0; e < P.b; ++e) flux[e] += F[e];
    } else {
        const int8_t t = P.d.bc_type[f.bidx];
        if (t == 1) {
            double F[2]; computeFlux(P, inside, f, vin, vout, F);
            for (int e = 0; e < P.b; ++e) flux[e] += F[e];
        } else if (t == 2) {
            const double s = f.area * vin.extr;
            for (int e = 0; e < P.b; ++e) flux[e] += P.d.bc_values[f.bidx * P.b + e] * s;
        } else throw std::invalid_argument("mixed/unknown boundary condition");
    }
    for (int e = 0; e < P.b; ++e) out[e] = flux[e];
}

// FVLocalAssemblerBase::evalLocalResidual for element I with (possibly deflected) vI
static void localResidual(const Problem& P, const ElemView& ev, const VolVars& vI, double* res)
{
    const int b = P.b;
    const int64_t I = ev.I;
    const double V = P.volume(I);
    double r[2] = {0.0, 0.0};
    // evalSource: residual -= source*V*extrusion
    {
        double src[2] = {0.0, 0.0};
        if (P.d.source) for (int e = 0; e < b; ++e) src[e] += P.d.source[I * b + e];
        const double s = V * vI.extr;
        for (int e = 0; e < b; ++e) { src[e] *= s; r[e] -= src[e]; }
    }
    // evalFlux over all faces of I
    for (int f = 0; f < 2 * P.dim; ++f) {
        double fl[2];
        evalFlux(P, I, ev.faces[f], vI, ev.vOut[f], fl);
        for (int e = 0; e < b; ++e) r[e] += fl[e];
    }
    if (ev.transient) {
        double st[2] = {0.0, 0.0};
        for (int ph = 0; ph < b; ++ph) {
            double prevS = ev.vPrev.phi * ev.vPrev.rho[ph] * ev.vPrev.S[ph];
            double curS = vI.phi * vI.rho[ph] * vI.S[ph];
            prevS *= ev.vPrev.extr;
            curS *= vI.extr;
            curS -= prevS;
            curS *= V;
            curS /= ev.dt;
            st[ph] += curS;
        }
        for (int e = 0; e < b; ++e) r[e] += st[e];
    }
    for (int e = 0; e < b; ++e) res[e] = r[e];
}

static int oppositeFace(int f) { return f ^ 1; }

// flux of neighbour J's face touching I, J as inside element (cclocalassembler.hh:186-218)
static void neighbourFlux(const Problem& P, const ElemView& ev, int f, const VolVars& vI, double* out)
{
    const Face& fI = ev.faces[f];
    const int64_t J = fI.outside;
    const Face fJ = P.face(J, oppositeFace(f));
    double r[2] = {0.0, 0.0};
    double fl[2];
    evalFlux(P, J, fJ, ev.vOut[f], vI, fl);
    for (int e = 0; e < P.b; ++e) r[e] += fl[e];
    for (int e = 0; e < P.b; ++e) out[e] = r[e];
}

static void bindElement(const Problem& P, int64_t I, const double* u, const double* uprev, double dt, ElemView& ev)
{
    const int b = P.b;
    ev.I = I;
    ev.vI = volVars(P, u + I * b, I);
    for (int f = 0; f < 2 * P.dim; ++f) {
        ev.faces[f] = P.face(I, f);
        const Face& fc = ev.faces[f];
        if (!fc.boundary) ev.vOut[f] = volVars(P, u + fc.outside * b, fc.outside);
        else if (P.d.bc_type[fc.bidx] == 1) ev.vOut[f] = volVars(P, P.d.bc_values + fc.bidx * b, I);
        else ev.vOut[f] = ev.vI;   // unused for Neumann faces
    }
    ev.transient = dt > 0.0;
    ev.dt = dt;
    if (ev.transient) ev.vPrev = volVars(P, uprev + I * b, I);
}

static double numericEpsilon(const Problem& P, double x, int pv)
{
    const double mag = P.d.privar_magnitude[pv];
    const double base = P.d.base_epsilon > 0 ? P.d.base_epsilon : 1e-10;
    if (mag > 0.0) return base * mag;
    return base * (std::abs(x) + 1.0);
}

struct Pattern {
    std::vector<int64_t> rowPtr;
    std::vector<int32_t> col;
    std::vector<int64_t> diag;               // block index of (I,I)
    std::vector<int64_t> colBlock;           // per cell I, per face f: block index of (J,I), -1 if none
    std::vector<int64_t> rowBlock;           // per cell I, per face f: block index of (I,J), -1 if none
};

static Pattern mpfaPattern(const Problem& P);
static Pattern buildPattern(const Problem& P)
{
    if (P.d.discretization == 1) return mpfaPattern(P);
    Pattern pt;
    const int nf = 2 * P.dim;
    std::vector<std::vector<int32_t>> rows(P.N);
    for (int64_t I = 0; I < P.N; ++I) {
        rows[I].push_back((int32_t)I);
        for (int f = 0; f < nf; ++f) {
            const Face fc = P.face(I, f);
            if (!fc.boundary) rows[fc.outside].push_back((int32_t)I);
        }
    }
    pt.rowPtr.resize(P.N + 1);
    pt.rowPtr[0] = 0;
    for (int64_t I = 0; I < P.N; ++I) {
        std::sort(rows[I].begin(), rows[I].end());
        rows[I].erase(std::unique(rows[I].begin(), rows[I].end()), rows[I].end());
        pt.rowPtr[I + 1] = pt.rowPtr[I] + (int64_t)rows[I].size();
    }
    pt.col.resize(pt.rowPtr[P.N]);
    for (int64_t I = 0; I < P.N; ++I) std::copy(rows[I].begin(), rows[I].end(), pt.col.begin() + pt.rowPtr[I]);
    auto find = [&](int64_t row, int64_t c) -> int64_t {
        auto b0 = pt.col.begin() + pt.rowPtr[row], b1 = pt.col.begin() + pt.rowPtr[row + 1];
        auto it = std::lower_bound(b0, b1, (int32_t)c);
        return (it != b1 && *it == c) ? (int64_t)(it - pt.col.begin()) : -1;
    };
    pt.diag.resize(P.N);
    pt.colBlock.assign(P.N * nf, -1);
    pt.rowBlock.assign(P.N * nf, -1);
    for (int64_t I = 0; I < P.N; ++I) {
        pt.diag[I] = find(I, I);
        for (int f = 0; f < nf; ++f) {
            const Face fc = P.face(I, f);
            if (!fc.boundary) {
                pt.colBlock[I * nf + f] = find(fc.outside, I);
                pt.rowBlock[I * nf + f] = find(I, fc.outside);
            }
        }
    }
    return pt;
}

// ---------------------------------------------------------------- MPFA-O (1p)
// Cell-centred MPFA-O of dumux/discretization/cellcentered/mpfa/omethod for the 1p model on
// the tensor-product grid, continuity points at the face centres (MPFA.Q = 0):
//   * sub control volume faces: every element face split at its corners, the scvf of corner
//     c joining the facet centre and the corner vertex (helper.hh:122-167, 344-462;
//     fvgridgeometry.hh:300-350); scvfs in element order: faces by index in the element,
//     corners in reference-element order;
//   * interaction volume of a vertex: the scvs and scvfs around it; in each scv the basis
//     vectors from the cell centre to the integration points of its scvfs at the vertex, their
//     inner normals and determinant (localsubcontrolentities.hh:43-83, helper.hh:58-109,
//     255-299), w = n^T K nu area extrusion / detX (computetransmissibility.hh:32-50);
//   * local matrices A, B, C, D with the Dirichlet faces as knowns and interior/Neumann
//     faces as unknowns (omethod/localassembler.hh:150-330), T = D + (C A^-1) B
//     (localassemblerhelper.hh:70-80); gravity g = alpha rho area + C A^-1 deltaG
//     (localassemblerbase.hh:125-222);
//   * the advective flux of an scvf: (T u + g) * density * mobility (flux/ccmpfa/
//     darcyslaw.hh:150-205), negated for the element on the outside of the IV face;
//     Neumann scvfs: the given flux times area and extrusion (cclocalresidual.hh:89-97);
//   * numeric Jacobian as CCLocalAssembler<numeric> (cclocalassembler.hh:164-348): column I
//     from the perturbation of element I's unknown, the diagonal from I's whole residual, the
//     entry of neighbour J from J's scvf fluxes whose interaction volume contains I.
// The IV transmissibilities of the incompressible model are solution independent and are
// computed once per assembly call.

struct MpIvTerm { int64_t cell; double t; };
struct MpScvfRow {
    bool neumann = false;
    double c0 = 0.0;                 // 1p: Dirichlet part + gravity (IV faces), flux (Neumann)
    double c0p[2] = {0.0, 0.0};      // 2p: per phase Dirichlet part + gravity (IV faces)
    double neu[2] = {0.0, 0.0};      // 2p: per equation Neumann flux * area * extrusion
    std::vector<MpIvTerm> terms;     // IV cells in position order (existing cells only)
    int64_t outside = -1;            // the cell across the face, or -1 (boundary: bidx)
    int64_t bidx = -1;
};

// Gauss-Jordan elimination with partial pivoting: the inverse of A (n x n), in place
static void gjInverse(std::vector<double>& A, int n)
{
    std::vector<double> I((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) I[(size_t)i * n + i] = 1.0;
    for (int c = 0; c < n; ++c) {
        int p = c;
        for (int r = c + 1; r < n; ++r)
            if (std::fabs(A[(size_t)r * n + c]) > std::fabs(A[(size_t)p * n + c])) p = r;
        if (A[(size_t)p * n + c] == 0.0) throw std::invalid_argument("singular interaction-volume system");
        if (p != c)
            for (int k = 0; k < n; ++k) { std::swap(A[(size_t)p * n + k], A[(size_t)c * n + k]); std::swap(I[(size_t)p * n + k], I[(size_t)c * n + k]); }
        const double inv = 1.0 / A[(size_t)c * n + c];
        for (int k = 0; k < n; ++k) { A[(size_t)c * n + k] *= inv; I[(size_t)c * n + k] *= inv; }
        for (int r = 0; r < n; ++r) {
            if (r == c) continue;
            const double f = A[(size_t)r * n + c];
            if (f == 0.0) continue;
            for (int k = 0; k < n; ++k) { A[(size_t)r * n + k] -= f * A[(size_t)c * n + k]; I[(size_t)r * n + k] -= f * I[(size_t)c * n + k]; }
        }
    }
    A.swap(I);
}

static double mpVtmv(const Problem& P, int64_t cell, const double* n, const double* v)
{
    const int dim = P.dim;
    if (!P.d.permeability_tensor) {
        double s = 0.0;
        for (int i = 0; i < dim; ++i) s += n[i] * v[i];
        return P.d.permeability[cell] * s;
    }
    const double* K = P.d.permeability_tensor + (size_t)cell * dim * dim;
    double Kv[3] = {0, 0, 0};
    for (int i = 0; i < dim; ++i) { double s = 0.0; for (int j = 0; j < dim; ++j) s += K[i * dim + j] * v[j]; Kv[i] = s; }
    double s = 0.0;
    for (int i = 0; i < dim; ++i) s += n[i] * Kv[i];
    return s;
}

// The flux rows of every scvf of every element.
static std::vector<std::vector<MpScvfRow>> mpfaRows(const Problem& P)
{
    const int dim = P.dim, corners = 1 << (dim - 1), nPos = 1 << dim;
    const int nScvf = 2 * dim * corners;
    std::vector<std::vector<MpScvfRow>> rows(P.N, std::vector<MpScvfRow>(nScvf));
    const double rho = P.d.density[0];
    const bool grav = P.d.enable_gravity != 0;
    const int64_t nv[3] = {P.n[0] + 1, P.n[1] + 1, dim == 3 ? P.n[2] + 1 : 1};
    // the cell at IV position `pos` of vertex v, or -1
    auto cellAt = [&](const int64_t* v, int pos, int64_t* id) -> int64_t {
        for (int a = 0; a < 3; ++a) id[a] = a < dim ? v[a] - 1 + ((pos >> a) & 1) : 0;
        for (int a = 0; a < dim; ++a) if (id[a] < 0 || id[a] >= P.n[a]) return -1;
        return id[0] + P.n[0] * (id[1] + P.n[1] * id[2]);
    };
#pragma omp parallel for schedule(dynamic, 64) num_threads(orc_get_threads())
    for (int64_t vi = 0; vi < nv[0] * nv[1] * nv[2]; ++vi) {
        const int64_t v[3] = {vi % nv[0], (vi / nv[0]) % nv[1], vi / (nv[0] * nv[1])};
        double xv[3] = {0, 0, 0};
        for (int a = 0; a < dim; ++a) xv[a] = P.d.coords[a][v[a]];
        int64_t cell[8], cid[8][3];
        for (int q = 0; q < nPos; ++q) cell[q] = cellAt(v, q, cid[q]);
        // faces of the IV: for each axis the corners-many pairs (lower, upper) of positions
        struct F { int a, lo, hi, P, Q; bool bnd, dir; double uD, n[3], area; int64_t bidx; int dof, kn; };
        std::vector<F> faces;
        for (int a = 0; a < dim; ++a)
            for (int q = 0; q < nPos; ++q) {
                if ((q >> a) & 1) continue;
                F f{};
                f.a = a; f.lo = q; f.hi = q | (1 << a);
                if (cell[f.lo] < 0 && cell[f.hi] < 0) continue;
                f.P = cell[f.lo] >= 0 ? f.lo : f.hi;
                f.Q = (cell[f.lo] >= 0 && cell[f.hi] >= 0) ? f.hi : -1;
                f.bnd = f.Q < 0;
                f.n[a] = f.P == f.lo ? 1.0 : -1.0;
                const int64_t* pid = cid[f.P];
                f.area = 1.0;
                for (int k = 0; k < dim; ++k) if (k != a) f.area *= 0.5 * (P.hi(k, pid[k]) - P.lo(k, pid[k]));
                f.bidx = -1; f.dir = false; f.uD = 0.0;
                if (f.bnd) {
                    const Face fc = P.face(cell[f.P], 2 * a + (f.P == f.lo ? 1 : 0));
                    f.bidx = fc.bidx;
                    f.dir = P.d.bc_type[f.bidx] == 1;
                    f.uD = P.d.bc_values[f.bidx * P.b];
                }
                faces.push_back(f);
            }
        const int nF = (int)faces.size();
        // knowns: existing cells by position, then Dirichlet faces; unknowns: the other faces
        int cellKnown[8], nCells = 0, nU = 0, nD = 0;
        for (int q = 0; q < nPos; ++q) cellKnown[q] = cell[q] >= 0 ? nCells++ : -1;
        for (F& f : faces) { if (f.dir) f.kn = nCells + nD++; else f.dof = nU++; }
        const int nK = nCells + nD;
        auto faceOf = [&](int pos, int a) -> int {
            const int lo = pos & ~(1 << a);
            for (int k = 0; k < nF; ++k) if (faces[k].a == a && faces[k].lo == lo) return k;
            return -1;
        };
        // scv bases and inner normals
        double nu[8][3][3] = {}, detX[8] = {};
        for (int q = 0; q < nPos; ++q) {
            if (cell[q] < 0) continue;
            double xc[3]; P.center(cell[q], xc);
            double e[3][3] = {};
            for (int a = 0; a < dim; ++a) {
                double ip[3];
                for (int k = 0; k < 3; ++k) ip[k] = xc[k];
                ip[a] = xv[a];                               // facet centre of the face toward v
                for (int k = 0; k < 3; ++k) e[a][k] = ip[k] - xc[k];
            }
            if (dim == 2) {
                const double cr = e[0][0] * e[1][1] - e[0][1] * e[1][0];
                double n0[2] = {e[1][1], -e[1][0]}, n1[2] = {e[0][1], -e[0][0]};
                if (std::signbit(cr)) { n0[0] = -n0[0]; n0[1] = -n0[1]; }
                else { n1[0] = -n1[0]; n1[1] = -n1[1]; }
                nu[q][0][0] = n0[0]; nu[q][0][1] = n0[1];
                nu[q][1][0] = n1[0]; nu[q][1][1] = n1[1];
                detX[q] = std::abs(cr);
            } else {
                auto crossP = [](const double* x, const double* y, double* o) {
                    o[0] = x[1] * y[2] - x[2] * y[1]; o[1] = x[2] * y[0] - x[0] * y[2]; o[2] = x[0] * y[1] - x[1] * y[0];
                };
                double c12[3]; crossP(e[1], e[2], c12);
                const double tp = e[0][0] * c12[0] + e[0][1] * c12[1] + e[0][2] * c12[2];
                crossP(e[1], e[2], nu[q][0]); crossP(e[2], e[0], nu[q][1]); crossP(e[0], e[1], nu[q][2]);
                if (std::signbit(tp)) for (auto& r : nu[q]) for (double& z : r) z = -z;
                detX[q] = std::abs(tp);
            }
        }
        auto omega = [&](int q, const F& f, double* w) {
            const int64_t c = cell[q];
            for (int a = 0; a < dim; ++a) {
                double t = mpVtmv(P, c, f.n, nu[q][a]);
                t *= f.area * P.extr(c);
                t /= detX[q];
                w[a] = t;
            }
        };
        std::vector<double> A((size_t)nU * nU, 0.0), B((size_t)nU * nK, 0.0), C((size_t)nF * nU, 0.0),
            D((size_t)nF * nK, 0.0);
        for (int fi = 0; fi < nF; ++fi) {
            const F& f = faces[fi];
            double w[3];
            omega(f.P, f, w);
            for (int a = 0; a < dim; ++a) {
                const F& o = faces[faceOf(f.P, a)];
                if (!o.dir) { C[(size_t)fi * nU + o.dof] -= w[a]; if (!f.dir) A[(size_t)f.dof * nU + o.dof] -= w[a]; }
                else { D[(size_t)fi * nK + o.kn] -= w[a]; if (!f.dir) B[(size_t)f.dof * nK + o.kn] += w[a]; }
                D[(size_t)fi * nK + cellKnown[f.P]] += w[a];
                if (!f.dir) B[(size_t)f.dof * nK + cellKnown[f.P]] -= w[a];
            }
            if (!f.bnd) {
                double wq[3];
                omega(f.Q, f, wq);
                for (int a = 0; a < dim; ++a) {
                    const F& o = faces[faceOf(f.Q, a)];
                    if (!o.dir) A[(size_t)f.dof * nU + o.dof] += wq[a];
                    else B[(size_t)f.dof * nK + o.kn] -= wq[a];
                    B[(size_t)f.dof * nK + cellKnown[f.Q]] += wq[a];
                }
            }
        }
        std::vector<double> T = D, CA((size_t)nF * nU, 0.0);
        if (nU > 0) {
            gjInverse(A, nU);
            for (int fi = 0; fi < nF; ++fi)
                for (int j = 0; j < nU; ++j) { double s2 = 0.0; for (int k = 0; k < nU; ++k) s2 += C[(size_t)fi * nU + k] * A[(size_t)k * nU + j]; CA[(size_t)fi * nU + j] = s2; }
            for (int fi = 0; fi < nF; ++fi)
                for (int j = 0; j < nK; ++j) { double s2 = 0.0; for (int k = 0; k < nU; ++k) s2 += CA[(size_t)fi * nU + k] * B[(size_t)k * nK + j]; T[(size_t)fi * nK + j] += s2; }
        }
        // gravity per phase (rho the phase's density, averaged over the face's cells)
        std::vector<double> gph[2] = {std::vector<double>(nF, 0.0), std::vector<double>(nF, 0.0)};
        if (grav) {
            for (int ph = 0; ph < P.b; ++ph) {
                const double rhoPh = P.d.density[ph];
                std::vector<double>& g = gph[ph];
                std::vector<double> dG(nU, 0.0);
                for (int fi = 0; fi < nF; ++fi) {
                    const F& f = faces[fi];
                    const double aIn = P.extr(cell[f.P]) * mpVtmv(P, cell[f.P], f.n, P.g);
                    double r = rhoPh;
                    if (!f.dir) {
                        double d = 0.0; int nOut = 0;
                        if (!f.bnd) { r += rhoPh; d += P.extr(cell[f.Q]) * mpVtmv(P, cell[f.Q], f.n, P.g); nOut = 1; }
                        r /= nOut + 1;
                        d -= aIn;
                        d *= r * f.area;
                        dG[f.dof] = d;
                    }
                    g[fi] = aIn * r * f.area;
                }
                for (int fi = 0; fi < nF; ++fi) { double s2 = g[fi]; for (int k = 0; k < nU; ++k) s2 += CA[(size_t)fi * nU + k] * dG[k]; g[fi] = s2; }
            }
        }
        const std::vector<double>& g = gph[0];
        (void)rho;
        // rows of the scvfs of P (as computed) and of Q (negated)
        for (int fi = 0; fi < nF; ++fi) {
            const F& f = faces[fi];
            double c0 = 0.0;
            for (const F& fd : faces) if (fd.dir) c0 += T[(size_t)fi * nK + fd.kn] * fd.uD;
            c0 += g[fi];
            // 2p: the Dirichlet ghosts' phase pressures (built with the inside cell's spatial
            // parameters, elementvolumevariables.hh) and each phase's gravity
            double c0p[2] = {0.0, 0.0};
            if (P.b == 2)
                for (int ph = 0; ph < 2; ++ph) {
                    double cp = 0.0;
                    for (const F& fd : faces)
                        if (fd.dir) {
                            const VolVars gv = volVars(P, P.d.bc_values + fd.bidx * 2, cell[fd.P]);
                            cp += T[(size_t)fi * nK + fd.kn] * gv.p[ph];
                        }
                    cp += gph[ph][fi];
                    c0p[ph] = cp;
                }
            for (int side = 0; side < 2; ++side) {
                const int q = side == 0 ? f.P : f.Q;
                if (q < 0) continue;
                const int64_t I = cell[q];
                const int fSide = ((q >> f.a) & 1) ? 0 : 1;          // the element face toward v
                int corner = 0, bit = 0;
                for (int k = 0; k < dim; ++k) if (k != f.a) corner |= (((q >> k) & 1) ? 0 : 1) << bit++;
                MpScvfRow& row = rows[I][(2 * f.a + fSide) * corners + corner];
                const Face fc = P.face(I, 2 * f.a + fSide);
                if (fc.boundary && P.d.bc_type[fc.bidx] == 2) {
                    double area = 1.0;
                    int64_t id[3]; P.ijk(I, id);
                    for (int k = 0; k < dim; ++k) if (k != f.a) area *= 0.5 * (P.hi(k, id[k]) - P.lo(k, id[k]));
                    const double sA = area * P.extr(I);
                    row.neumann = true;
                    double qn = 0.0;
                    qn += P.d.bc_values[fc.bidx * P.b] * sA;
                    row.c0 = qn;
                    for (int e = 0; e < P.b; ++e) {
                        double q2 = 0.0;
                        q2 += P.d.bc_values[fc.bidx * P.b + e] * sA;
                        row.neu[e] = q2;
                    }
                    continue;
                }
                row.terms.clear();
                for (int qq = 0; qq < nPos; ++qq)
                    if (cell[qq] >= 0) {
                        const double t = T[(size_t)fi * nK + cellKnown[qq]];
                        row.terms.push_back({cell[qq], side == 0 ? t : -t});
                    }
                row.c0 = side == 0 ? c0 : -c0;
                for (int ph = 0; ph < 2; ++ph) row.c0p[ph] = side == 0 ? c0p[ph] : -c0p[ph];
                row.outside = fc.boundary ? -1 : fc.outside;
                row.bidx = fc.boundary ? fc.bidx : -1;
            }
        }
    }
    return rows;
}

static Pattern mpfaPattern(const Problem& P)
{
    Pattern pt;
    pt.rowPtr.assign(P.N + 1, 0);
    pt.diag.assign(P.N, -1);
    for (int64_t I = 0; I < P.N; ++I) {
        int64_t id[3]; P.ijk(I, id);
        for (int oz = (P.dim == 3 ? -1 : 0); oz <= (P.dim == 3 ? 1 : 0); ++oz)
            for (int oy = -1; oy <= 1; ++oy)
                for (int ox = -1; ox <= 1; ++ox) {
                    const int64_t x = id[0] + ox, y = id[1] + oy, z = id[2] + oz;
                    if (x < 0 || x >= P.n[0] || y < 0 || y >= P.n[1] || z < 0 || z >= P.n[2]) continue;
                    const int64_t J = x + P.n[0] * (y + P.n[1] * z);
                    if (J == I) pt.diag[I] = (int64_t)pt.col.size();
                    pt.col.push_back((int32_t)J);
                }
        pt.rowPtr[I + 1] = (int64_t)pt.col.size();
    }
    return pt;
}

static double mpScvfFlux(const MpScvfRow& row, const double* u, int64_t pert, double q, double mob)
{
    if (row.neumann) return row.c0;
    double t = 0.0;
    for (const MpIvTerm& k : row.terms) t += k.t * (k.cell == pert ? q : u[k.cell]);
    t += row.c0;
    return t * mob;
}

// Residual and numeric-difference Jacobian of the MPFA-O 1p model (column-wise as the
// reference's local assembler: element I perturbs its unknown and differentiates its own
// residual and the fluxes of its neighbours' scvfs that depend on it)
static void mpfaAssemble(const Problem& P, const Pattern& pt, const double* u, double dt, double* values, double* r)
{
    const auto rows = mpfaRows(P);
    const double mob = P.d.density[0] * (1.0 / P.d.viscosity[0]);
    const int method = P.d.numeric_difference_method;
    auto residual = [&](int64_t I, int64_t pert, double q) {
        double res = 0.0;
        {
            double src = 0.0;
            if (P.d.source) src += P.d.source[I];
            src *= P.volume(I) * P.extr(I);
            res -= src;
        }
        for (const MpScvfRow& row : rows[I]) res += mpScvfFlux(row, u, pert, q, mob);
        if (dt > 0.0) res += 0.0;      // incompressible 1p: the storage does not change
        return res;
    };
    auto dependsOn = [&](const MpScvfRow& row, int64_t I) {
        if (row.neumann) return false;
        for (const MpIvTerm& k : row.terms) if (k.cell == I) return true;
        return false;
    };
    auto neighbourFlux = [&](int64_t J, int64_t I, double q) {
        double s = 0.0;
        for (const MpScvfRow& row : rows[J]) if (dependsOn(row, I)) s += mpScvfFlux(row, u, I, q, mob);
        return s;
    };
    auto find = [&](int64_t row, int64_t c) -> int64_t {
        for (int64_t k = pt.rowPtr[row]; k < pt.rowPtr[row + 1]; ++k) if (pt.col[k] == c) return k;
        return -1;
    };
    if (values) std::fill(values, values + pt.rowPtr[P.N], 0.0);
    // analytic (CCLocalAssembler<analytic>, incompressiblelocalresidual.hh:126-160, 221-233):
    // row I collects, scvf by scvf in element order, (+/-) t_J * rho / mu for every IV cell J of
    // its non-Neumann scvfs
    const double up = P.d.density[0] / P.d.viscosity[0];
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
    for (int64_t I = 0; I < P.N; ++I) {
        r[I] = residual(I, -1, 0.0);
        if (!values) continue;
        if (P.d.diff_method == 1) {
            for (const MpScvfRow& row : rows[I]) {
                if (row.neumann) continue;
                for (const MpIvTerm& k : row.terms) values[find(I, k.cell)] += k.t * up;
            }
            continue;
        }
        const double x = u[I];
        const double eps = numericEpsilon(P, x, 0);
        // column I: rows J of the neighbourhood (J == I: whole residual)
        for (int64_t k = pt.rowPtr[I]; k < pt.rowPtr[I + 1]; ++k) {
            const int64_t J = pt.col[k];
            auto f = [&](double q) { return J == I ? residual(I, I, q) : neighbourFlux(J, I, q); };
            const double f0 = J == I ? r[I] : neighbourFlux(J, I, x);
            double d;
            if (method == 1) d = (f(x + eps) - f0) / eps;
            else if (method == -1) d = (f0 - f(x - eps)) / eps;
            else if (method == 0) d = (f(x + eps) - f(x - eps)) / (eps + eps);
            else {
                const double fp = f(x + eps), fm = f(x - eps), fm2 = f(x - 2.0 * eps), fp2 = f(x + 2.0 * eps);
                d = fp; d -= fm; d *= 8.0; d += fm2; d -= fp2; d /= 12.0 * eps;
            }
            values[find(J, I)] = d;
        }
    }
}

// The 2p immiscible model (p0s1) with MPFA-O fluxes: per phase the Darcy flux T p_alpha + g_alpha
// over the IV's cells (the phase pressures of their volume variables) times the upwinded
// density * mobility (flux/upwindscheme.hh), the source, and the storage of the time
// derivative; numeric Jacobian column-wise as the reference's local assembler, the element's
// unknowns perturbed one at a time (cclocalassembler.hh:164-348).
static void mpfaAssemble2p(const Problem& P, const Pattern& pt, const double* u, const double* uprev, double dt,
                           double* values, double* r)
{
    const auto rows = mpfaRows(P);
    const int method = P.d.numeric_difference_method;
    const double w = P.d.upwind_weight;
    std::vector<VolVars> vv(P.N);
    for (int64_t c = 0; c < P.N; ++c) vv[c] = volVars(P, u + c * 2, c);
    auto flux = [&](const MpScvfRow& row, int64_t I, int ph, int64_t pert, const VolVars* vp) {
        double t = 0.0;
        for (const MpIvTerm& k : row.terms) t += k.t * (k.cell == pert ? vp->p[ph] : vv[k.cell].p[ph]);
        t += row.c0p[ph];
        const VolVars& vin = I == pert ? *vp : vv[I];
        VolVars gh;
        const VolVars* vo;
        if (row.outside >= 0) vo = row.outside == pert ? vp : &vv[row.outside];
        else {
            gh = volVars(P, P.d.bc_values + row.bidx * 2, I);
            vo = &gh;
        }
        const double upIn = vin.rho[ph] * vin.mob[ph];
        const double upOut = vo->rho[ph] * vo->mob[ph];
        double mult;
        if (std::signbit(t)) mult = w * upOut + (1.0 - w) * upIn;
        else mult = w * upIn + (1.0 - w) * upOut;
        return t * mult;
    };
    auto residual = [&](int64_t I, int64_t pert, const VolVars* vp, double* res) {
        const double V = P.volume(I);
        double rr[2] = {0.0, 0.0};
        {
            double src[2] = {0.0, 0.0};
            if (P.d.source) for (int e = 0; e < 2; ++e) src[e] += P.d.source[I * 2 + e];
            const double sV = V * P.extr(I);
            for (int e = 0; e < 2; ++e) { src[e] *= sV; rr[e] -= src[e]; }
        }
        for (const MpScvfRow& row : rows[I]) {
            if (row.neumann) {
                for (int e = 0; e < 2; ++e) rr[e] += row.neu[e];
                continue;
            }
            for (int ph = 0; ph < 2; ++ph) rr[ph] += flux(row, I, ph, pert, vp);
        }
        if (dt > 0.0) {
            const VolVars vpr = volVars(P, uprev + I * 2, I);
            const VolVars& vi = I == pert ? *vp : vv[I];
            double st[2] = {0.0, 0.0};
            for (int ph = 0; ph < 2; ++ph) {
                double prevS = vpr.phi * vpr.rho[ph] * vpr.S[ph];
                double curS = vi.phi * vi.rho[ph] * vi.S[ph];
                prevS *= vpr.extr;
                curS *= vi.extr;
                curS -= prevS;
                curS *= V;
                curS /= dt;
                st[ph] += curS;
            }
            for (int e = 0; e < 2; ++e) rr[e] += st[e];
        }
        res[0] = rr[0];
        res[1] = rr[1];
    };
    auto dependsOn = [&](const MpScvfRow& row, int64_t I) {
        if (row.neumann) return false;
        for (const MpIvTerm& k : row.terms) if (k.cell == I) return true;
        return false;
    };
    auto neighbourFlux = [&](int64_t J, int64_t I, const VolVars* vp, double* out) {
        double s2[2] = {0.0, 0.0};
        for (const MpScvfRow& row : rows[J])
            if (dependsOn(row, I))
                for (int ph = 0; ph < 2; ++ph) s2[ph] += flux(row, J, ph, vp ? I : -1, vp);
        out[0] = s2[0];
        out[1] = s2[1];
    };
    auto find = [&](int64_t row, int64_t c) -> int64_t {
        for (int64_t k = pt.rowPtr[row]; k < pt.rowPtr[row + 1]; ++k) if (pt.col[k] == c) return k;
        return -1;
    };
    if (values) std::fill(values, values + pt.rowPtr[P.N] * 4, 0.0);
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
    for (int64_t I = 0; I < P.N; ++I) {
        residual(I, -1, nullptr, r + I * 2);
        if (!values) continue;
        for (int pv = 0; pv < 2; ++pv) {
            const double x = u[I * 2 + pv];
            const double eps = numericEpsilon(P, x, pv);
            auto state = [&](double q) {
                double pvq[2] = {u[I * 2], u[I * 2 + 1]};
                pvq[pv] = q;
                return volVars(P, pvq, I);
            };
            for (int64_t k = pt.rowPtr[I]; k < pt.rowPtr[I + 1]; ++k) {
                const int64_t J = pt.col[k];
                auto f = [&](double q, double* o) {
                    const VolVars vp = state(q);
                    if (J == I) residual(I, I, &vp, o);
                    else neighbourFlux(J, I, &vp, o);
                };
                double f0[2];
                if (J == I) { f0[0] = r[I * 2]; f0[1] = r[I * 2 + 1]; }
                else neighbourFlux(J, I, nullptr, f0);
                double d[2];
                if (method == 1) {
                    double fp[2]; f(x + eps, fp);
                    for (int e = 0; e < 2; ++e) d[e] = (fp[e] - f0[e]) / eps;
                } else if (method == -1) {
                    double fm[2]; f(x - eps, fm);
                    for (int e = 0; e < 2; ++e) d[e] = (f0[e] - fm[e]) / eps;
                } else if (method == 0) {
                    double fp[2], fm[2]; f(x + eps, fp); f(x - eps, fm);
                    for (int e = 0; e < 2; ++e) d[e] = (fp[e] - fm[e]) / (eps + eps);
                } else {
                    double fp[2], fm[2], fm2[2], fp2[2];
                    f(x + eps, fp); f(x - eps, fm); f(x - 2.0 * eps, fm2); f(x + 2.0 * eps, fp2);
                    for (int e = 0; e < 2; ++e) {
                        double t = fp[e]; t -= fm[e]; t *= 8.0; t += fm2[e]; t -= fp2[e]; d[e] = t / (12.0 * eps);
                    }
                }
                const int64_t blk = find(J, I);
                for (int e = 0; e < 2; ++e) values[blk * 4 + e * 2 + pv] = d[e];
            }
        }
    }
}

// CCLocalAssembler<numeric, implicit>::assembleJacobianAndResidualImpl for element I
static void assembleElement(const Problem& P, const Pattern& pt, int64_t I, const double* u, const double* uprev,
                            double dt, double* values, double* r)
{
    const int b = P.b, nf = 2 * P.dim;
    ElemView ev;
    bindElement(P, I, u, uprev, dt, ev);
    double orig0[2];
    localResidual(P, ev, ev.vI, orig0);
    if (values) {
        double origJ[6][2] = {};
        for (int f = 0; f < nf; ++f)
            if (!ev.faces[f].boundary) neighbourFlux(P, ev, f, ev.vI, origJ[f]);

        const int method = P.d.numeric_difference_method;
        for (int pv = 0; pv < b; ++pv) {
            double pvs[2] = {u[I * b], b > 1 ? u[I * b + 1] : 0.0};
            const double x0 = pvs[pv];
            // evaluates own residual and neighbour fluxes with u_I[pv] = x
            auto eval = [&](double x, double* d0, double (*dJ)[2]) {
                double q[2] = {pvs[0], pvs[1]};
                q[pv] = x;
                const VolVars vDef = volVars(P, q, I);
                localResidual(P, ev, vDef, d0);
                for (int f = 0; f < nf; ++f) {
                    dJ[f][0] = dJ[f][1] = 0.0;
                    if (!ev.faces[f].boundary) neighbourFlux(P, ev, f, vDef, dJ[f]);
                }
            };
            const double eps = numericEpsilon(P, x0, pv);
            double d0[2], dJ[6][2];
            // NumericDifferentiation::partialDerivative (numericdifferentiation.hh:67-123)
            if (method == 5) {
                double a0[2], aJ[6][2];
                eval(x0 + eps, d0, dJ);
                eval(x0 - eps, a0, aJ);
                for (int e = 0; e < b; ++e) { d0[e] -= a0[e]; for (int f = 0; f < nf; ++f) dJ[f][e] -= aJ[f][e]; }
                for (int e = 0; e < b; ++e) { d0[e] *= 8.0; for (int f = 0; f < nf; ++f) dJ[f][e] *= 8.0; }
                eval(x0 - 2.0 * eps, a0, aJ);
                for (int e = 0; e < b; ++e) { d0[e] += a0[e]; for (int f = 0; f < nf; ++f) dJ[f][e] += aJ[f][e]; }
                eval(x0 + 2.0 * eps, a0, aJ);
                for (int e = 0; e < b; ++e) { d0[e] -= a0[e]; for (int f = 0; f < nf; ++f) dJ[f][e] -= aJ[f][e]; }
                const double den = 12.0 * eps;
                for (int e = 0; e < b; ++e) { d0[e] /= den; for (int f = 0; f < nf; ++f) dJ[f][e] /= den; }
            } else {
                double delta = 0.0;
                if (method >= 0) {
                    delta += eps;
                    eval(x0 + eps, d0, dJ);
                } else {
                    for (int e = 0; e < b; ++e) { d0[e] = orig0[e]; for (int f = 0; f < nf; ++f) dJ[f][e] = origJ[f][e]; }
                }
                if (method <= 0) {
                    delta += eps;
                    double a0[2], aJ[6][2];
                    eval(x0 - eps, a0, aJ);
                    for (int e = 0; e < b; ++e) { d0[e] -= a0[e]; for (int f = 0; f < nf; ++f) dJ[f][e] -= aJ[f][e]; }
                } else {
                    for (int e = 0; e < b; ++e) { d0[e] -= orig0[e]; for (int f = 0; f < nf; ++f) dJ[f][e] -= origJ[f][e]; }
                }
                for (int e = 0; e < b; ++e) { d0[e] /= delta; for (int f = 0; f < nf; ++f) dJ[f][e] /= delta; }
            }
            // scatter column pv of block column I
            const int64_t di = pt.diag[I];
            for (int e = 0; e < b; ++e) {
                values[(di * b + e) * b + pv] += d0[e];
                for (int f = 0; f < nf; ++f) {
                    const int64_t blk = pt.colBlock[I * nf + f];
                    if (blk >= 0) values[(blk * b + e) * b + pv] += dJ[f][e];
                }
            }
        }
    }
    for (int e = 0; e < b; ++e) r[I * b + e] = orig0[e];
}

// CCLocalAssembler<analytic, implicit>::assembleJacobianAndResidualImpl
// (cclocalassembler.hh:510-573) for element I: residual, then block row I from the
// storage derivatives and each face's flux derivatives, in that order
// (porousmediumflow/1p/incompressiblelocalresidual.hh:55-123, 204-219;
//  porousmediumflow/2p/incompressiblelocalresidual.hh:80-252, 427-484)
static void assembleElementAnalytic(const Problem& P, const Pattern& pt, int64_t I, const double* u,
                                    const double* uprev, double dt, double* values, double* r)
{
    const int b = P.b, nf = 2 * P.dim;
    ElemView ev;
    bindElement(P, I, u, uprev, dt, ev);
    double res[2];
    localResidual(P, ev, ev.vI, res);
    for (int e = 0; e < b; ++e) r[I * b + e] = res[e];
    if (!values) return;
    double* dII = values + pt.diag[I] * b * b;
    const VolVars& vI = ev.vI;
    if (b == 2 && ev.transient) {
        const double poreVolume = P.volume(I) * vI.phi;
        dII[0 * 2 + 1] -= poreVolume * vI.rho[0] / dt;
        dII[1 * 2 + 1] += poreVolume * vI.rho[1] / dt;
    }
    const double w = P.d.upwind_weight;
    for (int f = 0; f < nf; ++f) {
        const Face& fc = ev.faces[f];
        const bool dirichlet = fc.boundary && P.d.bc_type[fc.bidx] == 1;
        if (fc.boundary && !dirichlet) continue;        // Neumann: no derivative (Robin hook empty)
        const VolVars& vO = ev.vOut[f];
        double* dIJ = dirichlet ? nullptr : values + pt.rowBlock[I * nf + f] * b * b;
        double tij;
        if (b == 1) {
            darcyFlux(P, I, fc, vI, vO, 0, &tij);
            const double up = vI.rho[0] / P.d.viscosity[0];
            const double deriv = tij * up;
            dII[0] += deriv;
            if (dIJ) dIJ[0] -= deriv;
            continue;
        }
        const double flux_w = darcyFlux(P, I, fc, vI, vO, 0, &tij);
        const double flux_n = darcyFlux(P, I, fc, vI, vO, 1, &tij);
        const double iw_w = std::signbit(flux_w) ? (1.0 - w) : w, ow_w = 1.0 - iw_w;
        const double iw_n = std::signbit(flux_n) ? (1.0 - w) : w, ow_n = 1.0 - iw_n;
        const double rhow_muw = vI.rho[0] / P.d.viscosity[0];
        const double rhon_mun = vI.rho[1] / P.d.viscosity[1];
        const double upW_in = vI.rho[0] * vI.mob[0], upN_in = vI.rho[1] * vI.mob[1];
        const double upW_out = vO.rho[0] * vO.mob[0], upN_out = vO.rho[1] * vO.mob[1];
        const auto& lawI = P.law(I);
        const double dKrw_in = -1.0 * lawI.dkrw_dsw(vI.S[0]);
        const double dKrn_in = -1.0 * lawI.dkrn_dsw(vI.S[0]);
        const double dpc_in = -1.0 * lawI.dpc_dsw(vI.S[0]);
        if (dirichlet) {
            const double up_w = upW_in * iw_w + upW_out * ow_w;
            dII[0] += tij * up_w;
            dII[1] += rhow_muw * flux_w * dKrw_in * iw_w;
            const double up_n = upN_in * iw_n + upN_out * ow_n;
            dII[2] += tij * up_n;
            dII[3] += rhon_mun * flux_n * dKrn_in * iw_n;
            dII[3] += tij * dpc_in * up_n;
        } else {
            const auto& lawJ = P.law(fc.outside);
            const double dKrw_out = -1.0 * lawJ.dkrw_dsw(vO.S[0]);
            const double dKrn_out = -1.0 * lawJ.dkrn_dsw(vO.S[0]);
            const double dpc_out = -1.0 * lawJ.dpc_dsw(vO.S[0]);
            const double up_w = upW_in * iw_w + upW_out * ow_w;
            const double up_n = upN_in * iw_n + upN_out * ow_n;
            const double rho_mu_flux_w = rhow_muw * flux_w;
            const double rho_mu_flux_n = rhon_mun * flux_n;
            const double tij_up_w = tij * up_w;
            const double tij_up_n = tij * up_n;
            dII[0] += tij_up_w;
            dIJ[0] -= tij_up_w;
            dII[1] += rho_mu_flux_w * dKrw_in * iw_w;
            dIJ[1] += rho_mu_flux_w * dKrw_out * ow_w;
            dII[2] += tij_up_n;
            dIJ[2] -= tij_up_n;
            dII[3] += rho_mu_flux_n * dKrn_in * iw_n;
            dIJ[3] += rho_mu_flux_n * dKrn_out * ow_n;
            dII[3] += tij_up_n * dpc_in;
            dIJ[3] -= tij_up_n * dpc_out;
        }
    }
}

// colors (partial reassembly): 1 red -- reassemble the element's Jacobian column, 0 green --
// keep it (FVAssembler::assemble_ with PartialReassembler::resetJacobian, fvassembler.hh:461-510,
// partialreassembler.hh:360-376, and CCLocalAssemblerBase::assembleJacobianAndResidual)
static void assemble(const Problem& P, const Pattern& pt, const double* u, const double* uprev, double dt,
                     double* values, double* r, const uint8_t* colors = nullptr)
{
    if (P.d.discretization == 1) {
        if (P.b == 2) mpfaAssemble2p(P, pt, u, uprev, dt, values, r);
        else mpfaAssemble(P, pt, u, dt, values, r);
        return;
    }
    const int b = P.b, bb = b * b, nf = 2 * P.dim;
    if (values && colors && P.d.diff_method != 1) {
        // reset the columns of the non-green elements only
        for (int64_t I = 0; I < P.N; ++I) {
            if (!colors[I]) continue;
            std::fill(values + pt.diag[I] * bb, values + (pt.diag[I] + 1) * bb, 0.0);
            for (int f = 0; f < nf; ++f) {
                const int64_t blk = pt.colBlock[I * nf + f];
                if (blk >= 0) std::fill(values + blk * bb, values + (blk + 1) * bb, 0.0);
            }
        }
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
        for (int64_t I = 0; I < P.N; ++I)
            assembleElement(P, pt, I, u, uprev, dt, colors[I] ? values : nullptr, r);
        return;
    }
    if (values) std::fill(values, values + pt.rowPtr[P.N] * b * b, 0.0);
    // Numeric: column-wise scatter, element I writes only block column I and r[I];
    // analytic: element I writes only block row I and r[I]; both race free.
    const bool analytic = P.d.diff_method == 1;
#pragma omp parallel for schedule(static) num_threads(orc_get_threads())
    for (int64_t I = 0; I < P.N; ++I) {
        if (analytic) assembleElementAnalytic(P, pt, I, u, uprev, dt, values, r);
        else assembleElement(P, pt, I, u, uprev, dt, values, r);
    }
}

// ---------------------------------------------------------------- dune-istl restatement
struct BCRS {
    int64_t n; int b;
    const int64_t* rowPtr; const int32_t* col;
    std::vector<double> val;   // ILU copy
    // level schedules of the lower (forward, factorisation) and upper (backward) triangle:
    // rows of one level depend only on rows of earlier levels, so a level's rows may run in
    // any order with identical results; empty when the linear solve runs sequentially
    std::vector<int64_t> fwdRows, fwdStart, bwdRows, bwdStart;
};

// Threads of the linear solve: 1 (default) runs ILU(0) and BiCGSTAB sequentially as
// dune-istl's SeqILU / BiCGSTABSolver; more threads run the SpMV rows, the vector updates and
// the ILU(0) rows of each wavefront level in parallel.  Every row and every entry is computed
// with the same operations in the same order, and the dot products stay sequential, so the
// results are identical bit for bit.
static int g_linear_threads = 1;

static void buildLevels(BCRS& M)
{
    const int64_t n = M.n;
    std::vector<int> lev(n, 0);
    int maxLev = 0;
    for (int64_t i = 0; i < n; ++i) {
        int l = 0;
        for (int64_t k = M.rowPtr[i]; k < M.rowPtr[i + 1] && M.col[k] < i; ++k) l = std::max(l, lev[M.col[k]] + 1);
        lev[i] = l;
        maxLev = std::max(maxLev, l);
    }
    auto bucket = [&](std::vector<int64_t>& rows, std::vector<int64_t>& start, int nl) {
        start.assign(nl + 2, 0);
        for (int64_t i = 0; i < n; ++i) ++start[lev[i] + 1];
        for (int l = 0; l <= nl; ++l) start[l + 1] += start[l];
        rows.resize(n);
        std::vector<int64_t> pos(start.begin(), start.end() - 1);
        for (int64_t i = 0; i < n; ++i) rows[pos[lev[i]]++] = i;
    };
    bucket(M.fwdRows, M.fwdStart, maxLev);
    std::fill(lev.begin(), lev.end(), 0);
    maxLev = 0;
    for (int64_t i = n - 1; i >= 0; --i) {
        int l = 0;
        for (int64_t k = M.rowPtr[i]; k < M.rowPtr[i + 1]; ++k)
            if (M.col[k] > i) l = std::max(l, lev[M.col[k]] + 1);
        lev[i] = l;
        maxLev = std::max(maxLev, l);
    }
    bucket(M.bwdRows, M.bwdStart, maxLev);
}

static void blkMul(int b, const double* A, const double* B, double* C)   // C = A*B
{
    for (int i = 0; i < b; ++i)
        for (int j = 0; j < b; ++j) {
            double s = 0.0;
            for (int k = 0; k < b; ++k) s += A[i * b + k] * B[k * b + j];
            C[i * b + j] = s;
        }
}

static void blkInvert(int b, double* A)
{
    if (b == 1) { A[0] = 1.0 / A[0]; return; }
    const double det = A[0] * A[3] - A[1] * A[2];
    if (det == 0.0) throw SolverAbort("singular pivot in ILU(0)");
    const double detInv = 1.0 / det;
    const double a00 = A[0], a01 = A[1], a10 = A[2], a11 = A[3];
    A[0] = a11 * detInv;
    A[1] = -a01 * detInv;
    A[2] = -a10 * detInv;
    A[3] = a00 * detInv;
}

// block ILU(0) in place; diagonal blocks hold the inverted pivots afterwards
static void ilu0DecomposeRow(BCRS& M, int64_t i)
{
    const int b = M.b, bb = b * b;
    double tmp[4], L[4];
    {
        int64_t ij = M.rowPtr[i];
        const int64_t endi = M.rowPtr[i + 1];
        for (; ij < endi && M.col[ij] < i; ++ij) {
            const int64_t j = M.col[ij];
            int64_t jj = M.rowPtr[j];
            while (M.col[jj] != j) ++jj;
            blkMul(b, &M.val[ij * bb], &M.val[jj * bb], L);      // L_ij = A_ij * D_j^{-1}
            std::memcpy(&M.val[ij * bb], L, sizeof(double) * bb);
            int64_t ik = ij + 1, jk = jj + 1;
            const int64_t endj = M.rowPtr[j + 1];
            while (ik < endi && jk < endj) {
                if (M.col[ik] == M.col[jk]) {
                    blkMul(b, L, &M.val[jk * bb], tmp);            // A_ik -= L_ij * A_jk
                    for (int e = 0; e < bb; ++e) M.val[ik * bb + e] -= tmp[e];
                    ++ik; ++jk;
                } else if (M.col[ik] < M.col[jk]) ++ik;
                else ++jk;
            }
        }
        if (ij >= endi || M.col[ij] != i) throw SolverAbort("ILU: missing diagonal");
        blkInvert(b, &M.val[ij * bb]);
    }
}

// Runs body(i) over the rows in sequence, or level by level on the solve's threads.
template <class F>
static void forRows(const BCRS& M, bool forward, F&& body)
{
    if (g_linear_threads == 1 || M.fwdStart.empty()) {
        if (forward)
            for (int64_t i = 0; i < M.n; ++i) body(i);
        else
            for (int64_t i = M.n - 1; i >= 0; --i) body(i);
        return;
    }
    const std::vector<int64_t>& rows = forward ? M.fwdRows : M.bwdRows;
    const std::vector<int64_t>& start = forward ? M.fwdStart : M.bwdStart;
    const int nl = (int)start.size() - 1;
    bool failed = false;
#pragma omp parallel num_threads(g_linear_threads > 0 ? g_linear_threads : orc_get_threads())
    for (int l = 0; l < nl; ++l) {
#pragma omp for schedule(static)
        for (int64_t k = start[l]; k < start[l + 1]; ++k) {
            try {
                body(rows[k]);
            } catch (...) {
#pragma omp atomic write
                failed = true;
            }
        }
    }
    if (failed) throw SolverAbort("singular pivot in ILU(0)");
}

static void ilu0Decompose(BCRS& M)
{
    if (g_linear_threads != 1) buildLevels(M);
    forRows(M, true, [&](int64_t i) { ilu0DecomposeRow(M, i); });
}

static void ilu0Apply(const BCRS& M, const double* d, double* v)
{
    const int b = M.b, bb = b * b;
    forRows(M, true, [&](int64_t i) {
        double rhs[2] = {d[i * b], b > 1 ? d[i * b + 1] : 0.0};
        for (int64_t ij = M.rowPtr[i]; ij < M.rowPtr[i + 1] && M.col[ij] < i; ++ij) {
            const double* L = &M.val[ij * bb];
            const double* vj = &v[(int64_t)M.col[ij] * b];
            for (int r = 0; r < b; ++r) {
                double s = 0.0;
                for (int c = 0; c < b; ++c) s += L[r * b + c] * vj[c];
                rhs[r] -= s;
            }
        }
        for (int r = 0; r < b; ++r) v[i * b + r] = rhs[r];
    });
    forRows(M, false, [&](int64_t i) {
        double rhs[2] = {v[i * b], b > 1 ? v[i * b + 1] : 0.0};
        int64_t ii = -1;
        for (int64_t ij = M.rowPtr[i]; ij < M.rowPtr[i + 1]; ++ij) {
            const int64_t j = M.col[ij];
            if (j == i) { ii = ij; continue; }
            if (j < i) continue;
            const double* U = &M.val[ij * bb];
            const double* vj = &v[j * b];
            for (int r = 0; r < b; ++r) {
                double s = 0.0;
                for (int c = 0; c < b; ++c) s += U[r * b + c] * vj[c];
                rhs[r] -= s;
            }
        }
        const double* Dinv = &M.val[ii * bb];
        for (int r = 0; r < b; ++r) {
            double s = 0.0;
            for (int c = 0; c < b; ++c) s += Dinv[r * b + c] * rhs[c];
            v[i * b + r] = s;
        }
    });
}

static int linThreads() { return g_linear_threads > 0 ? g_linear_threads : orc_get_threads(); }

static void spmv(int64_t n, int b, const int64_t* rowPtr, const int32_t* col, const double* A, const double* x, double* y)
{
    const int bb = b * b;
#pragma omp parallel for schedule(static) num_threads(linThreads()) if (g_linear_threads != 1)
    for (int64_t i = 0; i < n; ++i) {
        double acc[2] = {0.0, 0.0};
        for (int64_t k = rowPtr[i]; k < rowPtr[i + 1]; ++k) {
            const double* blk = A + k * bb;
            const double* xj = x + (int64_t)col[k] * b;
            for (int r = 0; r < b; ++r)
                for (int c = 0; c < b; ++c) acc[r] += blk[r * b + c] * xj[c];
        }
        for (int r = 0; r < b; ++r) y[i * b + r] = acc[r];
    }
}

// Summation order of the dot products: 0 (default) sequential, as dune-istl's
// SeqScalarProduct; 1 blocked (sums of 256 consecutive products, then the block sums in
// sequence) -- a second, equally valid order used to measure how far BiCGSTAB's results move
// under a change of summation order alone.
static int g_dot_order = 0;

static double dot(int64_t m, const double* a, const double* c)
{
    if (g_dot_order == 1) {
        double total = 0.0;
        for (int64_t b0 = 0; b0 < m; b0 += 256) {
            double s = 0.0;
            const int64_t e = std::min<int64_t>(m, b0 + 256);
            for (int64_t i = b0; i < e; ++i) s += a[i] * c[i];
            total += s;
        }
        return total;
    }
    double s = 0.0;
    for (int64_t i = 0; i < m; ++i) s += a[i] * c[i];
    return s;
}

static dxg_linear_result bicgstab(int64_t n, int b, const int64_t* rowPtr, const int32_t* col, const double* A,
                                  const double* rhs, double* x, double reduction, int maxit)
{
    const int64_t m = n * b;
    BCRS M{n, b, rowPtr, col, std::vector<double>(A, A + rowPtr[n] * b * b)};
    ilu0Decompose(M);
    std::vector<double> r(rhs, rhs + m), rt(m), p(m, 0.0), v(m, 0.0), t(m), y(m);
    std::fill(x, x + m, 0.0);
    const double EPSILON = 1e-80;
    dxg_linear_result res{};
    double def = std::sqrt(dot(m, r.data(), r.data()));
    const double def0 = def;
    res.initial_defect = def0;
    auto converged = [&](double d) { return d < def0 * reduction || d < 1e-30; };
    auto finish = [&](bool conv, double it, double d) {
        res.converged = conv;
        res.iterations = (int)std::ceil(it);
        res.final_defect = d;
        res.reduction = def0 > 0 ? d / def0 : 0.0;
        return res;
    };
    if (!std::isfinite(def)) throw SolverAbort("non-finite defect");
    if (converged(def)) return finish(true, 0.0, def);
    rt = r;
    double rho = 1, alpha = 1, omega = 1, rho_new, beta, h;
    double it;
    for (it = 0.5; it < maxit; it += .5) {
        rho_new = dot(m, rt.data(), r.data());
        if (std::abs(rho) <= EPSILON) throw SolverAbort("breakdown in BiCGSTAB - rho");
        if (std::abs(omega) <= EPSILON) throw SolverAbort("breakdown in BiCGSTAB - omega");
        if (it < 1)
            p = r;
        else {
            beta = (rho_new / rho) * (alpha / omega);
#pragma omp parallel for schedule(static) num_threads(linThreads()) if (g_linear_threads != 1)
            for (int64_t i = 0; i < m; ++i) p[i] += -omega * v[i];
#pragma omp parallel for schedule(static) num_threads(linThreads()) if (g_linear_threads != 1)
            for (int64_t i = 0; i < m; ++i) p[i] *= beta;
#pragma omp parallel for schedule(static) num_threads(linThreads()) if (g_linear_threads != 1)
            for (int64_t i = 0; i < m; ++i) p[i] += r[i];
        }
        ilu0Apply(M, p.data(), y.data());
        spmv(n, b, rowPtr, col, A, y.data(), v.data());
        h = dot(m, rt.data(), v.data());
        if (std::abs(h) < EPSILON) throw SolverAbort("breakdown in BiCGSTAB - h");
        alpha = rho_new / h;
#pragma omp parallel for schedule(static) num_threads(linThreads()) if (g_linear_threads != 1)
        for (int64_t i = 0; i < m; ++i) x[i] += alpha * y[i];
#pragma omp parallel for schedule(static) num_threads(linThreads()) if (g_linear_threads != 1)
        for (int64_t i = 0; i < m; ++i) r[i] += -alpha * v[i];
        def = std::sqrt(dot(m, r.data(), r.data()));
        if (!std::isfinite(def)) throw SolverAbort("non-finite defect");
        if (converged(def)) return finish(true, it, def);
        it += .5;
        ilu0Apply(M, r.data(), y.data());
        spmv(n, b, rowPtr, col, A, y.data(), t.data());
        omega = dot(m, t.data(), r.data()) / dot(m, t.data(), t.data());
#pragma omp parallel for schedule(static) num_threads(linThreads()) if (g_linear_threads != 1)
        for (int64_t i = 0; i < m; ++i) x[i] += omega * y[i];
#pragma omp parallel for schedule(static) num_threads(linThreads()) if (g_linear_threads != 1)
        for (int64_t i = 0; i < m; ++i) r[i] += -omega * t[i];
        rho = rho_new;
        def = std::sqrt(dot(m, r.data(), r.data()));
        if (!std::isfinite(def)) throw SolverAbort("non-finite defect");
        if (converged(def)) return finish(true, it, def);
    }
    return finish(false, it, def);
}

// ---------------------------------------------------------------- Newton driver
// The reference NewtonSolver<Assembler, LinearSolver> restated over an abstract
// assembler exposing the calls Newton makes (newtonsolver.hh:466-475, 488-524, 869-881).
struct NewtonAssembler {
    virtual ~NewtonAssembler() = default;
    virtual int64_t size() const = 0;                         // scalar entries of u
    virtual int blockSize() const { return 1; }
    // element colors for partial reassembly (nullptr: assemble everything)
    virtual void setColors(const uint8_t*) {}
    virtual void assembleJacobianAndResidual(const std::vector<double>& u) = 0;
    virtual void assembleResidual(const std::vector<double>& u) = 0;
    virtual double residualNorm() const = 0;
    // solves J delta = r, returns converged (throws SolverAbort on breakdown)
    virtual bool solveLinear(std::vector<double>& delta, double reduction, int maxit, int* iters) = 0;
};

struct Newton {
    dxg_newton_params prm;
    int numSteps = 0;
    double shift = 0, lastShift = 0, reduction = 0, lastReduction = 1, residualNorm = 0, initialResidual = 0;
    std::vector<double> uLastIter;
    dxg_newton_report* rep = nullptr;

    bool converged() const
    {
        if (!prm.enable_residual_criterion) return shift <= prm.max_relative_shift;
        return shift <= prm.max_relative_shift || reduction <= prm.residual_reduction;
    }
    bool proceed(bool conv) const
    {
        if (numSteps < prm.min_steps) return true;
        else if (conv) return false;
        else if (numSteps >= prm.max_steps) return shift * 4.0 < lastShift;
        return true;
    }
    static double maxRelShift(const std::vector<double>& a, const std::vector<double>& c)
    {
        double s = 0.0;
        for (size_t i = 0; i < a.size(); ++i) {
            const double v = std::abs(a[i] - c[i]) / std::max<double>(1.0, std::abs(a[i] + c[i]) * 0.5);
            s = std::max(s, v);
        }
        return s;
    }
    void computeResidualReduction(NewtonAssembler& A, const std::vector<double>& u)
    {
        A.assembleResidual(u);
        residualNorm = A.residualNorm();
        reduction = residualNorm / initialResidual;
    }
    // partial reassembly state: distance from the last linearisation and element colors
    std::vector<double> distance;
    std::vector<uint8_t> colors;

    // newtonUpdate's partial-reassembly block (newtonsolver.hh:565-603): threshold from
    // the achieved shift, accumulated per-cell shift, colors, reset of the red distances
    void updateColors(NewtonAssembler& A, const std::vector<double>& u)
    {
        const double tol = prm.max_relative_shift;
        const double minEps = prm.reassembly_min_threshold > 0 ? prm.reassembly_min_threshold : 1e-1 * tol;
        const double maxEps = prm.reassembly_max_threshold > 0 ? prm.reassembly_max_threshold : 1e2 * tol;
        const double threshold = std::max(minEps, std::min(maxEps, shift * prm.reassembly_shift_weight));
        const int b = A.blockSize();
        const size_t n = distance.size();
        for (size_t i = 0; i < n; ++i) {
            double s = 0.0;
            for (int e = 0; e < b; ++e) {
                const double x = uLastIter[i * b + e], y = u[i * b + e];
                s = std::max(s, std::abs(x - y) / std::max<double>(1.0, std::abs(x + y) * 0.5));
            }
            distance[i] += s;
        }
        // PartialReassemblerEngine<CCTpfa>::computeColors: red above the threshold
        for (size_t i = 0; i < n; ++i) colors[i] = distance[i] > threshold ? 1 : 0;
        for (size_t i = 0; i < n; ++i)
            if (colors[i]) distance[i] = 0;
    }

    // solveImpl_ (newtonsolver.hh:976-1072); throws NumericalProblem
    bool solveImpl(NewtonAssembler& A, std::vector<double>& u)
    {
        numSteps = 0;
        uLastIter = u;
        const bool partial = prm.enable_partial_reassembly != 0;
        if (partial) {
            // newtonBegin: resetColors -- everything red
            const size_t n = u.size() / A.blockSize();
            distance.assign(n, 0.0);
            colors.assign(n, 1);
            A.setColors(colors.data());
        }
        std::vector<double> deltaU(u.size(), 0.0);
        bool conv = false;
        using clk = std::chrono::steady_clock;
        while (proceed(conv)) {
            lastShift = shift;
            lastReduction = numSteps == 0 ? 1.0 : reduction;
            if (numSteps > 0) uLastIter = u;
            auto t0 = clk::now();
            A.assembleJacobianAndResidual(u);
            auto t1 = clk::now();
            std::fill(deltaU.begin(), deltaU.end(), 0.0);
            if (numSteps == 0) initialResidual = A.residualNorm();
            int iters = 0;
            bool lconv = false;
            try { lconv = A.solveLinear(deltaU, prm.linear_reduction, prm.linear_max_iter, &iters); }
            catch (const SolverAbort&) { lconv = false; }
            if (!lconv) throw NumericalProblem("Linear solver did not converge");
            auto t2 = clk::now();
            if (prm.use_line_search) {
                double lambda = 1.0;
                std::vector<double> uCur = uLastIter;
                while (true) {
                    for (size_t i = 0; i < u.size(); ++i) uCur[i] += -lambda * deltaU[i];
                    u = uCur;
                    computeResidualReduction(A, u);
                    if (reduction < lastReduction || lambda <= prm.line_search_min_relaxation) break;
                    lambda *= 0.5;
                    uCur = uLastIter;
                }
            } else {
                std::vector<double> uCur = uLastIter;
                for (size_t i = 0; i < u.size(); ++i) uCur[i] += -1.0 * deltaU[i];
                u = uCur;
                if (prm.enable_residual_criterion) computeResidualReduction(A, u);
            }
            shift = maxRelShift(uLastIter, u);
            if (partial) updateColors(A, u);
            auto t3 = clk::now();
            if (rep && numSteps < DXG_MAX_NEWTON_RECORD) {
                rep->shift[numSteps] = shift;
                rep->linear_iters[numSteps] = iters;
                if (prm.record_residual_norms) {
                    if (!(prm.use_line_search || prm.enable_residual_criterion)) {
                        A.assembleResidual(u);
                        residualNorm = A.residualNorm();
                    }
                    rep->residual_norm[numSteps] = residualNorm;
                }
            }
            if (rep) {
                rep->linear_iterations += iters;
                rep->time_assemble += std::chrono::duration<double>(t1 - t0).count();
                rep->time_solve += std::chrono::duration<double>(t2 - t1).count();
                rep->time_update += std::chrono::duration<double>(t3 - t2).count();
            }
            ++numSteps;
            conv = converged();
        }
        return converged();
    }
    bool solve_(NewtonAssembler& A, std::vector<double>& u)
    {
        bool conv = false;
        try { conv = solveImpl(A, u); }
        catch (const NumericalProblem&) { conv = false; }
        return conv;
    }
};

// FVAssembler + ILUBiCGSTABIstlSolver over the problem
struct FVAssembler final : NewtonAssembler {
    const Problem& P;
    const Pattern& pt;
    const double* uprev;
    double dt;
    std::vector<double> J, r;
    FVAssembler(const Problem& p, const Pattern& pat, const double* up, double dt_)
        : P(p), pt(pat), uprev(up), dt(dt_), J(pat.rowPtr[p.N] * p.b * p.b), r(p.N * p.b) {}
    const uint8_t* colors = nullptr;
    int64_t size() const override { return P.N * P.b; }
    int blockSize() const override { return P.b; }
    void setColors(const uint8_t* c) override { colors = c; }
    void assembleJacobianAndResidual(const std::vector<double>& u) override
    {
        assemble(P, pt, u.data(), uprev, dt, J.data(), r.data(), colors);
    }
    void assembleResidual(const std::vector<double>& u) override { assemble(P, pt, u.data(), uprev, dt, nullptr, r.data()); }
    double residualNorm() const override { return std::sqrt(dot((int64_t)r.size(), r.data(), r.data())); }
    bool solveLinear(std::vector<double>& delta, double reduction, int maxit, int* iters) override
    {
        auto res = bicgstab(P.N, P.b, pt.rowPtr.data(), pt.col.data(), J.data(), r.data(), delta.data(), reduction, maxit);
        *iters = res.iterations;
        return res.converged;
    }
};

struct ScalarMock final : NewtonAssembler {
    double jac = 0, res = 0;
    int64_t size() const override { return 1; }
    void assembleResidual(const std::vector<double>& u) override { res = u[0] * u[0] - 5.0; }
    void assembleJacobianAndResidual(const std::vector<double>& u) override { assembleResidual(u); jac = 2.0 * u[0]; }
    double residualNorm() const override { return std::abs(res); }
    bool solveLinear(std::vector<double>& delta, double, int, int* iters) override { delta[0] = res / jac; *iters = 1; return true; }
};

} // namespace orc

using namespace orc;

extern "C" {

void orc_set_threads(int n) { g_threads = n; }
void orc_set_pow_mode(int mode) { g_pow_mode = mode; }
int orc_get_pow_mode(void) { return g_pow_mode; }
void orc_set_linear_threads(int n) { g_linear_threads = n; }
void orc_set_dot_order(int order) { g_dot_order = order; }
void orc_pow_batch(int32_t mode, int64_t n, const double* x, const double* y, double* out)
{
    for (int64_t i = 0; i < n; ++i) out[i] = mode == 1 ? dxg::crPow(x[i], y[i]) : std::pow(x[i], y[i]);
}
int orc_get_threads(void)
{
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
    return 1;
#endif
}

int orc_num_blocks(const dxg_problem_desc* d, int64_t* nnzb)
{
    try {
        Problem P(*d);
        int64_t cnt = P.N;
        if (P.d.discretization == 1) cnt = buildPattern(P).rowPtr[P.N];
        else
            for (int64_t I = 0; I < P.N; ++I)
                for (int f = 0; f < 2 * P.dim; ++f) if (!P.face(I, f).boundary) ++cnt;
        *nnzb = cnt;
        return 0;
    } catch (...) { return DXG_ERR_ARG; }
}

int orc_pattern(const dxg_problem_desc* d, int64_t* row_ptr, int32_t* col_idx)
{
    try {
        Problem P(*d);
        Pattern pt = buildPattern(P);
        std::copy(pt.rowPtr.begin(), pt.rowPtr.end(), row_ptr);
        std::copy(pt.col.begin(), pt.col.end(), col_idx);
        return 0;
    } catch (...) { return DXG_ERR_ARG; }
}

int orc_assemble(const dxg_problem_desc* d, const double* u, const double* u_prev, double dt, double* values, double* r)
{
    try {
        Problem P(*d);
        Pattern pt = buildPattern(P);
        assemble(P, pt, u, u_prev, dt, values, r);
        return 0;
    } catch (...) { return DXG_ERR_ARG; }
}

int orc_linear_solve(int64_t n, int32_t b, const int64_t* row_ptr, const int32_t* col_idx, const double* values,
                     const double* rhs, double* x, double reduction, int32_t max_iter, dxg_linear_result* res)
{
    try {
        *res = bicgstab(n, b, row_ptr, col_idx, values, rhs, x, reduction, max_iter);
        return res->converged ? 0 : DXG_ERR_LINEAR_NOT_CONVERGED;
    } catch (const SolverAbort&) {
        std::memset(res, 0, sizeof(*res));
        return DXG_ERR_LINEAR_BREAKDOWN;
    }
}

int orc_newton_solve(const dxg_problem_desc* d, double* u, const double* u_prev, double dt,
                     const dxg_newton_params* p, dxg_newton_report* rep)
{
    try {
        Problem P(*d);
        Pattern pt = buildPattern(P);
        std::memset(rep, 0, sizeof(*rep));
        std::vector<double> x(u, u + P.N * P.b);
        const std::vector<double> x0 = x;
        Newton nw;
        nw.prm = *p;
        const int divisions = dt > 0 ? p->max_time_step_divisions : 0;
        int wasted = 0;
        dxg_newton_report attempt{};
        for (int i = 0; i <= divisions; ++i) {
            FVAssembler A(P, pt, u_prev, dt);
            attempt = dxg_newton_report{};
            nw.rep = &attempt;
            const bool conv = nw.solve_(A, x);
            attempt.iterations = nw.numSteps;
            attempt.initial_residual = nw.initialResidual;
            attempt.dt_used = dt;
            attempt.converged = conv;
            attempt.time_step_divisions = i;
            attempt.wasted_iterations = wasted;
            if (conv) {
                *rep = attempt;
                std::copy(x.begin(), x.end(), u);
                return 0;
            }
            wasted += nw.numSteps;
            // reset to the previous solution and retry with a reduced time step
            const double* src = u_prev ? u_prev : x0.data();
            x.assign(src, src + P.N * P.b);
            dt *= p->retry_time_step_reduction;
        }
        *rep = attempt;
        rep->converged = 0;
        rep->wasted_iterations = wasted;
        if (u_prev) std::copy(u_prev, u_prev + P.N * P.b, u);
        return DXG_ERR_NEWTON_NOT_CONVERGED;
    } catch (...) { return DXG_ERR_ARG; }
}

double orc_suggest_time_step(int32_t numSteps, double oldTimeStep, const dxg_newton_params* p)
{
    if (numSteps > p->target_steps) {
        const double percent = double(numSteps - p->target_steps) / p->target_steps;
        return oldTimeStep / (1.0 + percent);
    }
    const double percent = double(p->target_steps - numSteps) / p->target_steps;
    return oldTimeStep * (1.0 + percent / 1.2);
}

int orc_brooks_corey(const double* params, int32_t what, int64_t n, const double* sw, double* out)
{
    BrooksCoreyDefault law(params);
    for (int64_t i = 0; i < n; ++i) {
        if (what == 0) out[i] = law.pc(sw[i]);
        else if (what == 1) out[i] = law.krw(sw[i]);
        else out[i] = law.krn(sw[i]);
    }
    return 0;
}

int orc_van_genuchten(const double* params, int32_t what, int64_t n, const double* sw, double* out)
{
    VanGenuchtenDefault law(params);
    for (int64_t i = 0; i < n; ++i) {
        if (what == 0) out[i] = law.pc(sw[i]);
        else if (what == 1) out[i] = law.krw(sw[i]);
        else if (what == 2) out[i] = law.krn(sw[i]);
        else if (what == 3) out[i] = law.dpc_dsw(sw[i]);
        else if (what == 4) out[i] = law.dkrw_dsw(sw[i]);
        else out[i] = law.dkrn_dsw(sw[i]);
    }
    return 0;
}

double orc_numdiff_poly(int32_t method, double eps, double x0)
{
    auto f = [](double x) { return 1.0 / 24.0 * x * x * x * x + 1.0 / 6.0 * x * x * x + 1.0 / 2.0 * x * x + x; };
    const double fx0 = f(x0);
    if (method == 5) {
        double d = f(x0 + eps);
        d -= f(x0 - eps);
        d *= 8.0;
        d += f(x0 - 2.0 * eps);
        d -= f(x0 + 2.0 * eps);
        d /= 12.0 * eps;
        return d;
    }
    double delta = 0.0, d;
    if (method >= 0) { delta += eps; d = f(x0 + eps); }
    else d = fx0;
    if (method <= 0) { delta += eps; d -= f(x0 - eps); }
    else d -= fx0;
    d /= delta;
    return d;
}

int orc_newton_scalar(double x0, const dxg_newton_params* p, double* x_out, int32_t* iterations)
{
    ScalarMock A;
    Newton nw;
    nw.prm = *p;
    std::vector<double> x{x0};
    const bool conv = nw.solve_(A, x);
    *x_out = x[0];
    *iterations = nw.numSteps;
    return conv ? 0 : DXG_ERR_NEWTON_NOT_CONVERGED;
}

} // extern "C"
