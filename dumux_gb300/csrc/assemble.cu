// assemble.cu -- residual and numeric-difference Jacobian of the cc-TPFA scheme.
//
// Two kernels per assembly:
//   volvarsKernel   one thread per cell: volume variables of the cell at its own
//                   solution and at every perturbed state of the numeric
//                   differentiation (OnePVolumeVariables / TwoPVolumeVariables::update,
//                   dumux/porousmediumflow/{1p,2p}/volumevariables.hh), plus the
//                   epsilon of each primary variable (dumux/assembly/numericepsilon.hh:49-53).
//   rowKernel       one thread per cell I: the local residual r_I at the cell's own
//                   states and the whole block row I of the Jacobian.
//
// The reference assembles block columns (CCLocalAssembler<numeric>::assembleJacobian-
// AndResidualImpl, dumux/assembly/cclocalassembler.hh:164-348): element I perturbs its
// own unknowns and differences its own residual (diagonal block A[I][I]) and the
// fluxes of each neighbour J's face towards I, evaluated with J as the inside element
// (off-diagonal block A[J][I]).  Each of those numbers is a function of the two cells'
// volume variables only, so the same value can be produced in row order: A[I][J] is
// the difference of I's flux through the face towards J, with J perturbed, divided by
// J's epsilon.  Evaluating every flux with the reference's operation sequence (no FMA
// contraction in this file) yields the reference's values for every block while each
// volume variable is computed once per (cell, state) instead of once per element that
// binds it, and the rows are written coalesced.
#include <algorithm>

#include "common.cuh"
#include "kernels.cuh"
#include "materiallaw.cuh"

namespace dxg {

// ---------------------------------------------------------------- constitutive laws
// Regularised Brooks-Corey / Van Genuchten: materiallaw.cuh (lawPc, lawKrw, lawKrn and
// their derivatives w.r.t. sw).

// Volume variables needed by the residual: phase pressure, upwind term rho*lambda and
// the storage term (phi*rho*S)*extrusion (immiscible/localresidual.hh:64-86,
// fvlocalresidual.hh:293-297).
template <int B>
__device__ __forceinline__ void volVars(const ProblemConsts& pc, const double* pv, double phi, double extr,
                                        int mat, double* p, double* up, double* st)
{
    if (B == 1) {
        const double mob = 1.0 / pc.viscosity[0];
        p[0] = pv[0];
        up[0] = pc.density[0] * mob;
        double s = phi * pc.density[0] * 1.0;
        s *= extr;
        st[0] = s;
    } else {
        const MaterialLaw& m = pc.law[mat];
        const double Sn = pv[1];
        const double Sw = 1 - Sn;
        const double pcap = lawPc(m, Sw);
        p[0] = pv[0];
        p[1] = pv[0] + pcap;
        const double mobW = lawKrw(m, Sw) / pc.viscosity[0];
        const double mobN = lawKrn(m, Sw) / pc.viscosity[1];
        up[0] = pc.density[0] * mobW;
        up[1] = pc.density[1] * mobN;
        double sW = phi * pc.density[0] * Sw;
        double sN = phi * pc.density[1] * Sn;
        sW *= extr;
        sN *= extr;
        st[0] = sW;
        st[1] = sN;
    }
}

__device__ __forceinline__ double numericEps(const ProblemConsts& pc, double x, int pv)
{
    return pc.magnitude[pv] > 0.0 ? pc.baseEps * pc.magnitude[pv] : pc.baseEps * (fabs(x) + 1.0);
}

// States per cell: 0 = own solution; forward/backward: 1+pv = x[pv] +/- eps;
// central: 1+2pv = x+eps, 2+2pv = x-eps; five-point stencil (NumericDifferentiation,
// dumux/common/numericdifferentiation.hh:79-88, in its order of evaluation): 1+4pv = x+eps,
// 2+4pv = x-eps, 3+4pv = x-2eps, 4+4pv = x+2eps.  METHOD 2 selects state 0 only (residual).
template <int B, int METHOD>
__global__ void volvarsKernel(AssemblyArgs a0, const AssemblyArgs* __restrict__ batch)
{
    constexpr int SP = statesPerPv(METHOD);
    constexpr int NS = 1 + SP * B;
    const AssemblyArgs a = batch ? batch[blockIdx.y] : a0;
    const ProblemConsts& pc = *a.pc;
    const int64_t N = a.N;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
        double x[B];
#pragma unroll
        for (int e = 0; e < B; ++e) x[e] = a.u[i * B + e];
        const double ph = a.phi[i], ex = a.extr[i];
        const int m = (B == 2) ? a.mat[i] : 0;
        // a green cell keeps its Jacobian column: its perturbed states are not needed
        const int ns = (a.color && !a.color[i]) ? 1 : NS;
#pragma unroll
        for (int s = 0; s < NS; ++s) {
            if (s >= ns) break;
            double q[B];
#pragma unroll
            for (int e = 0; e < B; ++e) q[e] = x[e];
            if (s > 0) {
                const int pv = (s - 1) / SP, t = (s - 1) % SP;
                const double ep = numericEps(pc, x[pv], pv);
                if (METHOD == 5) {
                    if (t == 0) q[pv] = x[pv] + ep;
                    else if (t == 1) q[pv] = x[pv] - ep;
                    else if (t == 2) q[pv] = x[pv] - 2.0 * ep;
                    else q[pv] = x[pv] + 2.0 * ep;
                } else {
                    const bool minus = (METHOD == -1) || (METHOD == 0 && t == 1);
                    q[pv] = minus ? x[pv] - ep : x[pv] + ep;
                }
                if (t == 0) a.eps[pv * N + i] = ep;
            }
            double p[B], up[B], st[B];
            volVars<B>(pc, q, ph, ex, m, p, up, st);
#pragma unroll
            for (int k = 0; k < B; ++k) {
                a.vvP[(s * B + k) * N + i] = p[k];
                a.vvU[(s * B + k) * N + i] = up[k];
                a.vvS[(s * B + k) * N + i] = st[k];
            }
        }
        if (METHOD == 3 && B == 2) {
            // derivatives w.r.t. S_n are the negatives of those w.r.t. S_w
            // (2p/incompressiblelocalresidual.hh:198-205)
            const MaterialLaw& law = pc.law[m];
            const double Sw = 1 - x[B - 1];
            a.dvv[i] = -1.0 * lawDkrwDsw(law, Sw);
            a.dvv[N + i] = -1.0 * lawDkrnDsw(law, Sw);
            a.dvv[2 * N + i] = -1.0 * lawDpcDsw(law, Sw);
        }
    }
}

// Storage of the previous time level, ((phi*rho*S)*extr) at u_prev.
template <int B>
__global__ void prevStorageKernel(AssemblyArgs a0, const AssemblyArgs* __restrict__ batch)
{
    const AssemblyArgs a = batch ? batch[blockIdx.y] : a0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.N; i += (int64_t)gridDim.x * blockDim.x) {
        double x[B], p[B], up[B], st[B];
#pragma unroll
        for (int e = 0; e < B; ++e) x[e] = a.uprev[i * B + e];
        volVars<B>(*a.pc, x, a.phi[i], a.extr[i], (B == 2) ? a.mat[i] : 0, p, up, st);
#pragma unroll
        for (int k = 0; k < B; ++k) a.stPrev[k * a.N + i] = st[k];
    }
}

// Darcy flux times upwinded rho*lambda of one phase across one face
// (darcyslaw.hh:153-213, upwindscheme.hh:35-54, fluxvariables.hh:75-98).
// g1 = rho*area*alpha_inside, g2 = rho*tij/outsideTi*(alpha_inside-alpha_outside).
template <bool GRAV, bool FULLUP>
__device__ __forceinline__ double phaseFlux(double tij, double pin, double pout, double upin, double upout,
                                            double g1, double g2, double w)
{
    double flux = tij * (pin - pout);
    if (GRAV) {
        flux = flux + g1;
        flux = flux - g2;
    }
    double mult;
    if (FULLUP) mult = signbit(flux) ? (w * upout + (1.0 - w) * upin) : (w * upin + (1.0 - w) * upout);
    else mult = signbit(flux) ? upout : upin;
    return flux * mult;
}

// Five-point stencil of NumericDifferentiation::partialDerivative (method 5,
// dumux/common/numericdifferentiation.hh:79-88), in its operation order: f(x+e) - f(x-e),
// times 8, + f(x-2e), - f(x+2e), divided by 12 e.
__device__ __forceinline__ double fivePoint(double fp, double fm, double fm2, double fp2, double eps)
{
    double d = fp;
    d -= fm;
    d *= 8.0;
    d += fm2;
    d -= fp2;
    return d / (12.0 * eps);
}

template <int B, int DIM, int METHOD, bool GRAV, bool TRANSIENT, bool FULLUP, bool WANT_JAC>
__device__ __forceinline__ void rowCell(const AssemblyArgs& a, const int64_t I)
{
    constexpr bool ANALYTIC = METHOD == 3;
    constexpr int SP = statesPerPv(METHOD);
    constexpr int NS = ANALYTIC ? 1 : 1 + SP * B;
    constexpr int BB = B * B;
    constexpr int NF = 2 * DIM;
    constexpr int VA = DIM - 1;                 // vertical axis (gravity)
    const int64_t N = a.N;
    const ProblemConsts& pc = *a.pc;
    const double w = pc.upwindWeight;

    // analytic path: diagonal block accumulated in the reference's order -- storage
    // derivatives first (addStorageDerivatives), then each face in turn
    double dII[BB];
    double rhoMu[B], dI[3] = {0.0, 0.0, 0.0};
    if (ANALYTIC && WANT_JAC) {
#pragma unroll
        for (int e = 0; e < BB; ++e) dII[e] = 0.0;
#pragma unroll
        for (int k = 0; k < B; ++k) rhoMu[k] = pc.density[k] / pc.viscosity[k];
        if constexpr (B == 2) {
            dI[0] = a.dvv[I];
            dI[1] = a.dvv[N + I];
            dI[2] = a.dvv[2 * N + I];
            if (TRANSIENT) {
                const double poreVolume = a.vol[I] * a.phi[I];
                dII[0 * B + 1] -= poreVolume * pc.density[0] / a.dt;
                dII[1 * B + 1] += poreVolume * pc.density[1] / a.dt;
            }
        }
    }

    // partial reassembly: the column of a green cell keeps its values
    const bool jacI = WANT_JAC && !(a.color && !a.color[I]);
    // own states
    double pI[NS][B], uI[NS][B];
#pragma unroll
    for (int s = 0; s < (WANT_JAC ? NS : 1); ++s)
#pragma unroll
        for (int k = 0; k < B; ++k) {
            const bool have = s == 0 || jacI;
            pI[s][k] = have ? a.vvP[(s * B + k) * N + I] : 0.0;
            uI[s][k] = have ? a.vvU[(s * B + k) * N + I] : 0.0;
        }
    constexpr int NR = WANT_JAC ? NS : 1;
    double r[NS][B];
#pragma unroll
    for (int s = 0; s < NR; ++s)
#pragma unroll
        for (int e = 0; e < B; ++e) r[s][e] = 0.0 - a.srcterm[e * N + I];

    const int nx = pc.nx, ny = pc.ny;
    const int64_t strides[3] = {1, (int64_t)nx, (int64_t)nx * ny};
    const int ix = (int)(I % nx);
    const int iy = (int)((I / nx) % ny);
    const int iz = (DIM == 3) ? (int)(I / ((int64_t)nx * ny)) : 0;
    const int idx[3] = {ix, iy, iz};
    const int nn[3] = {nx, ny, pc.nz};

#pragma unroll
    for (int f = 0; f < NF; ++f) {
        const int ax = f >> 1, side = f & 1;
        const bool interior = side ? (idx[ax] < nn[ax] - 1) : (idx[ax] > 0);
        const int slot = (side ? DIM + 1 + ax : DIM - 1 - ax);
        if (interior) {
            const int64_t J = side ? I + strides[ax] : I - strides[ax];
            const double tij = a.tijPlus[ax * N + (side ? I : J)];
            double g1[B], g2[B];
#pragma unroll
            for (int k = 0; k < B; ++k) {
                g1[k] = 0.0;
                g2[k] = 0.0;
                if (GRAV && ax == VA) {
                    g1[k] = a.G1[(side * B + k) * N + I];
                    g2[k] = a.G2[(side * B + k) * N + I];
                }
            }
            double pJ[B], uJ[B];
#pragma unroll
            for (int k = 0; k < B; ++k) {
                pJ[k] = a.vvP[k * N + J];
                uJ[k] = a.vvU[k * N + J];
            }
            double F0[B];
#pragma unroll
            for (int s = 0; s < NR; ++s)
#pragma unroll
                for (int k = 0; k < B; ++k) {
                    const double F = (GRAV && ax == VA)
                                         ? phaseFlux<true, FULLUP>(tij, pI[s][k], pJ[k], uI[s][k], uJ[k], g1[k], g2[k], w)
                                         : phaseFlux<false, FULLUP>(tij, pI[s][k], pJ[k], uI[s][k], uJ[k], 0.0, 0.0, w);
                    if (s == 0) F0[k] = F;
                    r[s][k] += F;
                }
            const bool jacJ = !(a.color && !a.color[J]);
            if (ANALYTIC && WANT_JAC) {
                // addFluxDerivatives (1p: incompressiblelocalresidual.hh:117-123;
                // 2p: incompressiblelocalresidual.hh:169-252)
                double blk[BB];
                if constexpr (B == 1) {
                    const double deriv = tij * rhoMu[0];
                    dII[0] += deriv;
                    blk[0] = 0.0 - deriv;
                } else {
                    double flux[B];
#pragma unroll
                    for (int k = 0; k < B; ++k) {
                        double fl = tij * (pI[0][k] - pJ[k]);
                        if (GRAV && ax == VA) {
                            fl = fl + g1[k];
                            fl = fl - g2[k];
                        }
                        flux[k] = fl;
                    }
                    const double dJ0 = a.dvv[J], dJ1 = a.dvv[N + J], dJ2 = a.dvv[2 * N + J];
                    const double iw_w = signbit(flux[0]) ? (1.0 - w) : w, ow_w = 1.0 - iw_w;
                    const double iw_n = signbit(flux[1]) ? (1.0 - w) : w, ow_n = 1.0 - iw_n;
                    const double up_w = uI[0][0] * iw_w + uJ[0] * ow_w;
                    const double up_n = uI[0][1] * iw_n + uJ[1] * ow_n;
                    const double rho_mu_flux_w = rhoMu[0] * flux[0];
                    const double rho_mu_flux_n = rhoMu[1] * flux[1];
                    const double tij_up_w = tij * up_w;
                    const double tij_up_n = tij * up_n;
                    double bJ[BB] = {0.0, 0.0, 0.0, 0.0};
                    dII[0] += tij_up_w;
                    bJ[0] -= tij_up_w;
                    dII[1] += rho_mu_flux_w * dI[0] * iw_w;
                    bJ[1] += rho_mu_flux_w * dJ0 * ow_w;
                    dII[2] += tij_up_n;
                    bJ[2] -= tij_up_n;
                    dII[3] += rho_mu_flux_n * dI[1] * iw_n;
                    bJ[3] += rho_mu_flux_n * dJ1 * ow_n;
                    dII[3] += tij_up_n * dI[2];
                    bJ[3] -= tij_up_n * dJ2;
#pragma unroll
                    for (int e = 0; e < BB; ++e) blk[e] = bJ[e];
                }
                double* dst = a.A + ((int64_t)slot * N + I) * BB;
#pragma unroll
                for (int e = 0; e < BB; ++e) dst[e] = blk[e];
            } else if (WANT_JAC && jacJ) {
                double blk[BB];
#pragma unroll
                for (int pv = 0; pv < B; ++pv) {
                    const double epsJ = a.eps[pv * N + J];
                    double Fs[SP > 0 ? SP : 1][B];
#pragma unroll
                    for (int t = 0; t < SP; ++t) {
                        const int sJ = 1 + SP * pv + t;
                        double pJs[B], uJs[B];
#pragma unroll
                        for (int k = 0; k < B; ++k) {
                            pJs[k] = a.vvP[(sJ * B + k) * N + J];
                            uJs[k] = a.vvU[(sJ * B + k) * N + J];
                        }
#pragma unroll
                        for (int k = 0; k < B; ++k) {
                            const double F = (GRAV && ax == VA)
                                ? phaseFlux<true, FULLUP>(tij, pI[0][k], pJs[k], uI[0][k], uJs[k], g1[k], g2[k], w)
                                : phaseFlux<false, FULLUP>(tij, pI[0][k], pJs[k], uI[0][k], uJs[k], 0.0, 0.0, w);
                            Fs[t][k] = F;
                        }
                    }
#pragma unroll
                    for (int e = 0; e < B; ++e) {
                        double d;
                        if (METHOD == 1) d = (Fs[0][e] - F0[e]) / epsJ;
                        else if (METHOD == -1) d = (F0[e] - Fs[0][e]) / epsJ;
                        else if (METHOD == 0) d = (Fs[0][e] - Fs[1][e]) / (epsJ + epsJ);
                        else d = fivePoint(Fs[0][e], Fs[1][e], Fs[2][e], Fs[3][e], epsJ);
                        blk[e * B + pv] = d;
                    }
                }
                double* dst = a.A + ((int64_t)slot * N + I) * BB;
#pragma unroll
                for (int e = 0; e < BB; ++e) dst[e] = blk[e];
            }
        } else {
            // boundary face: index among the faces of this side
            int64_t pos;
            if (ax == 0) pos = iy + (int64_t)ny * iz;
            else if (ax == 1) pos = ix + (int64_t)nx * iz;
            else pos = ix + (int64_t)nx * iy;
            const int64_t bidx = pc.sideOffset[f] + pos;
            const int8_t type = a.btype[bidx];
            if (type == 1) {
                const double tij = a.bTij[bidx];
                double flux[B], gU[B];
#pragma unroll
                for (int k = 0; k < B; ++k) {
                    const double gp = a.bP[k * a.nb + bidx];
                    const double gu = a.bU[k * a.nb + bidx];
                    const double g1 = a.bG1[k * a.nb + bidx];
                    gU[k] = gu;
                    double fl = tij * (pI[0][k] - gp);
                    if (GRAV && ax == VA) {
                        fl = fl + g1;
                        fl = fl - 0.0;
                    }
                    flux[k] = fl;
#pragma unroll
                    for (int s = 0; s < NR; ++s) {
                        const double F = (GRAV && ax == VA)
                                             ? phaseFlux<true, FULLUP>(tij, pI[s][k], gp, uI[s][k], gu, g1, 0.0, w)
                                             : phaseFlux<false, FULLUP>(tij, pI[s][k], gp, uI[s][k], gu, 0.0, 0.0, w);
                        r[s][k] += F;
                    }
                }
                if (ANALYTIC && WANT_JAC) {
                    // addCCDirichletFluxDerivatives (1p: incompressiblelocalresidual.hh:212-219;
                    // 2p: incompressiblelocalresidual.hh:427-484)
                    if constexpr (B == 1) {
                        dII[0] += tij * rhoMu[0];
                    } else {
                        const double iw_w = signbit(flux[0]) ? (1.0 - w) : w, ow_w = 1.0 - iw_w;
                        const double iw_n = signbit(flux[1]) ? (1.0 - w) : w, ow_n = 1.0 - iw_n;
                        const double up_w = uI[0][0] * iw_w + gU[0] * ow_w;
                        dII[0] += tij * up_w;
                        dII[1] += rhoMu[0] * flux[0] * dI[0] * iw_w;
                        const double up_n = uI[0][1] * iw_n + gU[1] * ow_n;
                        dII[2] += tij * up_n;
                        dII[3] += rhoMu[1] * flux[1] * dI[1] * iw_n;
                        dII[3] += tij * dI[2] * up_n;
                    }
                }
            } else {
#pragma unroll
                for (int e = 0; e < B; ++e) {
                    const double q = a.bNeu[e * a.nb + bidx];
#pragma unroll
                    for (int s = 0; s < NR; ++s) r[s][e] += q;
                }
            }
            if (WANT_JAC) {
                double* dst = a.A + ((int64_t)slot * N + I) * BB;
#pragma unroll
                for (int e = 0; e < BB; ++e) dst[e] = 0.0;
            }
        }
    }

    if (TRANSIENT) {
        const double V = a.vol[I];
#pragma unroll
        for (int k = 0; k < B; ++k) {
            const double sp = a.stPrev[k * N + I];
#pragma unroll
            for (int s = 0; s < NR; ++s) {
                double st = a.vvS[(s * B + k) * N + I];
                st -= sp;
                st *= V;
                st /= a.dt;
                r[s][k] += st;
            }
        }
    }

#pragma unroll
    for (int e = 0; e < B; ++e) a.r[I * B + e] = r[0][e];

    if (ANALYTIC && WANT_JAC) {
        double* dst = a.A + ((int64_t)DIM * N + I) * BB;
#pragma unroll
        for (int e = 0; e < BB; ++e) dst[e] = dII[e];
    } else if (WANT_JAC && jacI) {
        double blk[BB];
#pragma unroll
        for (int pv = 0; pv < B; ++pv) {
            const double epsI = a.eps[pv * N + I];
#pragma unroll
            for (int e = 0; e < B; ++e) {
                double d;
                if (METHOD == 1) d = (r[1 + pv][e] - r[0][e]) / epsI;
                else if (METHOD == -1) d = (r[0][e] - r[1 + pv][e]) / epsI;
                else if (METHOD == 0) d = (r[1 + 2 * pv][e] - r[2 + 2 * pv][e]) / (epsI + epsI);
                else d = fivePoint(r[1 + 4 * pv][e], r[2 + 4 * pv][e], r[3 + 4 * pv][e], r[4 + 4 * pv][e], epsI);
                blk[e * B + pv] = d;
            }
        }
        double* dst = a.A + ((int64_t)DIM * N + I) * BB;
#pragma unroll
        for (int e = 0; e < BB; ++e) dst[e] = blk[e];
    }
}

template <int B, int DIM, int METHOD, bool GRAV, bool TRANSIENT, bool FULLUP, bool WANT_JAC>
__global__ void __launch_bounds__(128) rowKernel(AssemblyArgs a0, const AssemblyArgs* __restrict__ batch)
{
    const AssemblyArgs a = batch ? batch[blockIdx.y] : a0;
    for (int64_t I = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; I < a.N; I += (int64_t)gridDim.x * blockDim.x)
        rowCell<B, DIM, METHOD, GRAV, TRANSIENT, FULLUP, WANT_JAC>(a, I);
}

// ---------------------------------------------------------------- host launchers
static int blocksFor(int64_t n, int t) { return (int)((n + t - 1) / t); }

// launch geometry: single problem -> one thread per cell; batch -> blockIdx.y selects
// the problem, grid-stride loops cover problems of different sizes
struct Geo {
    dim3 grid;
    const AssemblyArgs* batch;
};
static Geo geo(int64_t n, int count, const AssemblyArgs* batch)
{
    if (!batch) return {dim3(blocksFor(n, 128)), nullptr};
    const int gx = std::max(1, std::min(blocksFor(n, 128), 1184));
    return {dim3(gx, count), batch};
}

template <int B, int METHOD>
static void volvarsT(const AssemblyArgs& a, const Geo& g, cudaStream_t st)
{
    volvarsKernel<B, METHOD><<<g.grid, 128, 0, st>>>(a, g.batch);
}

static void volvarsDispatch(const AssemblyArgs& a, const Geo& g, int b, int method, cudaStream_t st)
{
    if (b == 1) {
        if (method == 2) volvarsT<1, 2>(a, g, st);
        else if (method == 3) volvarsT<1, 3>(a, g, st);
        else if (method == 1) volvarsT<1, 1>(a, g, st);
        else if (method == -1) volvarsT<1, -1>(a, g, st);
        else if (method == 5) volvarsT<1, 5>(a, g, st);
        else volvarsT<1, 0>(a, g, st);
    } else {
        if (method == 2) volvarsT<2, 2>(a, g, st);
        else if (method == 3) volvarsT<2, 3>(a, g, st);
        else if (method == 1) volvarsT<2, 1>(a, g, st);
        else if (method == -1) volvarsT<2, -1>(a, g, st);
        else if (method == 5) volvarsT<2, 5>(a, g, st);
        else volvarsT<2, 0>(a, g, st);
    }
    DXG_CUDA(cudaGetLastError());
}

void launchVolvars(const AssemblyArgs& a, int b, int method, const double* u, cudaStream_t st)
{
    AssemblyArgs aa = a;
    aa.u = u;
    volvarsDispatch(aa, geo(a.N, 1, nullptr), b, method, st);
}
void launchVolvarsBatch(const AssemblyArgs* batch, int count, int64_t maxN, int b, int method, cudaStream_t st)
{
    volvarsDispatch(AssemblyArgs{}, geo(maxN, count, batch), b, method, st);
}

static void prevDispatch(const AssemblyArgs& a, const Geo& g, int b, cudaStream_t st)
{
    if (b == 1) prevStorageKernel<1><<<g.grid, 128, 0, st>>>(a, g.batch);
    else prevStorageKernel<2><<<g.grid, 128, 0, st>>>(a, g.batch);
    DXG_CUDA(cudaGetLastError());
}
void launchPrevStorage(const AssemblyArgs& a, int b, const double* uprev, cudaStream_t st)
{
    AssemblyArgs aa = a;
    aa.uprev = uprev;
    prevDispatch(aa, geo(a.N, 1, nullptr), b, st);
}
void launchPrevStorageBatch(const AssemblyArgs* batch, int count, int64_t maxN, int b, cudaStream_t st)
{
    prevDispatch(AssemblyArgs{}, geo(maxN, count, batch), b, st);
}

template <int B, int DIM, int METHOD, bool GRAV, bool TRANSIENT, bool FULLUP>
static void launchRow3(const AssemblyArgs& a, const Geo& g, bool jac, cudaStream_t st)
{
    if (jac) rowKernel<B, DIM, METHOD, GRAV, TRANSIENT, FULLUP, true><<<g.grid, 128, 0, st>>>(a, g.batch);
    else rowKernel<B, DIM, METHOD, GRAV, TRANSIENT, FULLUP, false><<<g.grid, 128, 0, st>>>(a, g.batch);
}
template <int B, int DIM, int METHOD>
static void launchRow2(const AssemblyArgs& a, const Geo& g, bool jac, bool grav, bool transient, bool fullup,
                       cudaStream_t st)
{
    if (fullup) {
        if (grav) {
            if (transient) launchRow3<B, DIM, METHOD, true, true, true>(a, g, jac, st);
            else launchRow3<B, DIM, METHOD, true, false, true>(a, g, jac, st);
        } else {
            if (transient) launchRow3<B, DIM, METHOD, false, true, true>(a, g, jac, st);
            else launchRow3<B, DIM, METHOD, false, false, true>(a, g, jac, st);
        }
    } else {
        if (grav) {
            if (transient) launchRow3<B, DIM, METHOD, true, true, false>(a, g, jac, st);
            else launchRow3<B, DIM, METHOD, true, false, false>(a, g, jac, st);
        } else {
            if (transient) launchRow3<B, DIM, METHOD, false, true, false>(a, g, jac, st);
            else launchRow3<B, DIM, METHOD, false, false, false>(a, g, jac, st);
        }
    }
}
template <int B, int DIM>
static void launchRow1(const AssemblyArgs& a, const Geo& g, int method, bool jac, bool grav, bool transient,
                       bool fullup, cudaStream_t st)
{
    if (method == 1) launchRow2<B, DIM, 1>(a, g, jac, grav, transient, fullup, st);
    else if (method == 3) launchRow2<B, DIM, 3>(a, g, jac, grav, transient, fullup, st);
    else if (method == -1) launchRow2<B, DIM, -1>(a, g, jac, grav, transient, fullup, st);
    else if (method == 5) launchRow2<B, DIM, 5>(a, g, jac, grav, transient, fullup, st);
    else launchRow2<B, DIM, 0>(a, g, jac, grav, transient, fullup, st);
}
static void rowDispatch(const AssemblyArgs& a, const Geo& g, int b, int dim, int method, bool jac, bool grav,
                        bool transient, bool fullup, cudaStream_t st)
{
    if (b == 1) {
        if (dim == 2) launchRow1<1, 2>(a, g, method, jac, grav, transient, fullup, st);
        else launchRow1<1, 3>(a, g, method, jac, grav, transient, fullup, st);
    } else {
        if (dim == 2) launchRow1<2, 2>(a, g, method, jac, grav, transient, fullup, st);
        else launchRow1<2, 3>(a, g, method, jac, grav, transient, fullup, st);
    }
    DXG_CUDA(cudaGetLastError());
}

void launchRow(const AssemblyArgs& a, int b, int dim, int method, bool jac, bool grav, bool transient, bool fullup,
               cudaStream_t st)
{
    rowDispatch(a, geo(a.N, 1, nullptr), b, dim, method, jac, grav, transient, fullup, st);
}
void launchRowBatch(const AssemblyArgs* batch, int count, int64_t maxN, int b, int dim, int method, bool jac, bool grav,
                    bool transient, bool fullup, cudaStream_t st)
{
    rowDispatch(AssemblyArgs{}, geo(maxN, count, batch), b, dim, method, jac, grav, transient, fullup, st);
}

}  // namespace dxg

// ---------------------------------------------------------------- device pow check
namespace dxg {
__global__ void powKernel(const double* x, const double* y, double* out, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = crPow(x[i], y[i]);
}

int runDevicePow(const double* x, const double* y, double* out, int64_t n)
{
    if (n == 0) return DXG_OK;
    double* d = nullptr;
    const size_t bytes = (size_t)n * sizeof(double);
    if (cudaMalloc(&d, 3 * bytes) != cudaSuccess) {
        cudaGetLastError();
        return DXG_ERR_OOM;
    }
    int rc = DXG_OK;
    if (cudaMemcpy(d, x, bytes, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(d + n, y, bytes, cudaMemcpyHostToDevice) != cudaSuccess)
        rc = DXG_ERR_CUDA;
    if (rc == DXG_OK) {
        const int64_t blocks = std::min<int64_t>((n + 255) / 256, 152 * 16);
        powKernel<<<(unsigned)blocks, 256>>>(d, d + n, d + 2 * n, n);
        if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) rc = DXG_ERR_CUDA;
    }
    if (rc == DXG_OK && cudaMemcpy(out, d + 2 * n, bytes, cudaMemcpyDeviceToHost) != cudaSuccess) rc = DXG_ERR_CUDA;
    cudaFree(d);
    return rc;
}
}  // namespace dxg

// ---------------------------------------------------------------- FP64 FMA rate
namespace dxg {
// Eight independent FMA chains per thread; the result is written so nothing is elided.
__global__ void fmaRateKernel(double* out, int iters, double a, double c)
{
    double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; ++i) {
        x0 = fma(x0, a, c); x1 = fma(x1, a, c); x2 = fma(x2, a, c); x3 = fma(x3, a, c);
        x4 = fma(x4, a, c); x5 = fma(x5, a, c); x6 = fma(x6, a, c); x7 = fma(x7, a, c);
    }
    out[blockIdx.x * (int64_t)blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

int runFp64Rate(double* tflops)
{
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return DXG_ERR_CUDA;
    const int threads = 256, iters = 2048;
    double* d = nullptr;
    if (cudaMalloc(&d, (size_t)sms * threads * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        return DXG_ERR_OOM;
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = DXG_OK;
    float ms = 0.f;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) rc = DXG_ERR_CUDA;
    if (rc == DXG_OK) {
        fmaRateKernel<<<sms, threads>>>(d, iters, 1.0000001, 1e-9);   // warm-up
        cudaEventRecord(e0);
        fmaRateKernel<<<sms, threads>>>(d, iters, 1.0000001, 1e-9);
        cudaEventRecord(e1);
        if (cudaGetLastError() != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
            cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess || ms <= 0.f)
            rc = DXG_ERR_CUDA;
    }
    if (rc == DXG_OK) *tflops = 2.0 * 8.0 * iters * (double)sms * threads / (ms * 1e-3) / 1e12;
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(d);
    return rc;
}
}  // namespace dxg
