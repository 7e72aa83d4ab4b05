// mpfa.cu -- cell-centred MPFA-O for the 1p model on tensor-product grids.
//
// The O-method of dumux/discretization/cellcentered/mpfa/omethod with continuity points at
// the face centres (MPFA.Q = 0, fvgridgeometry.hh:326, helper.hh:518-528):
//   * every cell face is split into 2^(dim-1) sub control volume faces (scvfs), one per face
//     corner; the scvfs around a grid vertex form its interaction volume (IV);
//   * in each IV cell the pressure gradient is reconstructed from the cell pressure and the
//     (unknown) pressures at the face centres of its dim IV faces, through the dual basis of
//     the vectors from the cell centre to those face centres (localsubcontrolentities.hh:
//     43-83, helper.hh:58-85 / 275-299); the flux of a face seen from cell P is
//     sum_d w_d (p_P - u_d) with w_d = n^T K nu_d * area * extrusion / detX
//     (computetransmissibility.hh:32-50);
//   * flux continuity on the IV's interior faces and zero flux on its Neumann faces give the
//     local system A u = B p; the face fluxes are f = C u + D p, so T = D + C A^-1 B
//     (omethod/localassembler.hh:60-330, localassemblerhelper.hh:70-80);
//   * gravity adds per face alpha rho area with alpha = extrusion * n^T K g, and the
//     continuity defect of the neighbours' alphas through C A^-1
//     (localassemblerbase.hh:125-222);
//   * the advective flux of the 1p model is (T p + g) * rho / mu (flux/ccmpfa/darcyslaw.hh:
//     150-205 with the upwinded density * mobility of the constant liquid).
// The transmissibilities of the incompressible 1p model depend on geometry and
// permeability only, so the IVs are built and solved once at upload (host, all threads)
// and every (cell, scvf) keeps its flux row over the IV's cells, signed for that cell, and
// a constant (the IV's Dirichlet values times their transmissibilities, plus gravity).
//
// On the device one thread per cell evaluates its residual -source*V + sum of its scvf
// fluxes (in the element's scvf order: faces -x,+x,-y,+y,-z,+z, corners of each face in
// reference-element order) and the numeric-difference Jacobian row over the 3^dim
// neighbourhood in the order of CCLocalAssembler<numeric> (cclocalassembler.hh:164-348):
// the diagonal from the cell's whole residual, the entry of neighbour j from the sum of the
// cell's scvf fluxes whose IV contains j, each at the perturbed and unperturbed state.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <exception>
#include <thread>
#include <vector>

#include "common.cuh"
#include "context.h"
#include "kernels.cuh"
#include "linalg_kernels.cuh"
#include "mpfa.cuh"

namespace dxg {

// ---------------------------------------------------------------- host: interaction volumes
namespace {

struct MpGrid {
    int dim = 2;
    int64_t n[3] = {1, 1, 1};
    const double* x[3] = {nullptr, nullptr, nullptr};
    int64_t stride[3] = {1, 1, 1};
    double center(int a, int64_t i) const { return 0.5 * (x[a][i] + x[a][i + 1]); }
    double width(int a, int64_t i) const { return x[a][i + 1] - x[a][i]; }
};

// One IV face: the sub-faces of the one or two cells meeting at a grid vertex across one
// cell face.  P is the first existing cell of the pair (lower along the axis), Q the other.
struct IvFace {
    int axis = 0;
    int P = -1, Q = -1;          // IV cell positions
    bool boundary = false, dirichlet = false;
    int64_t bidx = -1;
    double uD = 0.0;
    double n[3] = {0, 0, 0};
    double area = 0.0;
    int dof = -1, dIdx = -1;     // local unknown / Dirichlet known index
};

// body(i0, i1) over [0, n) on up to 16 host threads; the first exception is rethrown
template <class Fn>
void mpParallel(int64_t n, Fn&& body)
{
    const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
    const int nt = (int)std::min<int64_t>({(int64_t)std::min(hw, 16), (n + 4095) / 4096, (int64_t)16});
    if (nt <= 1) {
        body((int64_t)0, n);
        return;
    }
    std::vector<std::thread> th;
    std::vector<std::exception_ptr> err(nt);
    const int64_t chunk = (n + nt - 1) / nt;
    for (int t = 0; t < nt; ++t)
        th.emplace_back([&, t] {
            try {
                body(std::min(n, t * chunk), std::min(n, (t + 1) * chunk));
            } catch (...) {
                err[t] = std::current_exception();
            }
        });
    for (auto& x : th) x.join();
    for (auto& e : err)
        if (e) std::rethrow_exception(e);
}

double tripleProduct(const double* a, const double* b, const double* c)
{
    const double cx = b[1] * c[2] - b[2] * c[1], cy = b[2] * c[0] - b[0] * c[2], cz = b[0] * c[1] - b[1] * c[0];
    return a[0] * cx + a[1] * cy + a[2] * cz;
}
void cross(const double* a, const double* b, double* o)
{
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

// n^T K v as v1 * (K v2) (common/math.hh:880-885), K the cell's tensor or k * (n.v) for a
// scalar permeability (math.hh:906-913)
double vtmv(int dim, const double* n, const double* Kt, double Ks, const double* v)
{
    if (!Kt) {
        double d = 0.0;
        for (int i = 0; i < dim; ++i) d += n[i] * v[i];
        return Ks * d;
    }
    double mv[3] = {0, 0, 0};
    for (int i = 0; i < dim; ++i) {
        double s = 0.0;
        for (int j = 0; j < dim; ++j) s += Kt[i * dim + j] * v[j];
        mv[i] = s;
    }
    double d = 0.0;
    for (int i = 0; i < dim; ++i) d += n[i] * mv[i];
    return d;
}

// Gauss-Jordan inverse with partial pivoting, in place (n x n row-major); false if singular
bool invert(std::vector<double>& A, int n)
{
    std::vector<double> I((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) I[(size_t)i * n + i] = 1.0;
    for (int c = 0; c < n; ++c) {
        int p = c;
        for (int r = c + 1; r < n; ++r)
            if (std::fabs(A[(size_t)r * n + c]) > std::fabs(A[(size_t)p * n + c])) p = r;
        if (A[(size_t)p * n + c] == 0.0) return false;
        if (p != c)
            for (int k = 0; k < n; ++k) {
                std::swap(A[(size_t)p * n + k], A[(size_t)c * n + k]);
                std::swap(I[(size_t)p * n + k], I[(size_t)c * n + k]);
            }
        const double inv = 1.0 / A[(size_t)c * n + c];
        for (int k = 0; k < n; ++k) {
            A[(size_t)c * n + k] *= inv;
            I[(size_t)c * n + k] *= inv;
        }
        for (int r = 0; r < n; ++r) {
            if (r == c) continue;
            const double f = A[(size_t)r * n + c];
            if (f == 0.0) continue;
            for (int k = 0; k < n; ++k) {
                A[(size_t)r * n + k] -= f * A[(size_t)c * n + k];
                I[(size_t)r * n + k] -= f * I[(size_t)c * n + k];
            }
        }
    }
    A.swap(I);
    return true;
}

}  // namespace

MpfaLayout mpfaLayout(int dim)
{
    MpfaLayout L{};
    L.dim = dim;
    L.S = dim == 2 ? 9 : 27;
    L.center = (L.S - 1) / 2;
    L.K = 1 << dim;
    const int corners = 1 << (dim - 1);
    L.F = 2 * dim * corners;
    for (int f = 0; f < L.F; ++f) {
        const int face = f / corners, c = f % corners;
        const int a = face / 2, side = face % 2;
        // vertex of the scvf relative to the cell: along the face axis the face's side, along
        // the other axes (increasing) the corner's bits
        int vrel[3] = {0, 0, 0};
        vrel[a] = side;
        int bit = 0;
        for (int d = 0; d < dim; ++d)
            if (d != a) vrel[d] = (c >> bit++) & 1;
        uint32_t slots = 0;
        for (int k = 0; k < L.K; ++k) {
            // IV cell k at the vertex: cell = vertex - 1 + beta (beta = bits of k)
            int s = 0, mul = 1;
            for (int d = 0; d < dim; ++d) {
                const int o = vrel[d] - 1 + ((k >> d) & 1);   // offset from the cell, -1..1
                s += (o + 1) * mul;
                mul *= 3;
            }
            L.slotOf[f][k] = (int8_t)s;
            slots |= 1u << s;
        }
        L.scvfSlots[f] = slots;
    }
    return L;
}

void mpfaTriples(int dim, int& n, int8_t (*tri)[3])
{
    const int S = dim == 2 ? 9 : 27, center = (S - 1) / 2;
    auto offOf = [&](int s, int* o) {
        for (int d = 0; d < 3; ++d) {
            o[d] = d < dim ? s % 3 - 1 : 0;
            s /= 3;
        }
    };
    n = 0;
    for (int s = 0; s < center; ++s)
        for (int t = s + 1; t < S; ++t) {
            int os[3], ot[3];
            offOf(s, os);
            offOf(t, ot);
            int u = 0, mul = 1;
            bool ok = true;
            for (int d = 0; d < dim; ++d) {
                const int dd = ot[d] - os[d];
                if (dd < -1 || dd > 1) ok = false;
                u += (dd + 1) * mul;
                mul *= 3;
            }
            if (!ok || u <= center) continue;
            tri[n][0] = (int8_t)s;
            tri[n][1] = (int8_t)t;
            tri[n][2] = (int8_t)u;
            ++n;
        }
}

void mpfaTabulate(const dxg_problem_desc* d, const MpfaLayout& L, const int64_t* sideOffset, const double* dirP,
                  std::vector<double>& coef, std::vector<double>& cst, std::vector<int8_t>& kind)
{
    const int b = d->num_eq;
    const int64_t nb = sideOffset[2 * d->dim];
    const int dim = d->dim;
    MpGrid g;
    g.dim = dim;
    for (int a = 0; a < dim; ++a) {
        g.n[a] = d->cells[a];
        g.x[a] = d->coords[a];
    }
    g.stride[1] = g.n[0];
    g.stride[2] = g.n[0] * g.n[1];
    const int64_t N = g.n[0] * g.n[1] * g.n[2];
    const int K = L.K, F = L.F, corners = 1 << (dim - 1);
    coef.assign((size_t)F * K * N, 0.0);
    cst.assign((size_t)F * b * N, 0.0);
    kind.assign((size_t)F * N, 0);
    const bool grav = d->enable_gravity != 0;
    double gvec[3] = {0, 0, 0};
    if (grav)
        for (int a = 0; a < dim; ++a) gvec[a] = d->gravity[a];
    auto Kt = [&](int64_t i) -> const double* {
        return d->permeability_tensor ? d->permeability_tensor + (size_t)i * dim * dim : nullptr;
    };
    auto EX = [&](int64_t i) { return d->extrusion ? d->extrusion[i] : 1.0; };
    // Neumann scvfs: the given flux times the scvf area and the extrusion (cclocalresidual.hh:89-97)
    mpParallel(N, [&](int64_t i0, int64_t i1) {
        for (int64_t i = i0; i < i1; ++i) {
            int64_t id[3] = {i % g.n[0], (i / g.n[0]) % g.n[1], i / (g.n[0] * g.n[1])};
            for (int face = 0; face < 2 * dim; ++face) {
                const int a = face / 2, side = face % 2;
                const bool bnd = side == 0 ? id[a] == 0 : id[a] == g.n[a] - 1;
                if (!bnd) continue;
                int64_t pos = 0, mul = 1;
                for (int k = 0; k < dim; ++k)
                    if (k != a) {
                        pos += id[k] * mul;
                        mul *= g.n[k];
                    }
                const int64_t bidx = sideOffset[face] + pos;
                if (d->bc_type[bidx] != 2) continue;
                double area = 1.0;
                for (int k = 0; k < dim; ++k)
                    if (k != a) area *= 0.5 * g.width(k, id[k]);
                const double s = area * EX(i);
                for (int c = 0; c < corners; ++c) {
                    const int f = face * corners + c;
                    kind[(size_t)f * N + i] = 1;
                    for (int e = 0; e < b; ++e) {
                        double q = 0.0;
                        q += d->bc_values[bidx * b + e] * s;
                        cst[((size_t)f * b + e) * N + i] = q;
                    }
                }
            }
        }
    });

    const int64_t nv[3] = {g.n[0] + 1, g.n[1] + 1, dim == 3 ? g.n[2] + 1 : 1};
    const int64_t NV = nv[0] * nv[1] * nv[2];
    mpParallel(NV, [&](int64_t v0, int64_t v1) {
        for (int64_t vi = v0; vi < v1; ++vi) {
            const int64_t v[3] = {vi % nv[0], (vi / nv[0]) % nv[1], vi / (nv[0] * nv[1])};
            // IV cells
            int64_t cell[8];
            int64_t cid[8][3];
            int known[8];
            int nKnown = 0;
            for (int k = 0; k < K; ++k) {
                bool ok = true;
                for (int a = 0; a < 3; ++a) {
                    cid[k][a] = a < dim ? v[a] - 1 + ((k >> a) & 1) : 0;
                    if (a < dim && (cid[k][a] < 0 || cid[k][a] >= g.n[a])) ok = false;
                }
                cell[k] = ok ? cid[k][0] + g.stride[1] * cid[k][1] + g.stride[2] * cid[k][2] : -1;
                known[k] = ok ? nKnown++ : -1;
            }
            // IV faces: axis a, other-axis bits gamma (lower axis fastest)
            const int nF = dim * corners;
            IvFace faces[12];
            int nU = 0;
            for (int a = 0; a < dim; ++a)
                for (int gm = 0; gm < corners; ++gm) {
                    IvFace& fc = faces[a * corners + gm];
                    fc.axis = a;
                    int lower = 0, bit = 0;
                    for (int dd = 0; dd < dim; ++dd)
                        if (dd != a) lower |= ((gm >> bit++) & 1) << dd;
                    const int upper = lower | (1 << a);
                    const bool hasL = cell[lower] >= 0, hasU = cell[upper] >= 0;
                    if (!hasL && !hasU) {
                        fc.P = -1;
                        continue;
                    }
                    fc.P = hasL ? lower : upper;
                    fc.Q = (hasL && hasU) ? upper : -1;
                    fc.boundary = !(hasL && hasU);
                    fc.n[a] = hasL ? 1.0 : -1.0;
                    const int64_t* pid = cid[fc.P];
                    fc.area = 1.0;
                    for (int k = 0; k < dim; ++k)
                        if (k != a) fc.area *= 0.5 * g.width(k, pid[k]);
                    if (fc.boundary) {
                        const int face = 2 * a + (hasL ? 1 : 0);
                        int64_t pos = 0, mul = 1;
                        for (int k = 0; k < dim; ++k)
                            if (k != a) {
                                pos += pid[k] * mul;
                                mul *= g.n[k];
                            }
                        fc.bidx = sideOffset[face] + pos;
                        fc.dirichlet = d->bc_type[fc.bidx] == 1;
                        fc.uD = d->bc_values[fc.bidx * b];
                    }
                }
            int nD = 0;
            for (int f = 0; f < nF; ++f) {
                if (faces[f].P < 0) continue;
                if (faces[f].dirichlet) faces[f].dIdx = nKnown + nD++;
                else faces[f].dof = nU++;
            }
            const int nK = nKnown + nD;
            // local scvs: for each existing cell its IV face along every axis, the dual basis
            // of the centre-to-face-centre vectors and its determinant
            int localFace[8][3];
            double nu[8][3][3];
            double detX[8];
            for (int k = 0; k < K; ++k) {
                if (cell[k] < 0) continue;
                double e[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
                for (int dd = 0; dd < dim; ++dd) {
                    int gm = 0, bit = 0;
                    for (int o = 0; o < dim; ++o)
                        if (o != dd) gm |= ((k >> o) & 1) << bit++;
                    localFace[k][dd] = dd * corners + gm;
                    // face centre minus cell centre: along dd the vertex plane, else zero
                    e[dd][dd] = g.x[dd][v[dd]] - g.center(dd, cid[k][dd]);
                }
                if (dim == 2) {
                    // rotation R = [[0,1],[-1,0]] of the other basis vector, sign by orientation
                    double n0[3] = {e[1][1], -e[1][0], 0}, n1[3] = {e[0][1], -e[0][0], 0};
                    const double cr = e[0][0] * e[1][1] - e[0][1] * e[1][0];
                    if (std::signbit(cr)) for (double& z : n0) z *= -1.0;
                    else for (double& z : n1) z *= -1.0;
                    for (int q = 0; q < 3; ++q) {
                        nu[k][0][q] = n0[q];
                        nu[k][1][q] = n1[q];
                    }
                    detX[k] = std::fabs(cr);
                } else {
                    cross(e[1], e[2], nu[k][0]);
                    cross(e[2], e[0], nu[k][1]);
                    cross(e[0], e[1], nu[k][2]);
                    const double tp = tripleProduct(e[0], e[1], e[2]);
                    if (std::signbit(tp))
                        for (int q = 0; q < 3; ++q)
                            for (int r = 0; r < 3; ++r) nu[k][q][r] *= -1.0;
                    detX[k] = std::fabs(tp);
                }
            }
            auto omega = [&](int k, const IvFace& fc, double* w) {
                const int64_t i = cell[k];
                const double ae = fc.area * EX(i);
                for (int dd = 0; dd < dim; ++dd) {
                    double t = vtmv(dim, fc.n, Kt(i), d->permeability[i], nu[k][dd]);
                    t *= ae;
                    t /= detX[k];
                    w[dd] = t;
                }
            };
            std::vector<double> A((size_t)nU * nU, 0.0), B((size_t)nU * nK, 0.0), C((size_t)nF * nU, 0.0),
                D((size_t)nF * nK, 0.0);
            for (int f = 0; f < nF; ++f) {
                const IvFace& fc = faces[f];
                if (fc.P < 0) continue;
                double wp[3];
                omega(fc.P, fc, wp);
                const bool cur = fc.dirichlet;
                for (int dd = 0; dd < dim; ++dd) {
                    const IvFace& o = faces[localFace[fc.P][dd]];
                    if (!o.dirichlet) {
                        C[(size_t)f * nU + o.dof] -= wp[dd];
                        if (!cur) A[(size_t)fc.dof * nU + o.dof] -= wp[dd];
                    } else {
                        D[(size_t)f * nK + o.dIdx] -= wp[dd];
                        if (!cur) B[(size_t)fc.dof * nK + o.dIdx] += wp[dd];
                    }
                    D[(size_t)f * nK + known[fc.P]] += wp[dd];
                    if (!cur) B[(size_t)fc.dof * nK + known[fc.P]] -= wp[dd];
                }
                if (!fc.boundary) {
                    double wq[3];
                    omega(fc.Q, fc, wq);
                    for (int dd = 0; dd < dim; ++dd) {
                        const IvFace& o = faces[localFace[fc.Q][dd]];
                        if (!o.dirichlet) A[(size_t)fc.dof * nU + o.dof] += wq[dd];
                        else B[(size_t)fc.dof * nK + o.dIdx] -= wq[dd];
                        B[(size_t)fc.dof * nK + known[fc.Q]] += wq[dd];
                    }
                }
            }
            // T = D + (C A^-1) B
            std::vector<double> T = D, CA;
            if (nU > 0) {
                if (!invert(A, nU)) throw Error(DXG_ERR_ARG, "singular MPFA interaction-volume system");
                CA.assign((size_t)nF * nU, 0.0);
                for (int f = 0; f < nF; ++f)
                    for (int c = 0; c < nU; ++c) {
                        double s = 0.0;
                        for (int k = 0; k < nU; ++k) s += C[(size_t)f * nU + k] * A[(size_t)k * nU + c];
                        CA[(size_t)f * nU + c] = s;
                    }
                for (int f = 0; f < nF; ++f)
                    for (int j = 0; j < nK; ++j) {
                        double s = 0.0;
                        for (int k = 0; k < nU; ++k) s += CA[(size_t)f * nU + k] * B[(size_t)k * nK + j];
                        T[(size_t)f * nK + j] += s;
                    }
            }
            // gravity per phase and face, then the continuity defect of the neighbours' alphas
            double gF[2][12] = {};
            for (int ph = 0; ph < b && grav; ++ph) {
                const double rho = d->density[ph];
                std::vector<double> deltaG((size_t)nU, 0.0);
                for (int f = 0; f < nF; ++f) {
                    const IvFace& fc = faces[f];
                    if (fc.P < 0) continue;
                    const int64_t iP = cell[fc.P];
                    const double alphaIn = EX(iP) * vtmv(dim, fc.n, Kt(iP), d->permeability[iP], gvec);
                    double r = rho;
                    if (!fc.dirichlet) {
                        double dg = 0.0;
                        int nOut = 0;
                        if (!fc.boundary) {
                            const int64_t iQ = cell[fc.Q];
                            const double alphaOut = EX(iQ) * vtmv(dim, fc.n, Kt(iQ), d->permeability[iQ], gvec);
                            r += rho;
                            dg += alphaOut;
                            nOut = 1;
                        }
                        r /= nOut + 1;
                        dg -= alphaIn;
                        dg *= r * fc.area;
                        deltaG[fc.dof] = dg;
                    }
                    gF[ph][f] = alphaIn * r * fc.area;
                }
                for (int f = 0; f < nF; ++f) {
                    if (faces[f].P < 0) continue;
                    double s = gF[ph][f];
                    for (int k = 0; k < nU; ++k) s += CA[(size_t)f * nU + k] * deltaG[k];
                    gF[ph][f] = s;
                }
            }
            // scatter: each face's flux row to the scvf of P (as computed) and of Q (negated)
            for (int f = 0; f < nF; ++f) {
                const IvFace& fc = faces[f];
                if (fc.P < 0) continue;
                // per phase: the Dirichlet ghosts' phase pressures times their transmissibilities,
                // then gravity (1p: the Dirichlet values themselves)
                double c0[2] = {0.0, 0.0};
                for (int ph = 0; ph < b; ++ph) {
                    double cp = 0.0;
                    for (int j = nKnown; j < nK; ++j) {
                        const IvFace* fd = nullptr;
                        for (int q = 0; q < nF; ++q)
                            if (faces[q].P >= 0 && faces[q].dIdx == j) fd = &faces[q];
                        cp += T[(size_t)f * nK + j] * (b == 1 ? fd->uD : dirP[(size_t)ph * nb + fd->bidx]);
                    }
                    cp += gF[ph][f];
                    c0[ph] = cp;
                }
                for (int side = 0; side < 2; ++side) {
                    const int k = side == 0 ? fc.P : fc.Q;
                    if (k < 0) continue;
                    const int64_t i = cell[k];
                    // the cell's face toward the vertex along the face axis, and its corner
                    const int a = fc.axis;
                    const int faceSide = ((k >> a) & 1) ? 0 : 1;
                    int corner = 0, bit = 0;
                    for (int dd = 0; dd < dim; ++dd)
                        if (dd != a) corner |= (((k >> dd) & 1) ? 0 : 1) << bit++;
                    const int sf = (2 * a + faceSide) * corners + corner;
                    if (kind[(size_t)sf * N + i] == 1) continue;   // Neumann scvf
                    // IV cell kk of the scvf's own numbering is the same vertex's cell kk
                    for (int kk = 0; kk < K; ++kk) {
                        const double t = known[kk] >= 0 ? T[(size_t)f * nK + known[kk]] : 0.0;
                        coef[((size_t)sf * K + kk) * N + i] = side == 0 ? t : -t;
                    }
                    for (int ph = 0; ph < b; ++ph) cst[((size_t)sf * b + ph) * N + i] = side == 0 ? c0[ph] : -c0[ph];
                }
            }
        }
    });
}

// ---------------------------------------------------------------- device: assembly
namespace {

__device__ __forceinline__ double mpEps(const MpfaArgs& a, double x)
{
    return a.magnitude > 0.0 ? a.baseEps * a.magnitude : a.baseEps * (fabs(x) + 1.0);
}

// flux of scvf f of cell i with the neighbourhood pressures pn, slot sp replaced by q
__device__ __forceinline__ double scvfFlux(const MpfaArgs& a, int64_t i, int f, const double* pn, int sp, double q)
{
    const int64_t N = a.N;
    if (a.kind[(int64_t)f * N + i] == 1) return a.cst[(int64_t)f * N + i];
    double t = 0.0;
    for (int k = 0; k < a.K; ++k) {
        const int s = a.slotOf[f][k];
        const double p = s == sp ? q : pn[s];
        t += a.coef[((int64_t)f * a.K + k) * N + i] * p;
    }
    t += a.cst[(int64_t)f * N + i];
    return t * a.mob;
}

__device__ __forceinline__ double fivePointMp(double fp, double fm, double fm2, double fp2, double eps)
{
    double d = fp;
    d -= fm;
    d *= 8.0;
    d += fm2;
    d -= fp2;
    return d / (12.0 * eps);
}

template <int S, int METHOD>
__global__ void __launch_bounds__(128) mpfaAssembleKernel(MpfaArgs a, bool jac)
{
    constexpr int center = (S - 1) / 2;
    const int64_t N = a.N;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t m = a.mask[i];
        double pn[S];
#pragma unroll
        for (int s = 0; s < S; ++s) pn[s] = ((m >> s) & 1u) ? a.u[i + a.off[s]] : 0.0;
        // the whole residual with slot sp at q
        auto residual = [&](int sp, double q) {
            double r = 0.0;
            r -= a.srcterm[i];
            for (int f = 0; f < a.F; ++f) r += scvfFlux(a, i, f, pn, sp, q);
            if (a.transient) r += 0.0;   // incompressible 1p: the storage does not change
            return r;
        };
        // the fluxes of the scvfs whose IV holds slot s (Neumann scvfs have no IV flux), with
        // slot s at q
        auto partial = [&](int s, double q) {
            double r = 0.0;
            for (int f = 0; f < a.F; ++f)
                if (((a.scvfSlots[f] >> s) & 1u) && a.kind[(int64_t)f * N + i] != 1) r += scvfFlux(a, i, f, pn, s, q);
            return r;
        };
        const double r0 = residual(-1, 0.0);
        a.r[i] = r0;
        if (!jac) continue;
        if (METHOD == 3) {
            // CCLocalAssembler<analytic> with the incompressible 1p flux derivatives for MPFA
            // (porousmediumflow/1p/incompressiblelocalresidual.hh:126-160, 221-233): every
            // non-Neumann scvf adds (+/-) t_k * rho / mu to the column of its IV cell k, scvfs
            // in element order
            for (int s = 0; s < S; ++s) {
                double dv = 0.0;
                if ((m >> s) & 1u) {
                    for (int f = 0; f < a.F; ++f) {
                        if (!((a.scvfSlots[f] >> s) & 1u) || a.kind[(int64_t)f * N + i] == 1) continue;
                        for (int k = 0; k < a.K; ++k)
                            if (a.slotOf[f][k] == s) dv += a.coef[((int64_t)f * a.K + k) * N + i] * a.up;
                    }
                }
                a.A[(int64_t)s * N + i] = dv;
            }
            continue;
        }
        for (int s = 0; s < S; ++s) {
            double dv = 0.0;
            if ((m >> s) & 1u) {
                const double x = pn[s];
                const double ep = mpEps(a, x);
                auto eval = [&](double q) { return s == center ? residual(s, q) : partial(s, q); };
                const double f0 = s == center ? r0 : partial(s, x);
                if (METHOD == 1) dv = (eval(x + ep) - f0) / ep;
                else if (METHOD == -1) dv = (f0 - eval(x - ep)) / ep;
                else if (METHOD == 0) dv = (eval(x + ep) - eval(x - ep)) / (ep + ep);
                else {
                    const double fp = eval(x + ep), fm = eval(x - ep), fm2 = eval(x - 2.0 * ep),
                                 fp2 = eval(x + 2.0 * ep);
                    dv = fivePointMp(fp, fm, fm2, fp2, ep);
                }
            }
            a.A[(int64_t)s * N + i] = dv;
        }
    }
}

// The 2p immiscible model (p0s1): per scvf and phase the Darcy flux T p_alpha + c_alpha over
// the IV's cells' phase pressures, times the upwinded density * mobility of the scvf's inside
// cell and the cell across the face (or the Dirichlet ghost); source and storage as the TPFA
// rows; numeric Jacobian from the volume-variable kernel's perturbed states, the entry of
// neighbour j from the cell's scvf fluxes whose IV holds j (both phases), the diagonal from the
// whole residual.  Same operation order as the oracle.
template <int S, int DIM, int METHOD>
__global__ void __launch_bounds__(128) mpfa2pKernel(MpfaArgs a, bool jac)
{
    constexpr int center = (S - 1) / 2;
    constexpr int SP = statesPerPv(METHOD);
    const int64_t N = a.N;
    const int corners = 1 << (DIM - 1);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t m = a.mask[i];
        int64_t id[3] = {i % a.nx, (i / a.nx) % a.ny, i / ((int64_t)a.nx * a.ny)};
        double P0[S][2], U0[S][2];
#pragma unroll
        for (int s = 0; s < S; ++s)
#pragma unroll
            for (int ph = 0; ph < 2; ++ph) {
                const bool ok = (m >> s) & 1u;
                const int64_t j = i + (ok ? a.off[s] : 0);
                P0[s][ph] = ok ? a.vvP[(int64_t)ph * N + j] : 0.0;
                U0[s][ph] = ok ? a.vvU[(int64_t)ph * N + j] : 0.0;
            }
        // phase pressure / upwind term of the cell at slot s, at state stp when s == sp
        auto pAt = [&](int s, int ph, int sp, int stp) {
            return s == sp ? a.vvP[((int64_t)stp * 2 + ph) * N + i + a.off[s]] : P0[s][ph];
        };
        auto uAt = [&](int s, int ph, int sp, int stp) {
            return s == sp ? a.vvU[((int64_t)stp * 2 + ph) * N + i + a.off[s]] : U0[s][ph];
        };
        auto flux = [&](int f, int ph, int sp, int stp) {
            double t = 0.0;
            for (int k = 0; k < a.K; ++k)
                t += a.coef[((int64_t)f * a.K + k) * N + i] * pAt(a.slotOf[f][k], ph, sp, stp);
            t += a.cst[((int64_t)f * 2 + ph) * N + i];
            const int face = f / corners, ax = face >> 1, side = face & 1;
            int pw = 1;
            for (int q = 0; q < ax; ++q) pw *= 3;
            const int so = center + (side ? pw : -pw);
            const double upIn = uAt(center, ph, sp, stp);
            double upOut;
            if ((m >> so) & 1u) upOut = uAt(so, ph, sp, stp);
            else {
                int64_t pos = 0, mul = 1;
                for (int q = 0; q < DIM; ++q)
                    if (q != ax) {
                        pos += id[q] * mul;
                        mul *= q == 0 ? a.nx : q == 1 ? a.ny : a.nz;
                    }
                upOut = a.bU[(int64_t)ph * a.nb + a.sideOffset[face] + pos];
            }
            double mult;
            if (signbit(t)) mult = a.w * upOut + (1.0 - a.w) * upIn;
            else mult = a.w * upIn + (1.0 - a.w) * upOut;
            return t * mult;
        };
        auto residual = [&](int sp, int stp, double* out) {
            double r0 = 0.0, r1 = 0.0;
            r0 -= a.srcterm[i];
            r1 -= a.srcterm[N + i];
            for (int f = 0; f < a.F; ++f) {
                if (a.kind[(int64_t)f * N + i] == 1) {
                    r0 += a.cst[((int64_t)f * 2 + 0) * N + i];
                    r1 += a.cst[((int64_t)f * 2 + 1) * N + i];
                    continue;
                }
                r0 += flux(f, 0, sp, stp);
                r1 += flux(f, 1, sp, stp);
            }
            if (a.transient) {
                const int sti = sp == center ? stp : 0;
                const double V = a.vol[i];
                double st0 = a.vvS[((int64_t)sti * 2 + 0) * N + i];
                st0 -= a.stPrev[i];
                st0 *= V;
                st0 /= a.dt;
                double st1 = a.vvS[((int64_t)sti * 2 + 1) * N + i];
                st1 -= a.stPrev[N + i];
                st1 *= V;
                st1 /= a.dt;
                r0 += st0;
                r1 += st1;
            }
            out[0] = r0;
            out[1] = r1;
        };
        auto partial = [&](int s, int sp, int stp, double* out) {
            double p0 = 0.0, p1 = 0.0;
            for (int f = 0; f < a.F; ++f)
                if (((a.scvfSlots[f] >> s) & 1u) && a.kind[(int64_t)f * N + i] != 1) {
                    p0 += flux(f, 0, sp, stp);
                    p1 += flux(f, 1, sp, stp);
                }
            out[0] = p0;
            out[1] = p1;
        };
        double r0[2];
        residual(-1, 0, r0);
        a.r[i * 2] = r0[0];
        a.r[i * 2 + 1] = r0[1];
        if (!jac) continue;
        for (int s = 0; s < S; ++s) {
            double blk[4] = {0.0, 0.0, 0.0, 0.0};
            if ((m >> s) & 1u) {
                const int64_t j = i + a.off[s];
                auto eval = [&](int stp, double* out) {
                    if (s == center) residual(s, stp, out);
                    else partial(s, s, stp, out);
                };
                double f0[2];
                if (s == center) { f0[0] = r0[0]; f0[1] = r0[1]; }
                else partial(s, -1, 0, f0);
                for (int pv = 0; pv < 2; ++pv) {
                    const double ep = a.eps[(int64_t)pv * N + j];
                    double d[2];
                    if (METHOD == 1) {
                        double fp[2]; eval(1 + pv, fp);
                        for (int e = 0; e < 2; ++e) d[e] = (fp[e] - f0[e]) / ep;
                    } else if (METHOD == -1) {
                        double fm[2]; eval(1 + pv, fm);
                        for (int e = 0; e < 2; ++e) d[e] = (f0[e] - fm[e]) / ep;
                    } else if (METHOD == 0) {
                        double fp[2], fm[2]; eval(1 + SP * pv, fp); eval(2 + SP * pv, fm);
                        for (int e = 0; e < 2; ++e) d[e] = (fp[e] - fm[e]) / (ep + ep);
                    } else {
                        double fp[2], fm[2], fm2[2], fp2[2];
                        eval(1 + SP * pv, fp); eval(2 + SP * pv, fm); eval(3 + SP * pv, fm2); eval(4 + SP * pv, fp2);
                        for (int e = 0; e < 2; ++e) d[e] = fivePointMp(fp[e], fm[e], fm2[e], fp2[e], ep);
                    }
                    blk[0 * 2 + pv] = d[0];
                    blk[1 * 2 + pv] = d[1];
                }
            }
#pragma unroll
            for (int e = 0; e < 4; ++e) a.A[((int64_t)s * N + i) * 4 + e] = blk[e];
        }
    }
}

template <int S, int DIM>
void assemble2p(const MpfaArgs& a, int method, bool jac, cudaStream_t st)
{
    const int threads = 128;
    const int64_t blocks = std::min<int64_t>((a.N + threads - 1) / threads, 152 * 16);
    const dim3 g((unsigned)std::max<int64_t>(blocks, 1));
    if (method == 1) mpfa2pKernel<S, DIM, 1><<<g, threads, 0, st>>>(a, jac);
    else if (method == -1) mpfa2pKernel<S, DIM, -1><<<g, threads, 0, st>>>(a, jac);
    else if (method == 0) mpfa2pKernel<S, DIM, 0><<<g, threads, 0, st>>>(a, jac);
    else mpfa2pKernel<S, DIM, 5><<<g, threads, 0, st>>>(a, jac);
    DXG_CUDA(cudaGetLastError());
}

template <int S>
void assembleS(const MpfaArgs& a, int method, bool jac, cudaStream_t st)
{
    const int threads = 128;
    const int64_t blocks = std::min<int64_t>((a.N + threads - 1) / threads, 152 * 16);
    const dim3 g((unsigned)std::max<int64_t>(blocks, 1));
    if (method == 1) mpfaAssembleKernel<S, 1><<<g, threads, 0, st>>>(a, jac);
    else if (method == -1) mpfaAssembleKernel<S, -1><<<g, threads, 0, st>>>(a, jac);
    else if (method == 0) mpfaAssembleKernel<S, 0><<<g, threads, 0, st>>>(a, jac);
    else if (method == 3) mpfaAssembleKernel<S, 3><<<g, threads, 0, st>>>(a, jac);
    else mpfaAssembleKernel<S, 5><<<g, threads, 0, st>>>(a, jac);
    DXG_CUDA(cudaGetLastError());
}

}  // namespace

void launchMpfaAssemble(const MpfaArgs& a, int method, bool jac, cudaStream_t st)
{
    if (a.b == 2) {
        if (a.S == 9) assemble2p<9, 2>(a, method, jac, st);
        else assemble2p<27, 3>(a, method, jac, st);
        return;
    }
    if (a.S == 9) assembleS<9>(a, method, jac, st);
    else assembleS<27>(a, method, jac, st);
}

}  // namespace dxg
