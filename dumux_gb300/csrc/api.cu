// api.cu -- C ABI of the GB300 cc-TPFA hot path: context, problem tabulation,
// assembler, ILU(0)-BiCGSTAB driver and the Newton driver.
//
// Host code in this file is compiled with FP contraction disabled: the tabulated
// transmissibilities, gravity terms and Dirichlet ghost states are computed with the
// reference's operation order (dumux/flux/cctpfa/darcyslaw.hh:153-259,
// dumux/discretization/cellcentered/tpfa/computetransmissibility.hh:66-80) and so are
// bit-identical to what the reference evaluates for every face.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <exception>
#include <memory>
#include <thread>
#include <vector>

#include "amg.cuh"
#include "context.h"
#include "materiallaw.cuh"

using namespace dxg;

namespace {

std::string g_createError;

// ---------------------------------------------------------------- host geometry
struct HostGrid {
    int dim;
    int64_t n[3];
    const double* x[3];
    void ijk(int64_t c, int64_t* id) const
    {
        id[0] = c % n[0];
        id[1] = (c / n[0]) % n[1];
        id[2] = c / (n[0] * n[1]);
    }
    double lo(int a, int64_t i) const { return x[a][i]; }
    double hi(int a, int64_t i) const { return x[a][i + 1]; }
    void center(const int64_t* id, double* c) const
    {
        for (int a = 0; a < 3; ++a) c[a] = 0.0;
        for (int a = 0; a < dim; ++a) c[a] = 0.5 * (lo(a, id[a]) + hi(a, id[a]));
    }
    double volume(const int64_t* id) const
    {
        double v = 1.0;
        for (int a = 0; a < dim; ++a) v *= hi(a, id[a]) - lo(a, id[a]);
        return v;
    }
    double faceArea(const int64_t* id, int axis) const
    {
        double ar = 1.0;
        for (int k = 0; k < dim; ++k)
            if (k != axis) ar *= hi(k, id[k]) - lo(k, id[k]);
        return ar;
    }
};

// computeTpfaTransmissibility with a scalar permeability: K*extr*((ip-c)/|ip-c|^2 . n)
double tpfaT(int dim, const double* ip, const double* n, const double* c, double K, double extr)
{
    double d[3];
    for (int i = 0; i < dim; ++i) d[i] = ip[i] - c[i];
    double n2 = 0.0;
    for (int i = 0; i < dim; ++i) n2 += d[i] * d[i];
    for (int i = 0; i < dim; ++i) d[i] /= n2;
    double dot = 0.0;
    for (int i = 0; i < dim; ++i) dot += d[i] * n[i];
    return K * extr * dot;
}

double dotN(int dim, const double* n, const double* g)
{
    double s = 0.0;
    for (int i = 0; i < dim; ++i) s += n[i] * g[i];
    return s;
}

// BrooksCoreyDefault evaluated on the host (Dirichlet ghost states, law constants)
template <class T>
void upload(DevBuf<T>& buf, const std::vector<T>& h, cudaStream_t st)
{
    buf.alloc(h.size());
    if (!h.empty()) DXG_CUDA(cudaMemcpyAsync(buf.get(), h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, st));
}

int fail(dxg_ctx* ctx, const Error& e)
{
    if (ctx) ctx->err = e.what();
    return e.status;
}

template <class F>
int guarded(dxg_ctx* ctx, F&& f)
{
    try {
        return f();
    } catch (const Error& e) {
        return fail(ctx, e);
    } catch (const std::bad_alloc&) {
        if (ctx) ctx->err = "host allocation failed";
        return DXG_ERR_OOM;
    } catch (const std::exception& e) {
        if (ctx) ctx->err = e.what();
        return DXG_ERR_ARG;
    }
}

void requireUploaded(const dxg_ctx* ctx)
{
    if (!ctx || !ctx->uploaded) throw Error(DXG_ERR_STATE, "no problem uploaded");
}

cudaEvent_t takeEvent(dxg_ctx* c)
{
    if (!c->eventPool.empty()) {
        cudaEvent_t e = c->eventPool.back();
        c->eventPool.pop_back();
        return e;
    }
    cudaEvent_t e;
    DXG_CUDA(cudaEventCreate(&e));
    return e;
}

void resolveTimings(dxg_ctx* c)
{
    for (auto& t : c->pending) {
        DXG_CUDA(cudaEventSynchronize(t.stop));
        float ms = 0.f;
        DXG_CUDA(cudaEventElapsedTime(&ms, t.start, t.stop));
        c->kcLaunches[t.kclass] += 1;
        c->kcMs[t.kclass] += ms;
        c->kcBytes[t.kclass] += t.bytes;
        c->eventPool.push_back(t.start);
        c->eventPool.push_back(t.stop);
    }
    c->pending.clear();
}

// brackets one launch (or launch group) of a kernel class with events when timing is on
struct TimedScope {
    dxg_ctx* c;
    int kclass;
    double bytes;
    cudaEvent_t start = nullptr;
    TimedScope(dxg_ctx* ctx, int kc, double b) : c(ctx), kclass(kc), bytes(b)
    {
        if (c->timing) {
            start = takeEvent(c);
            DXG_CUDA(cudaEventRecord(start, c->stream));
        }
    }
    ~TimedScope() noexcept(false)
    {
        if (!start) return;
        cudaEvent_t stop = takeEvent(c);
        DXG_CUDA(cudaEventRecord(stop, c->stream));
        c->pending.push_back({start, stop, kclass, bytes});
        if (c->pending.size() >= 2048) resolveTimings(c);
    }
};

}  // namespace

dxg::AssemblyArgs dxg_ctx::asmArgs() const
{
    AssemblyArgs a{};
    a.pc = pcDev.get();
    a.N = N;
    a.nb = nb;
    a.vol = vol.get();
    a.phi = phi.get();
    a.extr = extr.get();
    a.mat = mat.get();
    a.srcterm = srcterm.get();
    a.tijPlus = tijPlus.get();
    a.G1 = G1.get();
    a.G2 = G2.get();
    a.btype = btype.get();
    a.bTij = bTij.get();
    a.bG1 = bG1.get();
    a.bP = bP.get();
    a.bU = bU.get();
    a.bNeu = bNeu.get();
    a.vvP = vvP.get();
    a.vvU = vvU.get();
    a.vvS = vvS.get();
    a.eps = eps.get();
    a.dvv = dvv.get();
    a.color = partialActive ? partialColor.get() : nullptr;
    a.stPrev = stPrev.get();
    a.A = A.get();
    a.r = r.get();
    a.dt = dt;
    return a;
}

namespace {

// f(begin, end) over [0, n) in contiguous chunks on the host's cores (at most 16 threads);
// every index belongs to exactly one chunk, so loops whose iterations write disjoint
// entries give the same tables as the serial loop.  The first exception is rethrown.
template <class F>
void parallelFor(int64_t n, F&& f)
{
    const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
    const int nt = (int)std::min<int64_t>({(int64_t)std::min(hw, 16), (n + 32767) / 32768, (int64_t)16});
    if (nt <= 1) {
        f((int64_t)0, n);
        return;
    }
    std::vector<std::thread> th;
    std::vector<std::exception_ptr> err(nt);
    const int64_t chunk = (n + nt - 1) / nt;
    for (int t = 0; t < nt; ++t)
        th.emplace_back([&, t] {
            try {
                f(std::min(n, t * chunk), std::min(n, (t + 1) * chunk));
            } catch (...) {
                err[t] = std::current_exception();
            }
        });
    for (auto& x : th) x.join();
    for (auto& e : err)
        if (e) std::rethrow_exception(e);
}

// ---------------------------------------------------------------- tabulation
void tabulateMpfa(dxg_ctx* c, const dxg_problem_desc* d);

void tabulate(dxg_ctx* c, const dxg_problem_desc* d)
{
    if (!d) throw Error(DXG_ERR_ARG, "null problem description");
    if (d->discretization != DXG_DISC_TPFA && d->discretization != DXG_DISC_MPFA_O)
        throw Error(DXG_ERR_ARG, "discretization must be DXG_DISC_TPFA or DXG_DISC_MPFA_O");
    if (d->discretization == DXG_DISC_MPFA_O) {
        tabulateMpfa(c, d);
        return;
    }
    if (d->permeability_tensor) throw Error(DXG_ERR_ARG, "a permeability tensor needs the MPFA-O discretization");
    c->mpfa = false;
    if (d->dim != 2 && d->dim != 3) throw Error(DXG_ERR_ARG, "dim must be 2 or 3");
    if (d->num_eq != 1 && d->num_eq != 2) throw Error(DXG_ERR_ARG, "num_eq must be 1 or 2");
    for (int a = 0; a < d->dim; ++a)
        if (d->cells[a] < 1 || !d->coords[a]) throw Error(DXG_ERR_ARG, "invalid cells/coords");
    if (!d->permeability || !d->porosity || !d->bc_type || !d->bc_values) throw Error(DXG_ERR_ARG, "missing tables");
    if (d->diff_method != 0 && d->diff_method != 1) throw Error(DXG_ERR_ARG, "diff_method must be 0 or 1");
    // internal method code: 1 / 0 / -1 numeric differences, 3 analytic derivatives
    const int method = d->diff_method == 1 ? 3 : d->numeric_difference_method;
    if (method != 1 && method != 0 && method != -1 && method != 5 && method != 3)
        throw Error(DXG_ERR_ARG, "numeric difference method must be 1, 0, -1 or 5");
    if (d->num_eq == 2 && d->material_law != 0 && d->material_law != 1)
        throw Error(DXG_ERR_ARG, "material_law must be 0 (Brooks-Corey) or 1 (Van Genuchten)");
    if (d->num_eq == 2 && (d->num_materials < 1 || d->num_materials > kMaxMaterials || !d->material_params))
        throw Error(DXG_ERR_ARG, "2p needs 1..16 Brooks-Corey parameter sets");

    const int dim = d->dim, b = d->num_eq;
    HostGrid g{};
    g.dim = dim;
    for (int a = 0; a < 3; ++a) g.n[a] = a < dim ? d->cells[a] : 1;
    for (int a = 0; a < dim; ++a) g.x[a] = d->coords[a];
    const int64_t N = g.n[0] * g.n[1] * g.n[2];
    if (N > (int64_t)INT32_MAX) throw Error(DXG_ERR_ARG, "too many cells");

    c->dim = dim;
    c->b = b;
    c->N = N;
    c->M = N * b;
    c->slots = 2 * dim + 1;
    c->bb = b * b;
    c->method = method;
    c->gravity = d->enable_gravity != 0;
    c->fullUpwind = d->upwind_weight != 1.0;

    double grav[3] = {0, 0, 0};
    if (c->gravity)
        for (int a = 0; a < dim; ++a) grav[a] = d->gravity[a];
    const int va = dim - 1;
    for (int a = 0; a < dim - 1; ++a)
        if (grav[a] != 0.0) throw Error(DXG_ERR_ARG, "gravity must act along the last axis");

    // problem constants
    ProblemConsts& pc = c->pcHost;
    pc = ProblemConsts{};
    pc.dim = dim;
    pc.b = b;
    pc.nx = (int)g.n[0];
    pc.ny = (int)g.n[1];
    pc.nz = (int)g.n[2];
    pc.N = N;
    pc.sideOffset[0] = 0;
    for (int f = 0; f < 2 * dim; ++f) {
        const int a = f / 2;
        int64_t cnt = 1;
        for (int k = 0; k < dim; ++k)
            if (k != a) cnt *= g.n[k];
        pc.sideOffset[f + 1] = pc.sideOffset[f] + cnt;
    }
    const int64_t nb = pc.sideOffset[2 * dim];
    c->nb = nb;
    pc.gravity = c->gravity;
    pc.gravAxisMask = (c->gravity && grav[va] != 0.0) ? (1 << va) : 0;
    for (int p = 0; p < 2; ++p) {
        pc.density[p] = d->density[p];
        pc.viscosity[p] = d->viscosity[p];
        pc.magnitude[p] = d->privar_magnitude[p];
    }
    pc.mobility1p = 1.0 / d->viscosity[0];
    pc.upwindWeight = d->upwind_weight;
    pc.upwindFull = c->fullUpwind;
    pc.method = method;
    pc.baseEps = d->base_epsilon > 0 ? d->base_epsilon : 1e-10;
    pc.numMaterials = b == 2 ? d->num_materials : 0;
    pc.hasSource = d->source != nullptr;
    const int lawWidth = d->material_law == 1 ? 9 : 5;
    for (int m = 0; m < pc.numMaterials; ++m)
        pc.law[m] = makeMaterialLaw(d->material_law, d->material_params + lawWidth * m);

    const int64_t strides[3] = {1, g.n[0], g.n[0] * g.n[1]};
    for (int s = 0; s < c->slots; ++s) c->off[s] = 0;
    for (int a = 0; a < dim; ++a) {
        c->off[dim - 1 - a] = -strides[a];
        c->off[dim + 1 + a] = strides[a];
    }

    // per-cell tables
    std::vector<double> vol(N), phi(N), extr(N), srcterm((size_t)b * N, 0.0), tijPlus((size_t)dim * N, 0.0);
    std::vector<double> G1((size_t)2 * b * N, 0.0), G2((size_t)2 * b * N, 0.0);
    std::vector<int32_t> mat(N, 0);
    std::vector<uint8_t> nbmask(N, 0);
    auto K = [&](int64_t i) { return d->permeability[i]; };
    auto EX = [&](int64_t i) { return d->extrusion ? d->extrusion[i] : 1.0; };
    parallelFor(N, [&](int64_t i0, int64_t i1) {
    for (int64_t i = i0; i < i1; ++i) {
        int64_t id[3];
        g.ijk(i, id);
        vol[i] = g.volume(id);
        phi[i] = d->porosity[i];
        extr[i] = EX(i);
        if (b == 2) {
            mat[i] = d->material ? d->material[i] : 0;
            if (mat[i] < 0 || mat[i] >= pc.numMaterials) throw Error(DXG_ERR_ARG, "material index out of range");
        }
        const double s = vol[i] * extr[i];
        for (int e = 0; e < b; ++e) {
            double src = 0.0;
            if (d->source) src += d->source[i * b + e];
            src *= s;
            srcterm[(size_t)e * N + i] = src;
        }
        unsigned m = 0;
        for (int f = 0; f < 2 * dim; ++f) {
            const int a = f / 2;
            const bool interior = (f & 1) ? id[a] < g.n[a] - 1 : id[a] > 0;
            if (interior) m |= 1u << f;
        }
        nbmask[i] = (uint8_t)m;
    }
    });
    // interior faces: transmissibility of the + face of every axis, gravity terms of the
    // vertical faces (both orientations; the entry of each (face side, cell) is written by
    // exactly one iteration)
    parallelFor(N, [&](int64_t i0, int64_t i1) {
    for (int64_t i = i0; i < i1; ++i) {
        int64_t id[3];
        g.ijk(i, id);
        double ci[3];
        g.center(id, ci);
        for (int a = 0; a < dim; ++a) {
            if (id[a] >= g.n[a] - 1) continue;
            const int64_t j = i + strides[a];
            int64_t jd[3] = {id[0], id[1], id[2]};
            jd[a] += 1;
            double cj[3];
            g.center(jd, cj);
            double ip[3] = {ci[0], ci[1], ci[2]};
            ip[a] = g.hi(a, id[a]);
            double n[3] = {0, 0, 0};
            n[a] = 1.0;
            const double area = g.faceArea(id, a);
            const double ti = tpfaT(dim, ip, n, ci, K(i), EX(i));
            const double tj = -1.0 * tpfaT(dim, ip, n, cj, K(j), EX(j));
            const double tij = (ti * tj <= 0.0) ? 0 : area * (ti * tj) / (ti + tj);
            tijPlus[(size_t)a * N + i] = tij;
            if (c->gravity && a == va && grav[va] != 0.0) {
                // directed from i (+ face of i) and from j (- face of j)
                for (int side = 0; side < 2; ++side) {
                    const int64_t in = side == 0 ? i : j, out = side == 0 ? j : i;
                    const double* cin = side == 0 ? ci : cj;
                    const double* cout = side == 0 ? cj : ci;
                    double nn[3] = {0, 0, 0};
                    nn[a] = side == 0 ? 1.0 : -1.0;
                    // recompute the transmissibility from this side, as the reference does
                    const double tIn = tpfaT(dim, ip, nn, cin, K(in), EX(in));
                    const double tOut = -1.0 * tpfaT(dim, ip, nn, cout, K(out), EX(out));
                    const double tijS = (tIn * tOut <= 0.0) ? 0 : area * (tIn * tOut) / (tIn + tOut);
                    if (tijS != tij) throw Error(DXG_ERR_ARG, "asymmetric transmissibility");
                    const double ng = dotN(dim, nn, grav);
                    const double alphaIn = K(in) * ng * EX(in);
                    const double alphaOut = K(out) * ng * EX(out);
                    const double outsideTi = -1.0 * tpfaT(dim, ip, nn, cout, K(out), EX(out));
                    for (int ph = 0; ph < b; ++ph) {
                        const double rho = (d->density[ph] + d->density[ph]) * 0.5;
                        const double g1 = rho * area * alphaIn;
                        const double g2 = rho * tijS / outsideTi * (alphaIn - alphaOut);
                        // stored at the inside cell under its face side (0: -va face, 1: +va face)
                        const int fs = side == 0 ? 1 : 0;
                        G1[((size_t)fs * b + ph) * N + in] = g1;
                        G2[((size_t)fs * b + ph) * N + in] = g2;
                    }
                }
            }
        }
    }
    });
    // boundary faces
    std::vector<int8_t> btype(nb);
    std::vector<double> bTij(nb, 0.0), bG1((size_t)b * nb, 0.0), bP((size_t)b * nb, 0.0), bU((size_t)b * nb, 0.0),
        bNeu((size_t)b * nb, 0.0);
    for (int f = 0; f < 2 * dim; ++f) {
        const int a = f / 2, side = f & 1;
        int o1 = -1, o2 = -1;
        for (int k = 0; k < dim; ++k)
            if (k != a) { if (o1 < 0) o1 = k; else o2 = k; }
        const int64_t n1 = g.n[o1], n2 = o2 >= 0 ? g.n[o2] : 1;
        for (int64_t q2 = 0; q2 < n2; ++q2)
            for (int64_t q1 = 0; q1 < n1; ++q1) {
                const int64_t bidx = pc.sideOffset[f] + q1 + n1 * q2;
                int64_t id[3] = {0, 0, 0};
                id[a] = side ? g.n[a] - 1 : 0;
                id[o1] = q1;
                if (o2 >= 0) id[o2] = q2;
                const int64_t i = id[0] + strides[1] * id[1] + strides[2] * id[2];
                const int8_t t = d->bc_type[bidx];
                if (t != 1 && t != 2) throw Error(DXG_ERR_ARG, "boundary type must be 1 (Dirichlet) or 2 (Neumann)");
                btype[bidx] = t;
                double ci[3];
                g.center(id, ci);
                double ip[3] = {ci[0], ci[1], ci[2]};
                ip[a] = side ? g.hi(a, id[a]) : g.lo(a, id[a]);
                double n[3] = {0, 0, 0};
                n[a] = side ? 1.0 : -1.0;
                const double area = g.faceArea(id, a);
                const double* bv = d->bc_values + bidx * b;
                if (t == 1) {
                    const double ti = tpfaT(dim, ip, n, ci, K(i), EX(i));
                    bTij[bidx] = area * ti;
                    // ghost volume variables from the Dirichlet values with the inside cell's
                    // spatial parameters (elementvolumevariables.hh:317-342)
                    if (b == 1) {
                        bP[bidx] = bv[0];
                        bU[bidx] = d->density[0] * (1.0 / d->viscosity[0]);
                    } else {
                        const MaterialLaw& m = pc.law[mat[i]];
                        const double Sn = bv[1];
                        const double Sw = 1 - Sn;
                        const double pcap = lawPc(m, Sw);
                        bP[0 * nb + bidx] = bv[0];
                        bP[1 * nb + bidx] = bv[0] + pcap;
                        bU[0 * nb + bidx] = d->density[0] * (lawKrw(m, Sw) / d->viscosity[0]);
                        bU[1 * nb + bidx] = d->density[1] * (lawKrn(m, Sw) / d->viscosity[1]);
                    }
                    if (c->gravity && a == va && grav[va] != 0.0) {
                        const double ng = dotN(dim, n, grav);
                        const double alphaIn = K(i) * ng * EX(i);
                        for (int ph = 0; ph < b; ++ph) bG1[(size_t)ph * nb + bidx] = d->density[ph] * area * alphaIn;
                    }
                } else {
                    const double s = area * EX(i);
                    for (int e = 0; e < b; ++e) {
                        double q = 0.0;
                        q += bv[e] * s;
                        bNeu[(size_t)e * nb + bidx] = q;
                    }
                }
            }
    }
    // level schedule of the ILU(0) wavefront
    const int numLevels = (int)(g.n[0] + g.n[1] + g.n[2] - 2);
    std::vector<int32_t> cnt(numLevels + 1, 0), perm(N);
    for (int64_t i = 0; i < N; ++i) {
        int64_t id[3];
        g.ijk(i, id);
        cnt[id[0] + id[1] + id[2] + 1]++;
    }
    for (int L = 0; L < numLevels; ++L) cnt[L + 1] += cnt[L];
    c->levels.numLevels = numLevels;
    c->levels.ptr = cnt;
    {
        std::vector<int32_t> pos(cnt.begin(), cnt.end() - 1);
        for (int64_t i = 0; i < N; ++i) {
            int64_t id[3];
            g.ijk(i, id);
            perm[pos[id[0] + id[1] + id[2]]++] = (int32_t)i;
        }
    }
    int64_t nnzb = N;
    for (int64_t i = 0; i < N; ++i)
        for (int f = 0; f < 2 * dim; ++f) nnzb += (nbmask[i] >> f) & 1;
    c->nnzb = nnzb;
    c->nbmaskHost = nbmask;
    {
        // algorithmic bytes per launch with 8-byte values: every block / entry once
        const double bb8 = 8.0 * b * b, v8 = 8.0 * b;
        const double offBlocks = (double)(nnzb - N);      // = lower + upper blocks
        // forward: lower blocks + rhs + z; backward: upper blocks + Dinv + z + y
        c->bytesSweep = (offBlocks * bb8 + N * (v8 + v8)) + (N * bb8 + N * (v8 + v8));
        // SpMV: all blocks + neighbour mask + x + y
        c->bytesSpmv = nnzb * bb8 + N * 1.0 + 2.0 * N * v8;
        // factor: lower and diagonal blocks read, lower factor and inverted pivots written
        c->bytesFactor = (double)N * bb8 * (2.0 * dim + 2.0);
        // assembly: u read, volume variables written and read back, coefficients,
        // Jacobian rows and residual written
        const int NS = method == 3 ? 1 : 1 + statesPerPv(method) * b;
        c->bytesAssembly = N * v8 + 3.0 * N * NS * v8 + N * b * 8.0 /*eps*/ + N * (8.0 * dim + 2.0 * 2 * b * 8.0) +
                           N * (3 * 8.0 + 1 + b * 8.0) + (double)c->slots * N * bb8 + N * v8;
    }

    cudaStream_t st = c->stream;
    // the first upload carves its buffers from one allocation of the problem's size
    std::unique_ptr<DevBlockScope> carve;
    if (!c->uploadBlock.get()) {
        const int64_t need = dxg_problem_device_bytes(d, c->precision);
        if (need > 0) {
            c->uploadBlock.alloc((size_t)need);
            c->uploadCarve = DevBlock{c->uploadBlock.get(), (size_t)need, 0};
            carve.reset(new DevBlockScope(&c->uploadCarve));
        }
    }
    c->pcDev.alloc(1);
    DXG_CUDA(cudaMemcpyAsync(c->pcDev.get(), &c->pcHost, sizeof(ProblemConsts), cudaMemcpyHostToDevice, st));
    upload(c->vol, vol, st);
    upload(c->phi, phi, st);
    upload(c->extr, extr, st);
    upload(c->srcterm, srcterm, st);
    upload(c->tijPlus, tijPlus, st);
    upload(c->G1, G1, st);
    upload(c->G2, G2, st);
    upload(c->mat, mat, st);
    upload(c->nbmask, nbmask, st);
    upload(c->btype, btype, st);
    upload(c->bTij, bTij, st);
    upload(c->bG1, bG1, st);
    upload(c->bP, bP, st);
    upload(c->bU, bU, st);
    upload(c->bNeu, bNeu, st);
    upload(c->perm, perm, st);
    DXG_CUDA(cudaStreamSynchronize(st));   // host vectors go out of scope

    const int NS = method == 3 ? 1 : 1 + statesPerPv(method) * b;
    const int64_t M = N * b;
    c->u.alloc(M);
    c->uprev.alloc(M);
    c->uLast.alloc(M);
    c->stPrev.alloc((size_t)b * N);
    c->vvP.alloc((size_t)NS * b * N);
    c->vvU.alloc((size_t)NS * b * N);
    c->vvS.alloc((size_t)NS * b * N);
    c->eps.alloc((size_t)b * N);
    if (method == 3 && b == 2) c->dvv.alloc((size_t)3 * N);   // d(krw, krn, pc)/dSn per cell
    c->A.alloc((size_t)c->slots * N * c->bb);
    c->r.alloc(M);
    c->delta.alloc(M);
    DXG_CUDA(cudaMemsetAsync(c->u.get(), 0, M * sizeof(double), st));
    DXG_CUDA(cudaMemsetAsync(c->uprev.get(), 0, M * sizeof(double), st));
    DXG_CUDA(cudaMemsetAsync(c->delta.get(), 0, M * sizeof(double), st));
    for (auto* v : {&c->kx, &c->kr, &c->krt, &c->kp, &c->kv, &c->kt, &c->ky}) v->alloc(M);
    if (c->precision == DXG_PRECISION_FP64) {
        c->L.alloc((size_t)dim * N * c->bb);
        c->Dinv.alloc((size_t)N * c->bb);
    } else {
        c->Af.alloc((size_t)c->slots * N * c->bb);
        c->Lf.alloc((size_t)dim * N * c->bb);
        c->Dinvf.alloc((size_t)N * c->bb);
        for (auto* v : {&c->fr, &c->fp, &c->fy}) v->alloc(M);
    }
    c->ks.alloc(1);
    c->partials.alloc(3 * kMaxReduceBlocks);
    c->counters.alloc(8);
    c->scal.alloc(4);
    c->singular.alloc(2);
    c->wavePlan = makeWavePlan(dim, (int)g.n[0], (int)g.n[1], (int)g.n[2], b, c->precision == DXG_PRECISION_FP64);
    c->lanePlan = c->precision == DXG_PRECISION_FP64 ? makeLanePlan<double>(dim, (int)g.n[0], (int)g.n[1], (int)g.n[2], b)
                                                      : makeLanePlan<float>(dim, (int)g.n[0], (int)g.n[1], (int)g.n[2], b);
    c->waveTuned = false;
    c->laneWave = false;
    c->laneTuneMs = 0.0;
    c->line2dOk = tpfaLine2dFits(dim, (int)g.n[0], (int)g.n[1], b);
    c->line2d = false;
    c->line2dMs = 0.0;
    c->laneHandoff.release();
    c->laneHandoffBytes = 0;
    c->waveTuneCount = 0;
    c->dropGraphs();   // the captured chunks hold the old buffers' addresses
    DXG_CUDA(cudaMemsetAsync(c->counters.get(), 0, 8 * sizeof(unsigned), st));
    DXG_CUDA(cudaMemsetAsync(c->singular.get(), 0, 2 * sizeof(int), st));
    DXG_CUDA(cudaMemsetAsync(c->ks.get(), 0, sizeof(KrylovState), st));
    DXG_CUDA(cudaMemsetAsync(c->scal.get(), 0, 4 * sizeof(double), st));
    DXG_CUDA(cudaStreamSynchronize(st));
    c->uploaded = true;
    c->havePrev = false;
    c->stPrevValid = false;
    c->haveJac = c->haveRes = c->haveFactor = false;
}

// MPFA-O (1p, FP64 single contexts): the interaction volumes solved on the host
// (mpfaTabulate), the per-cell flux rows, the 3^dim stencil and the Krylov buffers.
void tabulateMpfa2p(dxg_ctx* c, const dxg_problem_desc* d);

void tabulateMpfa(dxg_ctx* c, const dxg_problem_desc* d)
{
    if (d->dim != 2 && d->dim != 3) throw Error(DXG_ERR_ARG, "dim must be 2 or 3");
    if (d->num_eq != 1 && d->num_eq != 2) throw Error(DXG_ERR_ARG, "num_eq must be 1 or 2");
    if (c->precision != DXG_PRECISION_FP64) throw Error(DXG_ERR_ARG, "MPFA-O runs in FP64");
    if (d->num_eq == 2) {
        tabulateMpfa2p(c, d);
        return;
    }
    for (int a = 0; a < d->dim; ++a)
        if (d->cells[a] < 1 || !d->coords[a]) throw Error(DXG_ERR_ARG, "invalid cells/coords");
    if (!d->permeability || !d->porosity || !d->bc_type || !d->bc_values) throw Error(DXG_ERR_ARG, "missing tables");
    if (d->diff_method != 0 && d->diff_method != 1) throw Error(DXG_ERR_ARG, "diff_method must be 0 or 1");
    // internal method code as for TPFA: 1 / 0 / -1 / 5 numeric differences, 3 analytic
    const int method = d->diff_method == 1 ? 3 : d->numeric_difference_method;
    if (method != 1 && method != 0 && method != -1 && method != 5 && method != 3)
        throw Error(DXG_ERR_ARG, "numeric difference method must be 1, 0, -1 or 5");
    const int dim = d->dim;
    HostGrid g{};
    g.dim = dim;
    for (int a = 0; a < 3; ++a) g.n[a] = a < dim ? d->cells[a] : 1;
    for (int a = 0; a < dim; ++a) g.x[a] = d->coords[a];
    const int64_t N = g.n[0] * g.n[1] * g.n[2];
    if (N > (int64_t)INT32_MAX) throw Error(DXG_ERR_ARG, "too many cells");
    if (g.n[1] * g.n[2] > (int64_t)INT32_MAX) throw Error(DXG_ERR_ARG, "too many grid lines");
    const MpfaLayout L = mpfaLayout(dim);
    c->mpfa = true;
    c->mpLayout = L;
    c->dim = dim;
    c->b = 1;
    c->N = N;
    c->M = N;
    c->slots = L.S;
    c->bb = 1;
    c->method = method;
    c->gravity = d->enable_gravity != 0;
    c->fullUpwind = false;
    ProblemConsts& pc = c->pcHost;
    pc = ProblemConsts{};
    pc.dim = dim;
    pc.b = 1;
    pc.nx = (int)g.n[0];
    pc.ny = (int)g.n[1];
    pc.nz = (int)g.n[2];
    pc.N = N;
    pc.sideOffset[0] = 0;
    for (int f = 0; f < 2 * dim; ++f) {
        const int a = f / 2;
        int64_t cnt = 1;
        for (int k = 0; k < dim; ++k)
            if (k != a) cnt *= g.n[k];
        pc.sideOffset[f + 1] = pc.sideOffset[f] + cnt;
    }
    c->nb = pc.sideOffset[2 * dim];
    for (int64_t k = 0; k < c->nb; ++k)
        if (d->bc_type[k] != 1 && d->bc_type[k] != 2)
            throw Error(DXG_ERR_ARG, "boundary type must be 1 (Dirichlet) or 2 (Neumann)");
    pc.density[0] = d->density[0];
    pc.viscosity[0] = d->viscosity[0];
    pc.magnitude[0] = d->privar_magnitude[0];
    pc.baseEps = d->base_epsilon > 0 ? d->base_epsilon : 1e-10;
    pc.method = method;
    c->mpMob = d->density[0] * (1.0 / d->viscosity[0]);
    c->mpUp = d->density[0] / d->viscosity[0];
    const int64_t strides[3] = {1, g.n[0], g.n[0] * g.n[1]};
    for (int s = 0; s < L.S; ++s) {
        int o[3] = {0, 0, 0}, q = s;
        for (int a = 0; a < dim; ++a) {
            o[a] = q % 3 - 1;
            q /= 3;
        }
        c->mpOff[s] = o[0] * strides[0] + o[1] * strides[1] + o[2] * strides[2];
    }
    mpfaTriples(dim, c->mpNTri, c->mpTri);

    // per cell: source * volume * extrusion (the TPFA order), the stencil mask
    std::vector<double> srcterm(N, 0.0);
    std::vector<uint32_t> mask(N, 0);
    parallelFor(N, [&](int64_t i0, int64_t i1) {
        for (int64_t i = i0; i < i1; ++i) {
            int64_t id[3];
            g.ijk(i, id);
            const double sV = g.volume(id) * (d->extrusion ? d->extrusion[i] : 1.0);
            double src = 0.0;
            if (d->source) src += d->source[i];
            src *= sV;
            srcterm[i] = src;
            uint32_t m = 0;
            for (int s = 0; s < L.S; ++s) {
                int q = s;
                bool ok = true;
                for (int a = 0; a < dim; ++a) {
                    const int64_t x = id[a] + (q % 3 - 1);
                    q /= 3;
                    if (x < 0 || x >= g.n[a]) ok = false;
                }
                if (ok) m |= 1u << s;
            }
            mask[i] = m;
        }
    });
    std::vector<double> coef, cst;
    std::vector<int8_t> kind;
    mpfaTabulate(d, L, pc.sideOffset, nullptr, coef, cst, kind);
    int64_t nnz = 0;
    for (int64_t i = 0; i < N; ++i) nnz += __builtin_popcount(mask[i]);
    c->nnzb = nnz;
    c->mpMaskHost = mask;
    c->bytesAssembly = (double)N * (8.0 * L.F * (L.K + 1) + L.F + 4.0 + 8.0 * (L.S + 3) + 8.0 * L.S + 8.0);
    c->bytesSpmv = (double)nnz * 8.0 + N * 4.0 + 2.0 * N * 8.0;
    c->bytesSweep = (double)nnz * 8.0 + N * (8.0 + 4.0 * 8.0);
    c->bytesFactor = (double)nnz * 16.0 + N * 8.0;

    cudaStream_t st = c->stream;
    c->uploadBlock.release();
    c->pcDev.alloc(1);
    DXG_CUDA(cudaMemcpyAsync(c->pcDev.get(), &c->pcHost, sizeof(ProblemConsts), cudaMemcpyHostToDevice, st));
    upload(c->srcterm, srcterm, st);
    upload(c->mpMask, mask, st);
    upload(c->mpCoef, coef, st);
    upload(c->mpCst, cst, st);
    upload(c->mpKind, kind, st);
    DXG_CUDA(cudaStreamSynchronize(st));
    c->u.alloc(N);
    c->uprev.alloc(N);
    c->uLast.alloc(N);
    c->A.alloc((size_t)L.S * N);
    c->r.alloc(N);
    c->delta.alloc(N);
    DXG_CUDA(cudaMemsetAsync(c->u.get(), 0, N * sizeof(double), st));
    DXG_CUDA(cudaMemsetAsync(c->uprev.get(), 0, N * sizeof(double), st));
    DXG_CUDA(cudaMemsetAsync(c->delta.get(), 0, N * sizeof(double), st));
    DXG_CUDA(cudaMemsetAsync(c->A.get(), 0, (size_t)L.S * N * sizeof(double), st));
    for (auto* v : {&c->kx, &c->kr, &c->krt, &c->kp, &c->kv, &c->kt, &c->ky}) v->alloc(N);
    c->L.alloc((size_t)L.S * N);
    c->Dinv.alloc(N);
    c->ks.alloc(1);
    c->partials.alloc(3 * kMaxReduceBlocks);
    c->counters.alloc(8);
    c->scal.alloc(4);
    c->singular.alloc(2);
    c->wavePlan = WavePlan{};
    c->lanePlan = LanePlan{};
    c->line2dOk = c->line2d = false;
    c->waveTuned = true;
    c->laneWave = false;
    c->laneTuneMs = 0.0;
    c->laneHandoff.release();
    c->laneHandoffBytes = 0;
    c->waveTuneCount = 0;
    c->dropGraphs();
    DXG_CUDA(cudaMemsetAsync(c->counters.get(), 0, 8 * sizeof(unsigned), st));
    DXG_CUDA(cudaMemsetAsync(c->singular.get(), 0, 2 * sizeof(int), st));
    DXG_CUDA(cudaMemsetAsync(c->ks.get(), 0, sizeof(KrylovState), st));
    DXG_CUDA(cudaMemsetAsync(c->scal.get(), 0, 4 * sizeof(double), st));
    DXG_CUDA(cudaStreamSynchronize(st));
    c->uploaded = true;
    c->havePrev = false;
    c->stPrevValid = false;
    c->haveJac = c->haveRes = c->haveFactor = false;
}

// MPFA-O for the 2p model: the TPFA tabulation supplies the volume variables, storage,
// sources and the Dirichlet ghosts of the 2p model; the interaction volumes add the flux rows
// (per phase constants from the ghosts' phase pressures and gravity), and the Jacobian, its
// factor and the pivots take the 3^dim stencil of 2x2 blocks.
void tabulateMpfa2p(dxg_ctx* c, const dxg_problem_desc* d)
{
    if (d->diff_method != 0) throw Error(DXG_ERR_ARG, "MPFA-O with the 2p model assembles by numeric differentiation");
    dxg_problem_desc dt = *d;
    dt.discretization = DXG_DISC_TPFA;
    dt.permeability_tensor = nullptr;
    tabulate(c, &dt);
    const int dim = d->dim;
    const MpfaLayout L = mpfaLayout(dim);
    const ProblemConsts& pc = c->pcHost;
    const int64_t n[3] = {pc.nx, pc.ny, pc.nz};
    const int64_t N = c->N, nb = c->nb;
    // the Dirichlet ghosts' phase pressures (p_n = p_w + pc(1 - S_n) with the inside cell's law)
    std::vector<double> dirP((size_t)2 * nb, 0.0);
    for (int f = 0; f < 2 * dim; ++f) {
        const int a = f / 2, side = f & 1;
        int o1 = -1, o2 = -1;
        for (int k = 0; k < dim; ++k)
            if (k != a) { if (o1 < 0) o1 = k; else o2 = k; }
        const int64_t n1 = n[o1], n2 = o2 >= 0 ? n[o2] : 1;
        for (int64_t q2 = 0; q2 < n2; ++q2)
            for (int64_t q1 = 0; q1 < n1; ++q1) {
                const int64_t bidx = pc.sideOffset[f] + q1 + n1 * q2;
                if (d->bc_type[bidx] != 1) continue;
                int64_t id[3] = {0, 0, 0};
                id[a] = side ? n[a] - 1 : 0;
                id[o1] = q1;
                if (o2 >= 0) id[o2] = q2;
                const int64_t i = id[0] + n[0] * (id[1] + n[1] * id[2]);
                const MaterialLaw& m = pc.law[d->material ? d->material[i] : 0];
                const double* bv = d->bc_values + bidx * 2;
                const double Sw = 1 - bv[1];
                const double pcap = lawPc(m, Sw);
                dirP[bidx] = bv[0];
                dirP[nb + bidx] = bv[0] + pcap;
            }
    }
    c->mpfa = true;
    c->mpLayout = L;
    c->slots = L.S;
    const int64_t strides[3] = {1, n[0], n[0] * n[1]};
    for (int s = 0; s < L.S; ++s) {
        int o[3] = {0, 0, 0}, q = s;
        for (int a = 0; a < dim; ++a) {
            o[a] = q % 3 - 1;
            q /= 3;
        }
        c->mpOff[s] = o[0] * strides[0] + o[1] * strides[1] + o[2] * strides[2];
    }
    mpfaTriples(dim, c->mpNTri, c->mpTri);
    std::vector<uint32_t> mask(N, 0);
    for (int64_t i = 0; i < N; ++i) {
        const int64_t id[3] = {i % n[0], (i / n[0]) % n[1], i / (n[0] * n[1])};
        uint32_t mm = 0;
        for (int s = 0; s < L.S; ++s) {
            int q = s;
            bool ok = true;
            for (int a = 0; a < dim; ++a) {
                const int64_t x = id[a] + (q % 3 - 1);
                q /= 3;
                if (x < 0 || x >= n[a]) ok = false;
            }
            if (ok) mm |= 1u << s;
        }
        mask[i] = mm;
    }
    std::vector<double> coef, cst;
    std::vector<int8_t> kind;
    mpfaTabulate(d, L, pc.sideOffset, dirP.data(), coef, cst, kind);
    int64_t nnz = 0;
    for (int64_t i = 0; i < N; ++i) nnz += __builtin_popcount(mask[i]);
    c->nnzb = nnz;
    c->mpMaskHost = mask;
    c->mpMob = 0.0;
    c->mpUp = 0.0;
    c->bytesAssembly += (double)N * (8.0 * L.F * (L.K + 2) + L.F + 4.0);
    c->bytesSpmv = (double)nnz * 32.0 + N * 4.0 + 2.0 * N * 16.0;
    c->bytesSweep = (double)nnz * 32.0 + N * (32.0 + 4.0 * 16.0);
    c->bytesFactor = (double)nnz * 64.0 + N * 32.0;
    cudaStream_t st = c->stream;
    upload(c->mpMask, mask, st);
    upload(c->mpCoef, coef, st);
    upload(c->mpCst, cst, st);
    upload(c->mpKind, kind, st);
    c->A.alloc((size_t)L.S * N * 4);
    c->L.alloc((size_t)L.S * N * 4);
    c->Dinv.alloc((size_t)N * 4);
    DXG_CUDA(cudaMemsetAsync(c->A.get(), 0, (size_t)L.S * N * 4 * sizeof(double), st));
    DXG_CUDA(cudaStreamSynchronize(st));
    c->wavePlan = WavePlan{};
    c->lanePlan = LanePlan{};
    c->line2dOk = c->line2d = false;
    c->waveTuned = true;
    c->laneWave = false;
    c->dropGraphs();
    c->haveJac = c->haveRes = c->haveFactor = false;
}

MpfaArgs mpfaArgs(const dxg_ctx* c)
{
    const MpfaLayout& L = c->mpLayout;
    MpfaArgs a{};
    a.N = c->N;
    a.S = L.S;
    a.F = L.F;
    a.K = L.K;
    for (int s = 0; s < L.S; ++s) a.off[s] = c->mpOff[s];
    std::memcpy(a.slotOf, L.slotOf, sizeof(a.slotOf));
    std::memcpy(a.scvfSlots, L.scvfSlots, sizeof(a.scvfSlots));
    a.coef = c->mpCoef.get();
    a.cst = c->mpCst.get();
    a.kind = c->mpKind.get();
    a.mask = c->mpMask.get();
    a.srcterm = c->srcterm.get();
    a.u = c->u.get();
    a.mob = c->mpMob;
    a.up = c->mpUp;
    a.baseEps = c->pcHost.baseEps;
    a.magnitude = c->pcHost.magnitude[0];
    a.transient = c->dt > 0.0;
    a.A = c->A.get();
    a.r = c->r.get();
    a.b = c->b;
    if (c->b == 2) {
        a.nx = c->pcHost.nx;
        a.ny = c->pcHost.ny;
        a.nz = c->pcHost.nz;
        a.nb = c->nb;
        for (int f = 0; f < 7; ++f) a.sideOffset[f] = c->pcHost.sideOffset[f];
        a.vvP = c->vvP.get();
        a.vvU = c->vvU.get();
        a.vvS = c->vvS.get();
        a.eps = c->eps.get();
        a.stPrev = c->stPrev.get();
        a.vol = c->vol.get();
        a.bU = c->bU.get();
        a.w = c->pcHost.upwindWeight;
        a.dt = c->dt;
    }
    return a;
}

// The MPFA-O preconditioner apply: 1 the one-CTA line sweeps (2D with up to 1024 lines:
// DXG_ILU_WAVEFRONT or auto), 2 the cluster line sweeps (2D: DXG_ILU_LANES, or auto beyond
// 1024 lines), 3 the 3D cluster sweeps (one z-plane per CTA: DXG_ILU_LANES or auto), 0 the
// level-by-level kernel (DXG_ILU_LEVELS, or when none fits).  On 256 x 256 the one-CTA sweeps
// took 1.09 ms per apply, the cluster sweeps (two CTAs, polled hand-offs between warps)
// 1.0-2.4 ms.
int mpfaSweep(const dxg_ctx* c, const StencilArgs& sa)
{
    const bool lanes = stencilLane2dFits(sa), wave = stencilWave2dFits(sa), lanes3 = stencilLane3dFits(sa);
    switch (c->iluKernel) {
    case DXG_ILU_LEVELS: return 0;
    case DXG_ILU_LANES: return lanes ? 2 : lanes3 ? 3 : 0;
    case DXG_ILU_WAVEFRONT: return wave ? 1 : 0;
    default: return wave ? 1 : lanes ? 2 : lanes3 ? 3 : 0;
    }
}

StencilArgs stencilArgs(dxg_ctx* c)
{
    StencilArgs a{};
    a.b = c->b;
    a.nx = c->pcHost.nx;
    a.ny = c->pcHost.ny;
    a.nz = c->pcHost.nz;
    a.N = c->N;
    a.S = c->mpLayout.S;
    a.center = c->mpLayout.center;
    for (int s = 0; s < a.S; ++s) a.off[s] = c->mpOff[s];
    a.mask = c->mpMask.get();
    a.A = c->A.get();
    a.LU = c->L.get();
    a.Dinv = c->Dinv.get();
    a.singular = c->singular.get();
    a.ks = c->ks.get();
    a.scratch = c->scratch();
    a.nTri = c->mpNTri;
    std::memcpy(a.tri, c->mpTri, sizeof(a.tri));
    a.err = c->singular.get() + 1;
    a.waitNs = c->waitNs;
    return a;
}

// slot s of row i: inside the pattern, and its column offset
bool slotInPattern(const dxg_ctx* c, int64_t i, int s)
{
    if (c->mpfa) return (c->mpMaskHost[i] >> s) & 1u;
    if (s == c->dim) return true;
    const int f = s < c->dim ? 2 * (c->dim - 1 - s) : 2 * (s - c->dim - 1) + 1;
    return (c->nbmaskHost[i] >> f) & 1u;
}
int64_t slotOffset(const dxg_ctx* c, int s) { return c->mpfa ? c->mpOff[s] : c->off[s]; }

// ---------------------------------------------------------------- assembly
void ensurePrevStorage(dxg_ctx* c)
{
    if (c->dt > 0.0 && !c->stPrevValid) {
        launchPrevStorage(c->asmArgs(), c->b, c->uprev.get(), c->stream);
        c->launches += 1;
        c->stPrevValid = true;
    }
}

void assemble(dxg_ctx* c, bool jac)
{
    requireUploaded(c);
    if (c->dt > 0.0 && !c->havePrev) throw Error(DXG_ERR_STATE, "transient assembly needs the previous solution");
    if (c->mpfa) {
        TimedScope ts(c, DXG_KC_ASSEMBLY, jac ? c->bytesAssembly : 0.0);
        if (c->b == 2) {
            // the volume variables of every cell at its own and perturbed states
            ensurePrevStorage(c);
            launchVolvars(c->asmArgs(), 2, jac ? c->method : 2, c->u.get(), c->stream);
            c->launches += 1;
        }
        launchMpfaAssemble(mpfaArgs(c), c->method, jac, c->stream);
        c->launches += 1;
        c->haveRes = true;
        if (jac) {
            c->haveJac = true;
            c->haveFactor = false;
        }
        return;
    }
    ensurePrevStorage(c);
    const AssemblyArgs a = c->asmArgs();
    TimedScope ts(c, DXG_KC_ASSEMBLY, jac ? c->bytesAssembly : 0.0);
    launchVolvars(a, c->b, jac ? c->method : 2, c->u.get(), c->stream);
    launchRow(a, c->b, c->dim, c->method, jac, c->gravity && c->pcHost.gravAxisMask, c->dt > 0.0, c->fullUpwind,
              c->stream);
    c->launches += 2;
    c->haveRes = true;
    if (jac) {
        c->haveJac = true;
        c->haveFactor = false;
    }
}

double deviceNorm(dxg_ctx* c, const double* x)
{
    launchNorm2(x, c->M, c->scratch(), c->scal.get() + 1, c->stream);
    c->launches += 1;
    DXG_CUDA(cudaMemcpyAsync(c->scalHost + 1, c->scal.get() + 1, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    DXG_CUDA(cudaStreamSynchronize(c->stream));
    return c->scalHost[1];
}

// ---------------------------------------------------------------- linear solve
template <class T>
WaveArgs<T> waveArgs(dxg_ctx* c, const T* A, T* L, T* Dinv, const T* rhs, T* v)
{
    WaveArgs<T> w{};
    w.dim = c->dim;
    w.nx = c->pcHost.nx;
    w.ny = c->pcHost.ny;
    w.nz = c->pcHost.nz;
    w.N = c->N;
    w.ctas = c->wavePlan.ctas;
    w.linesPerCta = c->wavePlan.linesPerCta;
    w.haloLines = c->wavePlan.haloLines;
    w.A = A;
    w.L = L;
    w.Dinv = Dinv;
    w.rhs = rhs;
    w.v = v;
    w.err = c->singular.get() + 1;
    w.singular = c->singular.get();
    w.ks = c->ks.get();
    w.waitNs = c->waitNs;
    return w;
}

bool useWave(const dxg_ctx* c)
{
    return c->iluKernel != DXG_ILU_LEVELS && c->iluKernel != DXG_ILU_REDBLACK && c->wavePlan.ok;
}

// The lane sweeps apply the preconditioner (the factorisation stays with the cluster
// wavefront or the level-scheduled kernels).
bool useLane(const dxg_ctx* c)
{
    return c->lanePlan.ok && c->linearSolver == DXG_LINEAR_SOLVER_ILU_BICGSTAB &&
           (c->iluKernel == DXG_ILU_LANES || (c->iluKernel == DXG_ILU_AUTO && c->laneWave));
}

// The one-CTA line sweeps of 2D TPFA systems apply the preconditioner (DXG_ILU_LANES on a 2D
// grid, or DXG_ILU_AUTO when the timing at the first factorisation found them faster).
bool useLine2d(const dxg_ctx* c)
{
    return c->line2dOk && c->linearSolver == DXG_LINEAR_SOLVER_ILU_BICGSTAB &&
           (c->iluKernel == DXG_ILU_LANES || (c->iluKernel == DXG_ILU_AUTO && c->line2d));
}

template <class T>
LaneWaveArgs<T> line2dArgs(dxg_ctx* c, const T* A, const T* L, const T* Dinv, const T* rhs, T* v)
{
    LaneWaveArgs<T> w{};
    w.nx = c->pcHost.nx;
    w.ny = c->pcHost.ny;
    w.nz = 1;
    w.N = c->N;
    w.Lf = L;
    w.A = A;
    w.Dinv = Dinv;
    w.rhs = rhs;
    w.v = v;
    w.ks = c->ks.get();
    return w;
}

// The hand-off buffer of the lane sweeps between clusters, all bits set (the kernels' "not
// written yet" pattern); made on first use, refilled after a sweep gave up waiting.
template <class T>
T* laneHandoff(dxg_ctx* c)
{
    const size_t bytes = (size_t)c->lanePlan.ctas * c->pcHost.nx * 64 * 2 * sizeof(T);
    if (c->laneHandoffBytes != bytes) {
        c->laneHandoff.alloc(bytes);
        c->laneHandoffBytes = bytes;
        DXG_CUDA(cudaMemsetAsync(c->laneHandoff.get(), 0xff, bytes, c->stream));
    }
    return reinterpret_cast<T*>(c->laneHandoff.get());
}

template <class T>
LaneWaveArgs<T> laneArgs(dxg_ctx* c, const T* A, const T* L, const T* Dinv, const T* rhs, T* v)
{
    LaneWaveArgs<T> w{};
    w.nx = c->pcHost.nx;
    w.ny = c->pcHost.ny;
    w.nz = c->pcHost.nz;
    w.N = c->N;
    w.nyb = c->lanePlan.nyb;
    w.ctas = c->lanePlan.ctas;
    w.clusterSize = c->lanePlan.clusterSize;
    w.Lf = L;
    w.A = A;
    w.Dinv = Dinv;
    w.rhs = rhs;
    w.v = v;
    w.err = c->singular.get() + 1;
    w.ks = c->ks.get();
    w.handoff = laneHandoff<T>(c);
    w.waitNs = c->waitNs ? c->waitNs : 500000000ull;
    return w;
}

template <class T>
RbArgs<T> rbArgs(dxg_ctx* c, const T* A, T* Dinv)
{
    RbArgs<T> r{};
    r.A = A;
    r.Dinv = Dinv;
    r.nbmask = c->nbmask.get();
    r.N = c->N;
    for (int s = 0; s < 7; ++s) r.off[s] = c->off[s];
    r.nx = (int)c->pcHost.nx;
    r.ny = (int)c->pcHost.ny;
    r.nz = (int)c->pcHost.nz;
    r.singular = c->singular.get();
    r.ks = c->ks.get();
    return r;
}

// Levels of the aggregation AMG in value type T: level 0 is the Jacobian itself (A, the
// inverted pivots in Dinv, the preconditioner's input `in` and output `out`), the coarse
// levels live in one device allocation, made on first use.
template <class T>
std::vector<AmgLevel<T>> amgLevels(dxg_ctx* c, const T* A, T* Dinv, const T* in, T* out)
{
    const int dim = c->dim, b = c->b, bb = c->bb, S = 2 * dim + 1;
    const auto dims = amgLevelDims(dim, (int)c->pcHost.nx, (int)c->pcHost.ny, (int)c->pcHost.nz);
    auto align = [](size_t v) { return (v + 255) & ~(size_t)255; };
    size_t bytes = 2 * align((size_t)c->M * sizeof(T));
    for (const auto& d : dims) {
        const size_t n = (size_t)d[0] * d[1] * d[2];
        bytes += align((size_t)S * n * bb * sizeof(T)) + align(n * bb * sizeof(T)) + 4 * align(n * b * sizeof(T));
    }
    const size_t nLast = dims.empty() ? (size_t)c->N : (size_t)dims.back()[0] * dims.back()[1] * dims.back()[2];
    bytes += align(nLast * b * nLast * b * sizeof(T));   // dense inverse of the last level
    if (c->amgMem.bytes() < bytes) c->amgMem.alloc(bytes);
    unsigned char* p = c->amgMem.get();
    auto take = [&](size_t n) {
        T* q = reinterpret_cast<T*>(p);
        p += align(n * sizeof(T));
        return q;
    };
    std::vector<AmgLevel<T>> L(1 + dims.size());
    L[0].nx = (int)c->pcHost.nx;
    L[0].ny = (int)c->pcHost.ny;
    L[0].nz = dim == 3 ? (int)c->pcHost.nz : 1;
    L[0].N = c->N;
    L[0].A = A;
    L[0].Dinv = Dinv;
    L[0].b = const_cast<T*>(in);
    L[0].x = out;
    L[0].tmp = take((size_t)c->M);
    L[0].r = take((size_t)c->M);
    for (size_t k = 0; k < dims.size(); ++k) {
        AmgLevel<T>& l = L[k + 1];
        l.nx = dims[k][0];
        l.ny = dims[k][1];
        l.nz = dims[k][2];
        l.N = (int64_t)l.nx * l.ny * l.nz;
        l.A = take((size_t)S * l.N * bb);
        l.Dinv = take((size_t)l.N * bb);
        l.b = take((size_t)l.N * b);
        l.x = take((size_t)l.N * b);
        l.tmp = take((size_t)l.N * b);
        l.r = take((size_t)l.N * b);
    }
    for (AmgLevel<T>& l : L) l.sweeps = l.N <= kAmgSmallLevel ? kAmgSmallSweeps : 1;
    L.back().Ainv = take(nLast * b * nLast * b);
    return L;
}

// Launch shape of the wavefront sweeps, chosen once per context by timing: every plan
// that fits (cluster sizes 16..1) applies the preconditioner built by the first
// factorisation to `in` (a scratch read) into `out` (overwritten by the solve that
// follows); the fastest is kept.  Small grids run faster on fewer CTAs (fewer hand-offs
// per level), large ones on more (more SMs per level).
template <class T>
void tuneWavePlan(dxg_ctx* c, const T* A, T* L, T* Dinv, const T* in, T* out)
{
    c->waveTuned = true;
    const std::vector<WavePlan> cand = wavePlanCandidates(c->dim, (int)c->pcHost.nx, (int)c->pcHost.ny,
                                                          (int)c->pcHost.nz, c->b, sizeof(T) == 8);
    const bool lanes = c->lanePlan.ok && (c->iluKernel == DXG_ILU_AUTO || c->iluKernel == DXG_ILU_LANES);
    const bool lines2d = c->line2dOk && (c->iluKernel == DXG_ILU_AUTO || c->iluKernel == DXG_ILU_LANES);
    if (cand.size() < 2 && !lanes && !lines2d) return;
    cudaStream_t st = c->stream;
    cudaEvent_t e0, e1;
    DXG_CUDA(cudaEventCreate(&e0));
    DXG_CUDA(cudaEventCreate(&e1));
    const WavePlan chosen = c->wavePlan;
    WavePlan best = chosen;
    float bestMs = 0.f;
    constexpr int kReps = 3;
    c->waveTuneCount = 0;
    for (const WavePlan& p : cand) {
        c->wavePlan = p;
        WaveArgs<T> w = waveArgs<T>(c, A, L, Dinv, in, out);
        w.ks = nullptr;   // never skip while timing
        launchWaveApply<T>(p, w, w, c->b, st);   // warm-up
        DXG_CUDA(cudaEventRecord(e0, st));
        for (int r = 0; r < kReps; ++r) launchWaveApply<T>(p, w, w, c->b, st);
        DXG_CUDA(cudaEventRecord(e1, st));
        DXG_CUDA(cudaEventSynchronize(e1));
        c->launches += 2 * (1 + kReps);
        float ms = 0.f;
        DXG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        ms /= kReps;
        if (c->waveTuneCount < 5) {
            c->waveTuneMs[c->waveTuneCount] = ms;
            c->waveTuneCtas[c->waveTuneCount] = p.ctas;
            ++c->waveTuneCount;
        }
        if (bestMs == 0.f || ms < bestMs) {
            bestMs = ms;
            best = p;
        }
    }
    // the lane sweeps (3D, 2x2 blocks), when their plan fits: the register form and, where it
    // fits, the shared-memory-ring form (faster where most z hand-offs cross clusters), unless
    // dxg_set_lane_ring fixed one
    if (lanes) {
        LaneWaveArgs<T> lt = laneArgs<T>(c, A, L, Dinv, in, out);
        lt.ks = nullptr;   // never skip while timing
        c->laneFormMs[0] = c->laneFormMs[1] = 0.0;
        float laneBest = 0.f;
        int form = 0;
        for (int f = 0; f < 2; ++f) {
            if (f == 1 && !c->lanePlan.ringOk) continue;
            if (c->laneRingMode != 0 && c->laneRingMode != f + 1) continue;
            c->lanePlan.ring = f;
            launchLaneWaveApply<T>(c->lanePlan, lt, lt, st);   // warm-up
            DXG_CUDA(cudaEventRecord(e0, st));
            for (int r = 0; r < kReps; ++r) launchLaneWaveApply<T>(c->lanePlan, lt, lt, st);
            DXG_CUDA(cudaEventRecord(e1, st));
            DXG_CUDA(cudaEventSynchronize(e1));
            c->launches += 2 * (1 + kReps);
            float ms = 0.f;
            DXG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            ms /= kReps;
            c->laneFormMs[f] = ms;
            if (laneBest == 0.f || ms < laneBest) {
                laneBest = ms;
                form = f;
            }
        }
        c->lanePlan.ring = form;
        c->laneTuneMs = laneBest;
        int flag = 0;
        DXG_CUDA(cudaMemcpy(&flag, c->singular.get() + 1, sizeof(int), cudaMemcpyDeviceToHost));
        c->laneWave = flag == 0 && (bestMs == 0.f || laneBest < bestMs);
    }
    // the one-CTA line sweeps of 2D grids
    if (lines2d) {
        LaneWaveArgs<T> lt = line2dArgs<T>(c, A, L, Dinv, in, out);
        lt.ks = nullptr;   // never skip while timing
        launchTpfaLine2d<T>(lt, lt, c->b, st);   // warm-up
        DXG_CUDA(cudaEventRecord(e0, st));
        for (int r = 0; r < kReps; ++r) launchTpfaLine2d<T>(lt, lt, c->b, st);
        DXG_CUDA(cudaEventRecord(e1, st));
        DXG_CUDA(cudaEventSynchronize(e1));
        c->launches += 2 * (1 + kReps);
        float ms = 0.f;
        DXG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        ms /= kReps;
        c->line2dMs = ms;
        c->line2d = bestMs == 0.f || ms < bestMs;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    c->wavePlan = best;
}

template <class T>
int64_t iluApply(dxg_ctx* c, const IluArgs<T, T>& ia, const T* A, T* L, T* Dinv, const T* d, T* v)
{
    TimedScope ts(c, DXG_KC_ILU_SWEEP, c->bytesSweep * sizeof(T) / 8.0);
    if (c->iluKernel == DXG_ILU_REDBLACK) return launchRbApply<T>(rbArgs<T>(c, A, Dinv), c->b, c->dim, d, v, c->stream);
    if (useLine2d(c)) {
        const LaneWaveArgs<T> la = line2dArgs<T>(c, A, L, Dinv, d, v);
        launchTpfaLine2d<T>(la, la, c->b, c->stream);
        return 2;
    }
    if (useLane(c)) {
        const LaneWaveArgs<T> la = laneArgs<T>(c, A, L, Dinv, d, v);
        launchLaneWaveApply<T>(c->lanePlan, la, la, c->stream);
        return 2;
    }
    if (useWave(c)) {
        launchWaveApply<T>(c->wavePlan, waveArgs<T>(c, A, L, Dinv, d, v), waveArgs<T>(c, A, L, Dinv, d, v), c->b,
                           c->stream);
        return 2;
    }
    return launchIluApply<T, T>(ia, c->levels, c->b, c->dim, d, v, c->stream);
}

template <class T>
IluArgs<T, T> iluArgs(dxg_ctx* c, const T* A, T* L, T* Dinv)
{
    IluArgs<T, T> a{};
    a.A = A;
    a.L = L;
    a.Dinv = Dinv;
    a.nbmask = c->nbmask.get();
    a.perm = c->perm.get();
    a.N = c->N;
    for (int s = 0; s < 7; ++s) a.off[s] = c->off[s];
    a.singular = c->singular.get();
    a.ks = c->ks.get();
    return a;
}

// BiCGSTAB with ILU(0) on the device from x = 0 for rhs (FP64 in device memory):
// Krylov vectors and SpMV in FP64 on the FP64 Jacobian; the ILU(0) preconditioner in
// PT -- FP64 (plain path) or FP32 (mixed precision: FP32 copy of the Jacobian, FP32
// factors and sweeps, fed by FP32 copies of p and r and widened back to FP64).
template <class PT>
dxg_linear_result bicgstab(dxg_ctx* c, const double* rhs, double reduction, int maxit, bool refactor)
{
    constexpr bool mixed = sizeof(PT) == 4;
    cudaStream_t st = c->stream;
    const PT* PA = mixed ? (const PT*)c->Af.get() : (const PT*)c->A.get();
    PT* PL = mixed ? (PT*)c->Lf.get() : (PT*)c->L.get();
    PT* PD = mixed ? (PT*)c->Dinvf.get() : (PT*)c->Dinv.get();
    IluArgs<PT, PT> ia = iluArgs<PT>(c, PA, PL, PD);
    if (refactor) {
        TimedScope factorScope(c, DXG_KC_ILU_FACTOR, c->bytesFactor);
        if (mixed) {
            const int64_t nA = (int64_t)c->slots * c->N * c->bb;
            launchToFloat(ToFloatArgs{c->A.get(), c->Af.get(), nA}, st);
            c->launches += 1;
        }
        DXG_CUDA(cudaMemsetAsync(c->singular.get(), 0, 2 * sizeof(int), st));
        if (c->mpfa) {
            if constexpr (!mixed) {
                launchStencilFactor(stencilArgs(c), st);
                c->launches += 1;
            }
        } else if (c->linearSolver == DXG_LINEAR_SOLVER_AMG_BICGSTAB) {
            // AMG setup: fine pivots, then each coarse operator (with its pivots) from the one above
            std::vector<AmgLevel<PT>> L = amgLevels<PT>(c, PA, PD, nullptr, nullptr);
            launchAmgDiagInv<PT>(L[0], c->dim, c->b, c->singular.get(), st);
            for (size_t k = 1; k < L.size(); ++k) launchAmgCoarsen<PT>(L[k - 1], L[k], c->dim, c->b, c->singular.get(), st);
            launchAmgCoarseInvert<PT>(L.back(), c->dim, c->b, c->singular.get(), st);
            c->launches += (int64_t)L.size() + 1;
        } else if (c->iluKernel == DXG_ILU_REDBLACK) {
            c->launches += launchRbFactor<PT>(rbArgs<PT>(c, PA, PD), c->b, c->dim, st);
        } else if (useWave(c)) {
            // the factor kernel must not skip: give it no Krylov state
            WaveArgs<PT> w = waveArgs<PT>(c, PA, PL, PD, nullptr, nullptr);
            w.ks = nullptr;
            launchWaveFactor<PT>(c->wavePlan, w, c->b, st);
            c->launches += 1;
        } else {
            c->launches += launchIluFactor<PT>(ia, c->levels, c->b, c->dim, st);
        }
    }
    double *x = c->kx.get(), *r = c->kr.get(), *rt = c->krt.get(), *p = c->kp.get(), *v = c->kv.get(),
           *t = c->kt.get(), *y = c->ky.get();
    BicgArgs<double> ba{x, r, rt, p, v, t, y, c->M, c->ks.get(), c->scratch(), nullptr, 0.0, 0, nullptr, nullptr,
                        nullptr};
    // preconditioner operands: FP32 copies of p / r and an FP32 result, or the FP64 vectors
    const PT* pIn = mixed ? (const PT*)c->fp.get() : (const PT*)p;
    const PT* rIn = mixed ? (const PT*)c->fr.get() : (const PT*)r;
    PT* yOut = mixed ? (PT*)c->fy.get() : (PT*)y;
    if (mixed) {
        ba.pLow = c->fp.get();
        ba.rLow = c->fr.get();
        ba.yLow = c->fy.get();
    }
    KrylovState init{};
    init.reduction = reduction;
    init.maxHalf = 2 * maxit;
    DXG_CUDA(cudaMemcpyAsync(c->ks.get(), &init, sizeof(KrylovState), cudaMemcpyHostToDevice, st));
    launchBicgInit<double>(ba, rhs, st);
    c->launches += 1;
    // SpMV: the FP64 Jacobian times the preconditioner output (FP64, or the FP32 output of the
    // mixed form's FP32 preconditioner, widened on load), FP64 row sums, result and dots: the
    // operator is exact in both precisions, so BiCGSTAB converges on the FP64 system and the
    // FP32 factors only shape the preconditioner
    SpmvArgs<double, double, PT> sv{};
    sv.A = c->A.get();
    sv.nbmask = c->nbmask.get();
    sv.N = c->N;
    for (int s = 0; s < 7; ++s) sv.off[s] = c->off[s];
    sv.ks = c->ks.get();
    sv.scratch = c->scratch();
    const bool amg = c->linearSolver == DXG_LINEAR_SOLVER_AMG_BICGSTAB;
    if (refactor && !amg && useWave(c) && !c->waveTuned) tuneWavePlan<PT>(c, PA, PL, PD, pIn, yOut);
    std::vector<AmgLevel<PT>> amgP, amgR;
    if (amg) {
        amgP = amgLevels<PT>(c, PA, PD, pIn, yOut);
        amgR = amgLevels<PT>(c, PA, PD, rIn, yOut);
    }
    const StencilArgs sa = c->mpfa ? stencilArgs(c) : StencilArgs{};
    auto precondition = [&](const PT* in) -> int64_t {
        if constexpr (!mixed) {
            if (c->mpfa) {
                TimedScope ts(c, DXG_KC_ILU_SWEEP, c->bytesSweep);
                switch (mpfaSweep(c, sa)) {
                case 3: launchStencilLane3d(sa, in, yOut, st); return 2;
                case 2: launchStencilLane2d(sa, in, yOut, st); return 2;
                case 1: launchStencilWave2d(sa, in, yOut, st); return 2;
                default: launchStencilApplyLevels(sa, in, yOut, st); return 1;
                }
            }
        }
        if (amg) {
            TimedScope ts(c, DXG_KC_ILU_SWEEP, c->bytesSweep * sizeof(PT) / 8.0);
            return launchAmgVcycle<PT>(in == pIn ? amgP : amgR, c->dim, c->b, c->ks.get(), st);
        }
        return iluApply<PT>(c, ia, PA, PL, PD, in, yOut);
    };
    // one BiCGSTAB iteration; returns the number of kernels it launched
    auto iteration = [&]() -> int64_t {
        int64_t n = 0;
        // the rho step ran in the kernel that closed the previous iteration
        launchBicgUpdateP<double>(ba, st);
        n += 1 + precondition(pIn);
        sv.x = yOut; sv.y = v; sv.w = rt;
        {
            TimedScope ts(c, DXG_KC_SPMV, c->bytesSpmv - (mixed ? 0.5 * c->N * c->b * 8.0 : 0.0));
            if constexpr (!mixed) {
                if (c->mpfa) launchStencilSpmv(sa, yOut, v, rt, 1, st);
                else launchSpmv<double, double, PT>(sv, c->b, c->dim, 1, st);
            } else {
                launchSpmv<double, double, PT>(sv, c->b, c->dim, 1, st);
            }
        }
        launchBicgAxpyNorm<double>(ba, 0, st);
        n += 2 + precondition(rIn);
        sv.x = yOut; sv.y = t; sv.w = r;
        {
            TimedScope ts(c, DXG_KC_SPMV, c->bytesSpmv - (mixed ? 0.5 * c->N * c->b * 8.0 : 0.0));
            if constexpr (!mixed) {
                if (c->mpfa) launchStencilSpmv(sa, yOut, t, r, 2, st);
                else launchSpmv<double, double, PT>(sv, c->b, c->dim, 2, st);
            } else {
                launchSpmv<double, double, PT>(sv, c->b, c->dim, 2, st);
            }
        }
        launchBicgAxpyNorm<double>(ba, 1, st);
        return n + 2;
    };
    // Chunks of iterations between host checks of the Krylov state: replayed from a CUDA
    // graph (captured once per context, precision and preconditioner shape; every
    // argument lives at a fixed device address), or launched one by one while per-kernel
    // timing is on.  Kernels of iterations past the end of the solve return at once.
    const bool graphs = !c->timing;
    const int chunk = graphs ? 8 : 4;
    dxg_ctx::ChunkGraph& G = c->chunkGraph[mixed ? 1 : 0];
    if (graphs) {
        const int key[4] = {c->iluKernel + 16 * c->linearSolver, useLane(c) ? -1 : useWave(c) ? c->wavePlan.ctas : 0,
                            useWave(c) ? c->wavePlan.threads : 0, chunk};
        if (G.exec && !std::equal(key, key + 4, G.key)) {
            cudaGraphExecDestroy(G.exec);
            G.exec = nullptr;
        }
        if (!G.exec) {
            cudaGraph_t graph = nullptr;
            DXG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
            int64_t n = 0;
            try {
                for (int k = 0; k < chunk; ++k) n += iteration();
            } catch (...) {
                cudaStreamEndCapture(st, &graph);
                if (graph) cudaGraphDestroy(graph);
                throw;
            }
            DXG_CUDA(cudaStreamEndCapture(st, &graph));
            const cudaError_t e = cudaGraphInstantiate(&G.exec, graph, 0);
            cudaGraphDestroy(graph);
            DXG_CUDA(e);
            std::copy(key, key + 4, G.key);
            G.launches = n;
        }
    }
    int done = 0;
    while (true) {
        if (graphs) {
            DXG_CUDA(cudaGraphLaunch(G.exec, st));
            c->launches += G.launches;
        } else {
            for (int k = 0; k < chunk; ++k) c->launches += iteration();
        }
        done += chunk;
        DXG_CUDA(cudaMemcpyAsync(c->ksHost, c->ks.get(), sizeof(KrylovState), cudaMemcpyDeviceToHost, st));
        DXG_CUDA(cudaStreamSynchronize(st));
        if (c->ksHost->status != KS_RUNNING || done > maxit + chunk) break;
    }
    int flags[2] = {0, 0};
    DXG_CUDA(cudaMemcpyAsync(flags, c->singular.get(), 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
    DXG_CUDA(cudaStreamSynchronize(st));
    const int sing = flags[0];
    if (flags[1]) {
        // a sweep that gave up may leave hand-off entries written: start the next from scratch
        if (c->laneHandoffBytes)
            DXG_CUDA(cudaMemsetAsync(c->laneHandoff.get(), 0xff, c->laneHandoffBytes, st));
        DXG_CUDA(cudaMemsetAsync(c->singular.get() + 1, 0, sizeof(int), st));
        DXG_CUDA(cudaStreamSynchronize(st));
        throw Error(DXG_ERR_TIMEOUT, "ILU(0) wavefront wait timed out");
    }
    const KrylovState& ks = *c->ksHost;
    dxg_linear_result res{};
    res.converged = ks.status == KS_CONVERGED;
    res.iterations = (ks.halfsteps + 1) / 2;
    res.initial_defect = ks.def0;
    res.final_defect = ks.def;
    res.reduction = ks.def0 > 0 ? ks.def / ks.def0 : 0.0;
    if (sing) {
        res.converged = 0;
        throw Error(DXG_ERR_LINEAR_BREAKDOWN, "singular pivot block in ILU(0)");
    }
    if (ks.status == KS_BREAKDOWN) throw Error(DXG_ERR_LINEAR_BREAKDOWN, "BiCGSTAB breakdown");
    if (ks.status == KS_NAN) throw Error(DXG_ERR_NAN, "non-finite defect in BiCGSTAB");
    return res;
}

// Solves J delta = r into c->delta (FP64), in the context's precision.
dxg_linear_result linearSolve(dxg_ctx* c, double reduction, int maxit)
{
    requireUploaded(c);
    if (!c->haveJac || !c->haveRes) throw Error(DXG_ERR_STATE, "assemble before solving");
    dxg_linear_result res = c->precision == DXG_PRECISION_FP64
                                ? bicgstab<double>(c, c->r.get(), reduction, maxit, !c->haveFactor)
                                : bicgstab<float>(c, c->r.get(), reduction, maxit, !c->haveFactor);
    c->haveFactor = true;
    DXG_CUDA(cudaMemcpyAsync(c->delta.get(), c->kx.get(), c->M * sizeof(double), cudaMemcpyDeviceToDevice,
                             c->stream));
    return res;
}

// ---------------------------------------------------------------- Newton
struct NumericalProblem {};

struct NewtonRun {
    dxg_ctx* c;
    const dxg_newton_params& p;
    dxg_newton_report* rep;
    int numSteps = 0;
    double shift = 0, lastShift = 0, reduction = 0, lastReduction = 1, residualNorm = 0, initialResidual = 0;

    bool converged() const
    {
        if (!p.enable_residual_criterion) return shift <= p.max_relative_shift;
        return shift <= p.max_relative_shift || reduction <= p.residual_reduction;
    }
    bool proceed(bool conv) const
    {
        if (numSteps < p.min_steps) return true;
        else if (conv) return false;
        else if (numSteps >= p.max_steps) return shift * 4.0 < lastShift;
        return true;
    }
    double update(double lambda)
    {
        launchNewtonUpdate(c->uLast.get(), c->delta.get(), c->u.get(), lambda, c->M, c->scratch(), c->scal.get(),
                           c->stream);
        c->launches += 1;
        DXG_CUDA(cudaMemcpyAsync(c->scalHost, c->scal.get(), sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        DXG_CUDA(cudaStreamSynchronize(c->stream));
        return c->scalHost[0];
    }
    void residualReduction()
    {
        assemble(c, false);
        residualNorm = deviceNorm(c, c->r.get());
        reduction = residualNorm / initialResidual;
    }
    // partial reassembly: colors from the accumulated shifts (newtonsolver.hh:565-603)
    void updateColors()
    {
        const double tol = p.max_relative_shift;
        const double minEps = p.reassembly_min_threshold > 0 ? p.reassembly_min_threshold : 1e-1 * tol;
        const double maxEps = p.reassembly_max_threshold > 0 ? p.reassembly_max_threshold : 1e2 * tol;
        const double threshold = std::max(minEps, std::min(maxEps, shift * p.reassembly_shift_weight));
        launchPartialColors(c->uLast.get(), c->u.get(), c->partialDist.get(), c->partialColor.get(), c->N, c->b,
                            threshold, c->stream);
        c->launches += 1;
    }

    // NewtonSolver::solveImpl_ (newtonsolver.hh:976-1072); false on NumericalProblem
    bool run()
    {
        using clk = std::chrono::steady_clock;
        numSteps = 0;
        bool conv = false;
        // newtonBegin: all colors red (resetColors); numeric differentiation only
        if (p.enable_partial_reassembly && c->mpfa)
            throw Error(DXG_ERR_ARG, "partial reassembly is not available for MPFA-O");
        c->partialActive = p.enable_partial_reassembly != 0 && c->method != 3;
        if (c->partialActive) {
            c->partialDist.alloc(c->N);
            c->partialColor.alloc(c->N);
            DXG_CUDA(cudaMemsetAsync(c->partialDist.get(), 0, c->N * sizeof(double), c->stream));
            DXG_CUDA(cudaMemsetAsync(c->partialColor.get(), 1, c->N, c->stream));
        }
        struct Deactivate {
            dxg_ctx* c;
            ~Deactivate() { c->partialActive = false; }
        } deactivate{c};
        DXG_CUDA(cudaMemcpyAsync(c->uLast.get(), c->u.get(), c->M * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
        try {
            while (proceed(conv)) {
                lastShift = shift;
                lastReduction = numSteps == 0 ? 1.0 : reduction;
                if (numSteps > 0)
                    DXG_CUDA(cudaMemcpyAsync(c->uLast.get(), c->u.get(), c->M * sizeof(double),
                                             cudaMemcpyDeviceToDevice, c->stream));
                auto t0 = clk::now();
                assemble(c, true);
                if (numSteps == 0) initialResidual = deviceNorm(c, c->r.get());
                auto t1 = clk::now();
                dxg_linear_result lr{};
                bool lconv = false;
                try {
                    lr = linearSolve(c, p.linear_reduction, p.linear_max_iter);
                    lconv = lr.converged != 0;
                } catch (const Error& e) {
                    if (e.status != DXG_ERR_LINEAR_BREAKDOWN && e.status != DXG_ERR_NAN) throw;
                    lconv = false;
                }
                if (!lconv) throw NumericalProblem{};
                auto t2 = clk::now();
                if (p.use_line_search) {
                    double lambda = 1.0;
                    while (true) {
                        shift = update(lambda);
                        residualReduction();
                        if (reduction < lastReduction || lambda <= p.line_search_min_relaxation) break;
                        lambda *= 0.5;
                    }
                } else {
                    shift = update(1.0);
                    if (p.enable_residual_criterion) residualReduction();
                }
                if (c->partialActive) updateColors();
                auto t3 = clk::now();
                if (numSteps < DXG_MAX_NEWTON_RECORD) {
                    rep->shift[numSteps] = shift;
                    rep->linear_iters[numSteps] = lr.iterations;
                    if (p.record_residual_norms) {
                        if (!(p.use_line_search || p.enable_residual_criterion)) {
                            assemble(c, false);
                            residualNorm = deviceNorm(c, c->r.get());
                        }
                        rep->residual_norm[numSteps] = residualNorm;
                    }
                }
                rep->linear_iterations += lr.iterations;
                rep->time_assemble += std::chrono::duration<double>(t1 - t0).count();
                rep->time_solve += std::chrono::duration<double>(t2 - t1).count();
                rep->time_update += std::chrono::duration<double>(t3 - t2).count();
                ++numSteps;
                conv = converged();
            }
        } catch (const NumericalProblem&) {
            return false;
        }
        return converged();
    }
};

}  // namespace

namespace dxg {
template <class T>
std::vector<AmgLevel<T>> amgLevelsOf(dxg_ctx* c, const T* A, T* Dinv, const T* in, T* out)
{
    return amgLevels<T>(c, A, Dinv, in, out);
}
template std::vector<AmgLevel<double>> amgLevelsOf<double>(dxg_ctx*, const double*, double*, const double*, double*);
template std::vector<AmgLevel<float>> amgLevelsOf<float>(dxg_ctx*, const float*, float*, const float*, float*);
}  // namespace dxg

// ================================================================ C ABI
extern "C" {

int64_t dxg_num_boundary_faces(const dxg_problem_desc* d)
{
    if (!d || (d->dim != 2 && d->dim != 3)) return -1;
    int64_t n[3];
    for (int a = 0; a < 3; ++a) n[a] = a < d->dim ? d->cells[a] : 1;
    int64_t total = 0;
    for (int a = 0; a < d->dim; ++a) {
        int64_t cnt = 1;
        for (int k = 0; k < d->dim; ++k)
            if (k != a) cnt *= n[k];
        total += 2 * cnt;
    }
    return total;
}

int dxg_ctx_create(dxg_ctx** out, int device)
{
    if (!out) return DXG_ERR_ARG;
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        g_createError = std::string("no CUDA device: ") + cudaGetErrorString(e);
        return DXG_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= ndev) {
        g_createError = "device index out of range";
        return DXG_ERR_ARG;
    }
    auto* c = new dxg_ctx();
    int st = guarded(c, [&] {
        c->device = device;
        DXG_CUDA(cudaSetDevice(device));
        DXG_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
        // one pinned allocation for the Krylov state and the scalars read back
        const size_t ksBytes = (sizeof(KrylovState) + 63) & ~(size_t)63;
        void* pinned = nullptr;
        DXG_CUDA(cudaMallocHost(&pinned, ksBytes + 4 * sizeof(double)));
        c->ksHost = static_cast<KrylovState*>(pinned);
        c->scalHost = reinterpret_cast<double*>(static_cast<unsigned char*>(pinned) + ksBytes);
        return DXG_OK;
    });
    if (st != DXG_OK) {
        g_createError = c->err;
        delete c;
        return st;
    }
    *out = c;
    return DXG_OK;
}

int dxg_ctx_destroy(dxg_ctx* c)
{
    if (!c) return DXG_ERR_ARG;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (auto& t : c->pending) {
        cudaEventDestroy(t.start);
        cudaEventDestroy(t.stop);
    }
    for (auto e : c->eventPool) cudaEventDestroy(e);
    c->dropGraphs();
    if (c->ksHost) cudaFreeHost(c->ksHost);   // also holds scalHost
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return DXG_OK;
}

const char* dxg_last_error(const dxg_ctx* c) { return c ? c->err.c_str() : g_createError.c_str(); }

int dxg_set_precision(dxg_ctx* c, int precision)
{
    if (!c || (precision != DXG_PRECISION_FP64 && precision != DXG_PRECISION_MIXED)) return DXG_ERR_ARG;
    if (c->uploaded) {
        c->err = "precision must be set before dxg_problem_upload";
        return DXG_ERR_STATE;
    }
    c->precision = precision;
    return DXG_OK;
}

int dxg_problem_upload(dxg_ctx* c, const dxg_problem_desc* d)
{
    if (!c) return DXG_ERR_ARG;
    return guarded(c, [&] {
        DXG_CUDA(cudaSetDevice(c->device));
        tabulate(c, d);
        return DXG_OK;
    });
}

int dxg_sizes(const dxg_ctx* c, int64_t* n, int32_t* b, int64_t* nnzb)
{
    if (!c || !c->uploaded) return DXG_ERR_STATE;
    if (n) *n = c->N;
    if (b) *b = c->b;
    if (nnzb) *nnzb = c->nnzb;
    return DXG_OK;
}

static int copyIn(dxg_ctx* c, DevBuf<double>& dst, const double* src)
{
    return guarded(c, [&] {
        requireUploaded(c);
        if (!src) throw Error(DXG_ERR_ARG, "null host buffer");
        DXG_CUDA(cudaMemcpyAsync(dst.get(), src, c->M * sizeof(double), cudaMemcpyHostToDevice, c->stream));
        DXG_CUDA(cudaStreamSynchronize(c->stream));
        return DXG_OK;
    });
}
static int copyOut(dxg_ctx* c, const double* src, double* dst)
{
    return guarded(c, [&] {
        requireUploaded(c);
        if (!dst) throw Error(DXG_ERR_ARG, "null host buffer");
        DXG_CUDA(cudaMemcpyAsync(dst, src, c->M * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        DXG_CUDA(cudaStreamSynchronize(c->stream));
        return DXG_OK;
    });
}

int dxg_set_solution(dxg_ctx* c, const double* u)
{
    if (!c) return DXG_ERR_ARG;
    const int st = copyIn(c, c->u, u);
    if (st == DXG_OK) c->haveJac = c->haveRes = c->haveFactor = false;
    return st;
}
int dxg_get_solution(dxg_ctx* c, double* u) { return c ? copyOut(c, c->u.get(), u) : DXG_ERR_ARG; }
int dxg_set_prev_solution(dxg_ctx* c, const double* up)
{
    if (!c) return DXG_ERR_ARG;
    const int st = copyIn(c, c->uprev, up);
    if (st == DXG_OK) {
        c->havePrev = true;
        c->stPrevValid = false;
    }
    return st;
}
int dxg_set_time_step(dxg_ctx* c, double dt)
{
    if (!c) return DXG_ERR_ARG;
    c->dt = dt > 0.0 ? dt : 0.0;
    c->haveJac = c->haveRes = c->haveFactor = false;
    return DXG_OK;
}

int dxg_assemble_jacobian_and_residual(dxg_ctx* c)
{
    if (!c) return DXG_ERR_ARG;
    return guarded(c, [&] {
        assemble(c, true);
        DXG_CUDA(cudaStreamSynchronize(c->stream));
        return DXG_OK;
    });
}
int dxg_assemble_residual(dxg_ctx* c)
{
    if (!c) return DXG_ERR_ARG;
    return guarded(c, [&] {
        assemble(c, false);
        DXG_CUDA(cudaStreamSynchronize(c->stream));
        return DXG_OK;
    });
}
int dxg_get_residual(dxg_ctx* c, double* r) { return c ? copyOut(c, c->r.get(), r) : DXG_ERR_ARG; }
int dxg_get_update(dxg_ctx* c, double* d) { return c ? copyOut(c, c->delta.get(), d) : DXG_ERR_ARG; }

int dxg_get_jacobian(dxg_ctx* c, int64_t* row_ptr, int32_t* col_idx, double* values)
{
    if (!c) return DXG_ERR_ARG;
    return guarded(c, [&] {
        requireUploaded(c);
        if (!c->haveJac) throw Error(DXG_ERR_STATE, "no Jacobian assembled");
        std::vector<double> h((size_t)c->slots * c->N * c->bb);
        DXG_CUDA(cudaMemcpyAsync(h.data(), c->A.get(), h.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        DXG_CUDA(cudaStreamSynchronize(c->stream));
        int64_t k = 0;
        for (int64_t i = 0; i < c->N; ++i) {
            if (row_ptr) row_ptr[i] = k;
            for (int s = 0; s < c->slots; ++s) {
                if (!slotInPattern(c, i, s)) continue;
                if (col_idx) col_idx[k] = (int32_t)(i + slotOffset(c, s));
                if (values)
                    std::memcpy(values + k * c->bb, h.data() + ((size_t)s * c->N + i) * c->bb, sizeof(double) * c->bb);
                ++k;
            }
        }
        if (row_ptr) row_ptr[c->N] = k;
        return DXG_OK;
    });
}

int dxg_set_linear_system(dxg_ctx* c, const int64_t* row_ptr, const int32_t* col_idx, const double* values,
                          const double* rhs)
{
    if (!c) return DXG_ERR_ARG;
    return guarded(c, [&] {
        requireUploaded(c);
        if (!row_ptr || !col_idx || !values || !rhs) throw Error(DXG_ERR_ARG, "null buffer");
        std::vector<double> h((size_t)c->slots * c->N * c->bb, 0.0);
        for (int64_t i = 0; i < c->N; ++i)
            for (int64_t k = row_ptr[i]; k < row_ptr[i + 1]; ++k) {
                const int64_t dc = (int64_t)col_idx[k] - i;
                int slot = -1;
                for (int s = 0; s < c->slots; ++s)
                    if (slotOffset(c, s) == dc && slotInPattern(c, i, s)) slot = s;
                if (slot < 0) throw Error(DXG_ERR_ARG, "entry outside the stencil pattern");
                std::memcpy(h.data() + ((size_t)slot * c->N + i) * c->bb, values + k * c->bb, sizeof(double) * c->bb);
            }
        DXG_CUDA(cudaMemcpyAsync(c->A.get(), h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
        DXG_CUDA(cudaMemcpyAsync(c->r.get(), rhs, c->M * sizeof(double), cudaMemcpyHostToDevice, c->stream));
        DXG_CUDA(cudaStreamSynchronize(c->stream));
        c->haveJac = c->haveRes = true;
        c->haveFactor = false;
        return DXG_OK;
    });
}

int dxg_linear_solve(dxg_ctx* c, double reduction, int32_t max_iter, dxg_linear_result* res)
{
    if (!c) return DXG_ERR_ARG;
    return guarded(c, [&] {
        DXG_CUDA(cudaSetDevice(c->device));
        dxg_linear_result r = linearSolve(c, reduction, max_iter);
        if (res) *res = r;
        return r.converged ? DXG_OK : DXG_ERR_LINEAR_NOT_CONVERGED;
    });
}

int dxg_residual_norm(dxg_ctx* c, double* norm)
{
    if (!c || !norm) return DXG_ERR_ARG;
    return guarded(c, [&] {
        requireUploaded(c);
        if (!c->haveRes) throw Error(DXG_ERR_STATE, "no residual assembled");
        *norm = deviceNorm(c, c->r.get());
        return DXG_OK;
    });
}

void dxg_newton_default_params(dxg_newton_params* p)
{
    if (!p) return;
    p->max_relative_shift = 1e-8;
    p->min_steps = 2;
    p->max_steps = 18;
    p->target_steps = 10;
    p->use_line_search = 0;
    p->line_search_min_relaxation = 0.125;
    p->enable_residual_criterion = 0;
    p->residual_reduction = 1e-5;
    p->max_time_step_divisions = 10;
    p->retry_time_step_reduction = 0.5;
    p->linear_reduction = 1e-6;
    p->linear_max_iter = 250;
    p->record_residual_norms = 0;
    p->enable_partial_reassembly = 0;
    p->reassembly_min_threshold = 0.0;
    p->reassembly_max_threshold = 0.0;
    p->reassembly_shift_weight = 1e-3;
}

int dxg_newton_solve(dxg_ctx* c, double dt, const dxg_newton_params* params, dxg_newton_report* report)
{
    if (!c) return DXG_ERR_ARG;
    return guarded(c, [&] {
        requireUploaded(c);
        DXG_CUDA(cudaSetDevice(c->device));
        dxg_newton_params p;
        if (params) p = *params;
        else dxg_newton_default_params(&p);
        dxg_newton_report local{};
        dxg_newton_report* rep = report ? report : &local;
        std::memset(rep, 0, sizeof(*rep));
        const bool transient = dt > 0.0;
        if (transient && !c->havePrev) throw Error(DXG_ERR_STATE, "transient solve needs the previous solution");
        const int divisions = transient ? p.max_time_step_divisions : 0;
        int wasted = 0;
        for (int i = 0; i <= divisions; ++i) {
            c->dt = transient ? dt : 0.0;
            dxg_newton_report attempt{};
            NewtonRun run{c, p, &attempt};
            const bool conv = run.run();
            attempt.iterations = run.numSteps;
            attempt.initial_residual = run.initialResidual;
            attempt.dt_used = dt;
            attempt.converged = conv;
            attempt.time_step_divisions = i;
            attempt.wasted_iterations = wasted;
            c->lastNewtonSteps = run.numSteps;
            *rep = attempt;
            if (conv) return DXG_OK;
            wasted += run.numSteps;
            rep->wasted_iterations = wasted;
            if (transient) {
                // reset to the previous solution and retry with a reduced time step
                DXG_CUDA(cudaMemcpyAsync(c->u.get(), c->uprev.get(), c->M * sizeof(double), cudaMemcpyDeviceToDevice,
                                         c->stream));
                dt *= p.retry_time_step_reduction;
            }
        }
        DXG_CUDA(cudaStreamSynchronize(c->stream));
        c->err = "Newton solver did not converge";
        return DXG_ERR_NEWTON_NOT_CONVERGED;
    });
}

double dxg_suggest_time_step(const dxg_ctx* c, double oldTimeStep, const dxg_newton_params* params)
{
    dxg_newton_params p;
    if (params) p = *params;
    else dxg_newton_default_params(&p);
    const int numSteps = c ? c->lastNewtonSteps : p.target_steps;
    if (numSteps > p.target_steps) {
        const double percent = double(numSteps - p.target_steps) / p.target_steps;
        return oldTimeStep / (1.0 + percent);
    }
    const double percent = double(p.target_steps - numSteps) / p.target_steps;
    return oldTimeStep * (1.0 + percent / 1.2);
}

int dxg_advance_time_step(dxg_ctx* c)
{
    if (!c) return DXG_ERR_ARG;
    return guarded(c, [&] {
        requireUploaded(c);
        DXG_CUDA(cudaMemcpyAsync(c->uprev.get(), c->u.get(), c->M * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
        DXG_CUDA(cudaStreamSynchronize(c->stream));
        c->havePrev = true;
        c->stPrevValid = false;
        return DXG_OK;
    });
}

int dxg_set_ilu_kernel(dxg_ctx* c, int kind)
{
    if (!c || kind < DXG_ILU_AUTO || kind > DXG_ILU_LANES) return DXG_ERR_ARG;
    if (c->mpfa) {
        // levels / wavefront (one-CTA line sweeps) / lanes (cluster line sweeps) / auto;
        // the kinds a grid does not fit fall back to the level kernel
        if (kind == DXG_ILU_REDBLACK) {
            c->err = "MPFA-O contexts use the natural-order ILU(0) of their stencil";
            return DXG_ERR_ARG;
        }
        c->iluKernel = kind;
        return DXG_OK;
    }
    if (kind == DXG_ILU_WAVEFRONT && c->uploaded && !c->wavePlan.ok) {
        c->err = "no wavefront plan fits this grid";
        return DXG_ERR_ARG;
    }
    if (kind == DXG_ILU_LANES && c->uploaded && !c->lanePlan.ok && !c->line2dOk) {
        c->err = "the lane sweeps need a 3D grid of 2x2 blocks or a 2D grid of up to 512 lines that fits them";
        return DXG_ERR_ARG;
    }
    c->iluKernel = kind;
    c->haveFactor = false;
    return DXG_OK;
}

int dxg_set_lane_ring(dxg_ctx* c, int form)
{
    if (!c || form < 0 || form > 2) return DXG_ERR_ARG;
    if (form == 2 && c->uploaded && !c->lanePlan.ringOk) {
        c->err = "the shared-memory-ring form of the lane sweeps does not fit this grid";
        return DXG_ERR_ARG;
    }
    c->laneRingMode = form;
    // time (or fix) the form again at the next factorisation; captured chunks hold the old one
    c->waveTuned = false;
    c->haveFactor = false;
    c->dropGraphs();
    return DXG_OK;
}

int dxg_set_wait_limit(dxg_ctx* c, double seconds)
{
    if (!c || !(seconds > 0.0) || seconds > 60.0) return DXG_ERR_ARG;
    c->waitNs = (unsigned long long)(seconds * 1e9);
    c->dropGraphs();   // the captured chunks hold the old limit in their arguments
    return DXG_OK;
}

int dxg_set_linear_solver(dxg_ctx* c, int kind)
{
    if (!c || (kind != DXG_LINEAR_SOLVER_ILU_BICGSTAB && kind != DXG_LINEAR_SOLVER_AMG_BICGSTAB)) return DXG_ERR_ARG;
    if (c->mpfa && kind != DXG_LINEAR_SOLVER_ILU_BICGSTAB) {
        c->err = "MPFA-O contexts solve with ILU(0)-BiCGSTAB";
        return DXG_ERR_ARG;
    }
    c->linearSolver = kind;
    c->haveFactor = false;
    return DXG_OK;
}

int dxg_describe(const dxg_ctx* c, char* buf, int64_t len)
{
    if (!c || !buf || len <= 0) return DXG_ERR_ARG;
    std::string out;
    if (!c->uploaded) out = "no problem uploaded";
    else if (c->mpfa) {
        StencilArgs sa{};
        sa.b = c->b;
        sa.S = c->mpLayout.S;
        sa.nx = c->pcHost.nx;
        sa.ny = c->pcHost.ny;
        sa.nz = c->pcHost.nz;
        const int k = mpfaSweep(c, sa);
        out = std::string("MPFA-O, ") + std::to_string(c->mpLayout.S) + "-point stencil; ILU(0): natural order, " +
              (k == 3   ? "line sweeps (one lane per grid line and block row, levels x+2y+4z), one z-plane "
                          "per CTA over a cluster of " +
                            std::to_string(sa.nz) + " CTAs"
               : k == 2 ? "line sweeps (one thread per grid line, levels x+2y) over a cluster of " +
                            std::to_string((sa.ny + 127) / 128) + " CTAs"
               : k == 1 ? "line sweeps (one thread per grid line, levels x+2y) in one CTA"
                        : "hyperplanes x+2y+4z level by level in one CTA");
    }
    else if (c->linearSolver == DXG_LINEAR_SOLVER_AMG_BICGSTAB)
        out = "AMG-BiCGSTAB: " + std::to_string(amgLevelDims(c->dim, (int)c->pcHost.nx, (int)c->pcHost.ny,
                                                               (int)c->pcHost.nz).size() + 1) +
              " levels of 2x2(x2) aggregation, damped block-Jacobi smoothing";
    else if (c->iluKernel == DXG_ILU_REDBLACK) out = "ILU(0): red-black ordering, two parallel passes per sweep";
    else if (useLine2d(c)) {
        out = "ILU(0): line sweeps in one CTA (one thread per grid line, levels x+y)";
        if (c->line2dMs > 0) {
            char tmp[96];
            std::snprintf(tmp, sizeof tmp, ", tuned (ms per apply: line sweeps %.3f", c->line2dMs);
            out += tmp;
            for (int k = 0; k < c->waveTuneCount; ++k) {
                std::snprintf(tmp, sizeof tmp, ", cluster wavefront %d CTAs %.3f", c->waveTuneCtas[k], c->waveTuneMs[k]);
                out += tmp;
            }
            out += ")";
        }
    }
    else if (useLane(c)) {
        const LanePlan& p = c->lanePlan;
        char tmp[200];
        std::snprintf(tmp, sizeof tmp, "ILU(0): lane wavefront (%s), %d CTAs of 128 threads in clusters of %d",
                      p.ring == 1 ? "shared-memory ring" : "register ring", p.ctas, p.clusterSize);
        out = tmp;
        if (c->laneTuneMs > 0) {
            std::snprintf(tmp, sizeof tmp, ", tuned (ms per apply: lanes %.3f", c->laneTuneMs);
            out += tmp;
            if (c->laneFormMs[0] > 0 && c->laneFormMs[1] > 0) {
                std::snprintf(tmp, sizeof tmp, " (register ring %.3f, shared-memory ring %.3f)", c->laneFormMs[0],
                              c->laneFormMs[1]);
                out += tmp;
            }
            for (int k = 0; k < c->waveTuneCount; ++k) {
                std::snprintf(tmp, sizeof tmp, ", cluster wavefront %d CTAs %.3f", c->waveTuneCtas[k], c->waveTuneMs[k]);
                out += tmp;
            }
            out += ")";
        }
    } else if (!useWave(c)) out = "ILU(0): level-scheduled kernels";
    else {
        const WavePlan& p = c->wavePlan;
        out = "ILU(0): wavefront, cluster " + std::to_string(p.ctas) + " x " + std::to_string(p.threads) +
              " threads";
        if (c->waveTuned && c->waveTuneCount > 0) {
            out += ", tuned (ms per apply:";
            char tmp[64];
            for (int k = 0; k < c->waveTuneCount; ++k) {
                std::snprintf(tmp, sizeof tmp, " %d CTAs %.3f", c->waveTuneCtas[k], c->waveTuneMs[k]);
                out += tmp;
            }
            if (c->laneTuneMs > 0) {
                std::snprintf(tmp, sizeof tmp, "; lane wavefront %.3f", c->laneTuneMs);
                out += tmp;
            }
            out += ")";
        }
    }
    std::strncpy(buf, out.c_str(), (size_t)len - 1);
    buf[len - 1] = 0;
    return DXG_OK;
}

int64_t dxg_kernel_launch_count(const dxg_ctx* c) { return c ? c->launches : -1; }

void* dxg_stream_handle(const dxg_ctx* c) { return c ? (void*)c->stream : nullptr; }

int dxg_set_kernel_timing(dxg_ctx* c, int enable)
{
    if (!c) return DXG_ERR_ARG;
    return guarded(c, [&] {
        resolveTimings(c);
        c->timing = enable != 0;
        for (int k = 0; k < DXG_KC_COUNT; ++k) {
            c->kcLaunches[k] = 0;
            c->kcMs[k] = 0;
            c->kcBytes[k] = 0;
        }
        return DXG_OK;
    });
}

int dxg_get_kernel_timing(dxg_ctx* c, int kc, int64_t* launches, double* ms, double* bytes)
{
    if (!c || kc < 0 || kc >= DXG_KC_COUNT) return DXG_ERR_ARG;
    return guarded(c, [&] {
        resolveTimings(c);
        if (launches) *launches = c->kcLaunches[kc];
        if (ms) *ms = c->kcMs[kc];
        if (bytes) *bytes = c->kcBytes[kc];
        return DXG_OK;
    });
}

int dxg_selftest_bounded_wait(int device, int32_t kind, int64_t limit_ns, int32_t* kernel_status,
                              double* waited_ms)
{
    if (!kernel_status || (kind != 0 && kind != 1) || limit_ns <= 0 || limit_ns > 1000000000LL) return DXG_ERR_ARG;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return DXG_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= count || cudaSetDevice(device) != cudaSuccess) return DXG_ERR_ARG;
    int ks = -1;
    const int rc = runBoundedWaitSelfTest(kind, limit_ns, &ks, waited_ms);
    *kernel_status = ks;
    return rc;
}

int dxg_fp64_fma_rate(int device, double* tflops)
{
    if (!tflops) return DXG_ERR_ARG;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return DXG_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= count || cudaSetDevice(device) != cudaSuccess) return DXG_ERR_ARG;
    return dxg::runFp64Rate(tflops);
}

int dxg_device_pow(int device, const double* x, const double* y, double* out, int64_t n)
{
    if (n < 0 || (n > 0 && (!x || !y || !out))) return DXG_ERR_ARG;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return DXG_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= count || cudaSetDevice(device) != cudaSuccess) return DXG_ERR_ARG;
    return dxg::runDevicePow(x, y, out, n);
}

int dxg_sync(dxg_ctx* c)
{
    if (!c) return DXG_ERR_ARG;
    return guarded(c, [&] {
        DXG_CUDA(cudaStreamSynchronize(c->stream));
        DXG_CUDA(cudaGetLastError());
        return DXG_OK;
    });
}

}  // extern "C"
