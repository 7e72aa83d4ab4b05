// stencillane.cu -- ILU(0) sweeps of the 3D 27-point MPFA-O stencil (1x1 or 2x2 blocks) over a
// thread-block cluster: one z-plane per CTA, one lane per grid line and block row.
//
// Natural order: cell (x, y, z) sits on level L = x + 2y + 4z, and its 13 lower neighbours (slots
// 0..12: the 9 cells of plane z-1 around it, then (x-1, y-1), (x, y-1), (x+1, y-1) and (x-1, y))
// lie on levels L-7 .. L-1.  Plane z is CTA z of one cluster (nz <= 16); in it, line y handles
// cell x = s - 2y at step s, so the plane's step s is level s + 4z.  The 13 terms enter the
// accumulator in ascending slot order, the order of the level-by-level kernel
// (stencilApplyKernel / stencilApply2Kernel), and with the same explicit FMAs, so both give the
// same bits.  The backward sweep is the forward one in mirrored coordinates (slot q of the
// sweep is matrix slot 26 - q, entered in descending matrix-slot order as the level kernel
// does), followed by the pivot-inverse product.
// Sources of the terms:
//   * slots 0..8 (plane z-1): the CTA of the plane before writes every result into this CTA's
//     shared-memory copy of its plane by a remote store; the entries start all ones (a NaN no
//     sweep produces) and are polled until written;
//   * slots 9..11 (line y-1's cells x-1, x, x+1, computed 3, 2, 1 steps before): the last three
//     results of line y-1's lanes, by shuffles; the first line of a warp reads them from a
//     per-step history that the previous warp's last line writes into shared memory;
//   * slot 12 (cell x-1 of the same line): the lane's own previous result.
// A cell's factor rows, right-hand side (backward: and pivot-inverse row) and slot mask are
// loaded PF steps ahead into registers; entries of slots outside the cell's pattern enter as
// zero times zero, which leaves the accumulator's bits unchanged.
//
// On GB300 a dependent FP64 FMA takes ~64 cycles, so a step costs about 13 B such FMAs per lane
// against the 13 dependent levels a level-by-level CTA barrier would wait for.  Every wait is
// bounded (the context's wait limit); one that expires records DXG_ERR_TIMEOUT and stops the
// CTA's sweep (its later waits return at once), and all CTAs leave through a final cluster
// barrier, so no CTA exits while another may still write into its shared memory.
#include <cooperative_groups.h>

#include "common.cuh"
#include "linalg_kernels.cuh"

namespace cg = cooperative_groups;

namespace dxg {
namespace {

constexpr unsigned long long kSlDefaultWaitNs = 500000000ull;
constexpr size_t kSlSmemLimit = 200 * 1024;
constexpr int kSlMaxThreads = 256;
constexpr int kSlPf = 1;

template <int B>
struct SlVec;
template <>
struct SlVec<1> {
    using type = double;
};
template <>
struct SlVec<2> {
    using type = double2;
};

__device__ __forceinline__ unsigned long long slTimer()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ uint32_t slSmem(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ uint32_t slMapa(uint32_t addr, int rank)
{
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
    return r;
}
__device__ __forceinline__ void slStCluster(uint32_t dst, double v)
{
    asm volatile("st.relaxed.cluster.shared::cluster.f64 [%0], %1;" ::"r"(dst), "d"(v));
}
__device__ __forceinline__ bool slEmpty(double v) { return __double_as_longlong(v) == -1ll; }
__device__ __forceinline__ double slEmptyValue() { return __longlong_as_double(-1ll); }

template <int B>
__device__ __forceinline__ typename SlVec<B>::type slZero()
{
    if constexpr (B == 1) return 0.0;
    else return make_double2(0.0, 0.0);
}
template <int B>
__device__ __forceinline__ bool slEmptyV(typename SlVec<B>::type v)
{
    if constexpr (B == 1) return slEmpty(v);
    else return slEmpty(v.x) || slEmpty(v.y);
}
// relaxed load of both rows of an entry of this CTA's shared memory (each half single-copy atomic)
template <int B>
__device__ __forceinline__ typename SlVec<B>::type slLd(const double* p)
{
    typename SlVec<B>::type v;
    if constexpr (B == 1)
        asm volatile("ld.relaxed.cluster.shared::cta.f64 %0, [%1];" : "=d"(v) : "r"(slSmem(p)));
    else
        asm volatile("ld.relaxed.cluster.shared::cta.v2.f64 {%0, %1}, [%2];" : "=d"(v.x), "=d"(v.y) : "r"(slSmem(p)));
    return v;
}
// read-only loads of the records
template <int B>
__device__ __forceinline__ typename SlVec<B>::type slLdg(const double* p)
{
    if constexpr (B == 1) return __ldg(p);
    else return __ldg(reinterpret_cast<const double2*>(p));
}

// The slow path of a poll: waits, bounded, until the entry at p holds no empty half, and
// returns it; zeros once the CTA's sweep has stopped or when the wait expires (which records
// DXG_ERR_TIMEOUT and stops the CTA's sweep).
template <int B>
__device__ __noinline__ typename SlVec<B>::type slWait(const double* p, int* stop, int* err, unsigned long long waitNs)
{
    const unsigned long long deadline = slTimer() + waitNs;
    for (;;) {
        const typename SlVec<B>::type v = slLd<B>(p);
        if (!slEmptyV<B>(v)) return v;
        if (*(volatile int*)stop) break;
        if (slTimer() > deadline) {
            atomicExch(err, DXG_ERR_TIMEOUT);
            *(volatile int*)stop = 1;
            break;
        }
    }
    return slZero<B>();
}

// shared memory: the plane before [nx][ny][B] (sweep coordinates), then the per-step histories
// of each warp's last line [warps - 1][steps][B]
__host__ __device__ inline size_t slSmemBytes(int nx, int ny, int b)
{
    const int warps = (ny * b + 31) / 32;
    const int steps = (nx - 1) + 2 * (ny - 1) + 1;
    return ((size_t)nx * ny * b + (size_t)(warps - 1) * steps * b) * sizeof(double);
}

// term q of the sweep (ascending): offsets in sweep coordinates
__device__ __forceinline__ int slOx(int q) { return q < 9 ? q % 3 - 1 : (q == 12 ? -1 : q - 10); }
__device__ __forceinline__ int slOy(int q) { return q < 9 ? q / 3 - 1 : (q == 12 ? 0 : -1); }

template <int B, int DIR, int PF>
__global__ void __launch_bounds__(kSlMaxThreads) stencilLane3dKernel(StencilArgs a, const double* __restrict__ d,
                                                                     double* __restrict__ v)
{
    using V = typename SlVec<B>::type;
    constexpr int LPW = 32 / B;   // lines per warp
    extern __shared__ __align__(16) unsigned char slRaw[];
    __shared__ int stopFlag;
    cg::cluster_group cluster = cg::this_cluster();
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const int64_t N = a.N;
    const int nWarps = (ny * B + 31) / 32;
    const int nSteps = (nx - 1) + 2 * (ny - 1) + 1;
    double* zin = reinterpret_cast<double*>(slRaw);    // [nx][ny][B]
    double* ybuf = zin + (size_t)nx * ny * B;          // [nWarps - 1][nSteps][B]
    const int sz = (int)blockIdx.x;                    // the grid is one cluster
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int j = t / B, r = t % B;
    const bool lineOk = j < ny;
    const int z = DIR > 0 ? sz : nz - 1 - sz;
    const int y = DIR > 0 ? j : ny - 1 - j;
    const int64_t lineBase = lineOk ? ((int64_t)z * ny + y) * nx : 0;

    if (sz > 0)
        for (int k = t; k < nx * ny * B; k += blockDim.x) zin[k] = slEmptyValue();
    for (int k = t; k < (nWarps - 1) * nSteps * B; k += blockDim.x) ybuf[k] = slEmptyValue();
    if (t == 0) stopFlag = 0;
    cluster.sync();
    const bool skip = a.ks && a.ks->status != KS_RUNNING;
    const unsigned long long waitNs = a.waitNs ? a.waitNs : kSlDefaultWaitNs;

    const bool hasDown = sz + 1 < nz;
    const uint32_t zinDown = hasDown ? slMapa(slSmem(zin), sz + 1) : 0u;   // + ((x * ny + j) * B + r) * 8
    const int jw = j - warp * LPW;                                         // line within the warp
    const bool firstOfWarp = lineOk && jw == 0 && warp > 0;                // line j-1 is in the warp before
    const bool lastOfWarp = lineOk && jw == LPW - 1 && warp < nWarps - 1;  // publishes for the warp after
    const double* yIn = ybuf + (size_t)(warp > 0 ? warp - 1 : 0) * nSteps * B;
    const uint32_t yOut = slSmem(ybuf + (size_t)warp * nSteps * B + r);    // + step * B * 8
    const double* LUr = a.LU + (B == 2 ? 2 * r : 0);
    const double* DIr = a.Dinv + (B == 2 ? 2 * r : 0);
    const double* src = DIR > 0 ? d : v;

    // the register ring: records of step s in entry s % PF
    V rm[PF][13];
    V rD[PF];
    double rv[PF];
    uint32_t rk[PF];
    auto load = [&](int s, int k) {
        const int sx = s - 2 * j;
        const bool act = lineOk && sx >= 0 && sx < nx;
        const int64_t i = lineBase + (DIR > 0 ? sx : nx - 1 - sx);
        rk[k] = act ? __ldg(a.mask + i) : 0u;
#pragma unroll
        for (int q = 0; q < 13; ++q) {
            const int sm = DIR > 0 ? q : 26 - q;
            rm[k][q] = act ? slLdg<B>(LUr + ((int64_t)sm * N + i) * (B * B)) : slZero<B>();
        }
        rv[k] = act ? __ldg(src + i * B + r) : 0.0;
        if (DIR < 0) rD[k] = act ? slLdg<B>(DIr + i * (B * B)) : slZero<B>();
    };

    const bool works = !skip && (warp * LPW < ny);
    if (works) {
        // results of this lane's line 1, 2 and 3 steps before
        double h1 = 0.0, h2 = 0.0, h3 = 0.0;
#pragma unroll
        for (int k = 0; k < PF; ++k) load(k, k);
        for (int s0 = 0; s0 < nSteps; s0 += PF) {
#pragma unroll
            for (int k = 0; k < PF; ++k) {
                const int s = s0 + k;
                const int sx = s - 2 * j;
                const bool act = lineOk && sx >= 0 && sx < nx;
                V m[13];
#pragma unroll
                for (int q = 0; q < 13; ++q) m[q] = rm[k][q];
                const double rhs = rv[k];
                V Dr = rD[k];
                const uint32_t msk = rk[k];
                load(s + PF, k);
                // the plane before: loads issued ahead of the chain, checked where used
                V zv[9];
#pragma unroll
                for (int q = 0; q < 9; ++q) {
                    const int sm = DIR > 0 ? q : 26 - q;
                    const bool ok = act && ((msk >> sm) & 1u);
                    zv[q] = ok ? slLd<B>(zin + ((size_t)(sx + slOx(q)) * ny + (j + slOy(q))) * B) : slZero<B>();
                }
                // line j-1's results of 3, 2, 1 steps before (its cells x-1, x, x+1) and this
                // line's previous cell, both rows
                V n1, n2, n3, o;
                if constexpr (B == 1) {
                    n1 = __shfl_up_sync(0xffffffffu, h1, 1);
                    n2 = __shfl_up_sync(0xffffffffu, h2, 1);
                    n3 = __shfl_up_sync(0xffffffffu, h3, 1);
                    o = h1;
                } else {
                    const int l0 = (lane - r - 2) & 31, l1 = (lane - r - 1) & 31;
                    n1.x = __shfl_sync(0xffffffffu, h1, l0);
                    n1.y = __shfl_sync(0xffffffffu, h1, l1);
                    n2.x = __shfl_sync(0xffffffffu, h2, l0);
                    n2.y = __shfl_sync(0xffffffffu, h2, l1);
                    n3.x = __shfl_sync(0xffffffffu, h3, l0);
                    n3.y = __shfl_sync(0xffffffffu, h3, l1);
                    const double partner = __shfl_xor_sync(0xffffffffu, h1, 1);
                    o.x = r == 0 ? h1 : partner;
                    o.y = r == 0 ? partner : h1;
                }
                double acc = rhs;
#pragma unroll
                for (int q = 0; q < 13; ++q) {
                    const int sm = DIR > 0 ? q : 26 - q;
                    const bool ok = (msk >> sm) & 1u;
                    V val;
                    if (q < 9) {
                        val = zv[q];
                        if (act && ok && slEmptyV<B>(val))
                            val = slWait<B>(zin + ((size_t)(sx + slOx(q)) * ny + (j + slOy(q))) * B, &stopFlag, a.err,
                                            waitNs);
                    } else if (q < 12) {
                        // q 9, 10, 11: line j-1 at steps s-3, s-2, s-1
                        val = q == 9 ? n3 : q == 10 ? n2 : n1;
                        if (firstOfWarp && act && ok) {
                            const double* p = yIn + (size_t)(s - (12 - q)) * B;
                            val = slLd<B>(p);
                            if (slEmptyV<B>(val)) val = slWait<B>(p, &stopFlag, a.err, waitNs);
                        }
                    } else {
                        val = o;
                    }
                    // a slot outside the row's pattern holds +0 in the factor (the assembly
                    // kernels and dxg_set_linear_system write +0 there, the factorisation never
                    // updates it) and its plane-below value was not loaded (+0), so no select is
                    // needed for it: -(+0) * (+0) leaves the accumulator's bits unchanged; the
                    // line-below and own-line values come from shuffles and are zeroed
                    const V mul = m[q];
                    if (q >= 9) val = ok ? val : slZero<B>();
                    if constexpr (B == 1) {
                        acc = fma(-mul, val, acc);
                    } else {
                        acc = fma(-mul.x, val.x, acc);
                        acc = fma(-mul.y, val.y, acc);
                    }
                }
                double res;
                if (DIR > 0) {
                    res = acc;
                } else if constexpr (B == 1) {
                    res = Dr * acc;
                } else {
                    const double accOther = __shfl_xor_sync(0xffffffffu, acc, 1);
                    const double a0 = r == 0 ? acc : accOther, a1 = r == 0 ? accOther : acc;
                    double tt = Dr.x * a0;
                    tt = fma(Dr.y, a1, tt);
                    res = tt;
                }
                if (act) {
                    v[(lineBase + (DIR > 0 ? sx : nx - 1 - sx)) * B + r] = res;
                    if (hasDown) slStCluster(zinDown + (uint32_t)((((size_t)sx * ny + j) * B + r) * sizeof(double)), res);
                    if (lastOfWarp) slStCluster(yOut + (uint32_t)((size_t)s * B * sizeof(double)), res);
                }
                h3 = h2;
                h2 = h1;
                h1 = act ? res : 0.0;
            }
        }
    }
    // no CTA may leave while another can still write into its shared memory
    cluster.sync();
}

template <int B, int DIR>
cudaError_t slLaunch(const StencilArgs& a, const double* d, double* v, cudaStream_t st)
{
    auto kern = stencilLane3dKernel<B, DIR, kSlPf>;
    const size_t smem = slSmemBytes(a.nx, a.ny, B);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSlSmemLimit);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)a.nz);
    cfg.blockDim = dim3((unsigned)((a.ny * B + 31) / 32 * 32));
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)a.nz;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, a, d, v);
}

// ---------------------------------------------------------------- factorisation
// ILU(0) of a 3D stencil matrix over a cluster of 16 CTAs, level by level (hyperplanes
// x + 2y + 4z), one warp per row.  The row's blocks are staged in shared memory; its lower
// slots s are taken in ascending order (every lane forms the multiplier l = a_is Dinv_j, lane 0
// stores it) and the update triples (s, t, u) of one s, whose targets t differ, run on separate
// lanes; a cluster barrier ends each level.  Products, operand order and FMAs are those of
// stencilFactorKernel / stencilFactor2Kernel, so the factors are the same bits.  Before a row's
// elimination its warp stages everything the row reads (its blocks, the lower neighbours'
// pivots, masks and the neighbour blocks of every update triple) in shared memory with all loads
// in flight together: one memory latency per row instead of one per lower slot.  Rows of
// earlier levels are read past L1 (ld.global.cg): another SM of the cluster wrote them.
constexpr int kSfWarps = 16;
constexpr int kSfCtas = 16;

// the k-th row of level L (lines ordered by z, then y), or false
__device__ __forceinline__ bool sfLevelRow(int L, int k, int nx, int ny, int nz, int64_t& i)
{
    const int zLo = max(0, (L - (nx - 1) - 2 * (ny - 1) + 3) >> 2);
    const int zHi = min(nz - 1, L >> 2);
    for (int zz = zLo; zz <= zHi; ++zz) {
        const int rest = L - 4 * zz;
        const int yLo = max(0, (rest - (nx - 1) + 1) >> 1);
        const int yHi = min(ny - 1, rest >> 1);
        const int cnt = yHi - yLo + 1;
        if (cnt <= 0) continue;
        if (k < cnt) {
            const int yy = yLo + k;
            i = ((int64_t)zz * ny + yy) * nx + (rest - 2 * yy);
            return true;
        }
        k -= cnt;
    }
    return false;
}

// shared memory of one warp: the row's blocks [27], the inverted pivots of its 13 lower
// neighbours, per update triple the neighbour's block it reads [104], the neighbours' slot masks
template <int B>
__host__ __device__ constexpr size_t sfWarpBytes()
{
    return (size_t)(27 + 13 + 104) * B * B * sizeof(double) + 64;
}

template <int B>
__global__ void __launch_bounds__(kSfWarps * 32) stencilFactorClusterKernel(StencilArgs a)
{
    constexpr int BB = B * B;
    extern __shared__ __align__(16) unsigned char sfRaw[];
    // the update triples in shared memory: lanes read different triples, which from the kernel
    // parameters (constant bank) would serialise
    __shared__ int8_t tri[104][3];
    for (int e = threadIdx.x; e < a.nTri * 3; e += blockDim.x) tri[e / 3][e % 3] = a.tri[e / 3][e % 3];
    __syncthreads();
    cg::cluster_group cluster = cg::this_cluster();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nW = (int)gridDim.x * kSfWarps;
    const int gw = (int)blockIdx.x * kSfWarps + warp;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const int64_t N = a.N;
    const int S = a.S, center = a.center, nTri = a.nTri;
    const int levels = (nx - 1) + 2 * (ny - 1) + 4 * (nz - 1) + 1;
    double* R = reinterpret_cast<double*>(sfRaw + (size_t)warp * sfWarpBytes<B>());
    double* Dn = R + 27 * BB;
    double* Un = Dn + 13 * BB;
    uint32_t* Mn = reinterpret_cast<uint32_t*>(Un + 104 * BB);
    for (int L = 0; L < levels; ++L) {
        int64_t i;
        for (int k = gw; sfLevelRow(L, k, nx, ny, nz, i); k += nW) {
            const uint32_t m = __ldg(a.mask + i);
            // everything the row reads, staged with all loads in flight together
            for (int e = lane; e < S * BB; e += 32) R[e] = a.A[((int64_t)(e / BB) * N + i) * BB + e % BB];
            for (int e = lane; e < center * BB; e += 32) {
                const int s = e / BB;
                Dn[e] = ((m >> s) & 1u) ? __ldcg(a.Dinv + (i + a.off[s]) * BB + e % BB) : 0.0;
            }
            for (int s = lane; s < center; s += 32) Mn[s] = ((m >> s) & 1u) ? __ldg(a.mask + i + a.off[s]) : 0u;
            for (int e = lane; e < nTri * BB; e += 32) {
                const int kk = e / BB;
                const int s = tri[kk][0], t = tri[kk][1], u = tri[kk][2];
                Un[e] = (((m >> s) & 1u) && ((m >> t) & 1u))
                            ? __ldcg(a.LU + ((int64_t)u * N + i + a.off[s]) * BB + e % BB)
                            : 0.0;
            }
            __syncwarp();
            int t0 = 0;
            // 2x2 blocks: lane q works on entry e = q % 4 (row er, column ec) of update triple
            // t0 + q / 4 + 8 n; every entry of a block product is its own two-FMA chain, so this
            // is the arithmetic of the whole-block products with 3 FP64 instructions per lane and
            // lower slot instead of 12 per triple
            const int e4 = lane & 3, er = e4 >> 1, ec = e4 & 1;
            for (int s = 0; s < center; ++s) {
                if (!((m >> s) & 1u)) continue;
                const uint32_t mj = Mn[s];
                while (t0 < nTri && tri[t0][0] < s) ++t0;
                if constexpr (B == 1) {
                    const double l = R[s] * Dn[s];
                    __syncwarp();
                    if (lane == 0) R[s] = l;
                    for (int k2 = t0 + lane; k2 < nTri && tri[k2][0] == s; k2 += 32) {
                        const int t = tri[k2][1], u = tri[k2][2];
                        if (((m >> t) & 1u) && ((mj >> u) & 1u)) R[t] = fma(-l, Un[k2], R[t]);
                    }
                } else {
                    // row er of the multiplier l = a_is Dinv_j (the entries this lane needs)
                    const double* X = R + s * 4;
                    const double* Y = Dn + s * 4;
                    double l0 = 0.0, l1 = 0.0;
                    l0 = fma(X[er * 2 + 0], Y[0 * 2 + 0], l0);
                    l0 = fma(X[er * 2 + 1], Y[1 * 2 + 0], l0);
                    l1 = fma(X[er * 2 + 0], Y[0 * 2 + 1], l1);
                    l1 = fma(X[er * 2 + 1], Y[1 * 2 + 1], l1);
                    __syncwarp();
                    if (lane < 4) R[s * 4 + e4] = ec == 0 ? l0 : l1;
                    for (int k2 = t0 + (lane >> 2); k2 < nTri && tri[k2][0] == s; k2 += 8) {
                        const int t = tri[k2][1], u = tri[k2][2];
                        if (((m >> t) & 1u) && ((mj >> u) & 1u)) {
                            const double* U = Un + k2 * 4;
                            double pr = 0.0;
                            pr = fma(l0, U[0 * 2 + ec], pr);
                            pr = fma(l1, U[1 * 2 + ec], pr);
                            R[t * 4 + e4] -= pr;
                        }
                    }
                }
                __syncwarp();
            }
            for (int e = lane; e < S * BB; e += 32) a.LU[((int64_t)(e / BB) * N + i) * BB + e % BB] = R[e];
            if (lane == 0) {
                const double* D = R + center * BB;
                if constexpr (B == 1) {
                    if (D[0] == 0.0) atomicExch(a.singular, 1);
                    a.Dinv[i] = 1.0 / D[0];
                } else {
                    const double p12 = D[1] * D[2];
                    const double det = fma(D[0], D[3], -p12);
                    if (det == 0.0) atomicExch(a.singular, 1);
                    const double di = 1.0 / det;
                    a.Dinv[i * 4 + 0] = D[3] * di;
                    a.Dinv[i * 4 + 1] = -D[1] * di;
                    a.Dinv[i * 4 + 2] = -D[2] * di;
                    a.Dinv[i * 4 + 3] = D[0] * di;
                }
            }
            __syncwarp();
        }
        cluster.sync();
    }
}

template <int B>
cudaError_t sfLaunch(const StencilArgs& a, cudaStream_t st)
{
    auto kern = stencilFactorClusterKernel<B>;
    const size_t smem = kSfWarps * sfWarpBytes<B>();
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(kSfCtas);
    cfg.blockDim = dim3(kSfWarps * 32);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = kSfCtas;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, a);
}

}  // namespace

void launchStencilFactorCluster(const StencilArgs& a, cudaStream_t st)
{
    if (a.b == 2) DXG_CUDA(sfLaunch<2>(a, st));
    else DXG_CUDA(sfLaunch<1>(a, st));
}

// 3D 27-point stencils of 1x1 or 2x2 blocks whose planes fit one cluster (nz <= 16), whose
// lines and block rows fit one CTA of at most 256 threads, and whose plane copy and warp
// histories fit the shared memory.
bool stencilLane3dFits(const StencilArgs& a)
{
    if ((a.b != 1 && a.b != 2) || a.S != 27 || a.nx < 1 || a.ny < 1 || a.nz < 1 || a.nz > 16) return false;
    if (a.ny * a.b > kSlMaxThreads) return false;
    return slSmemBytes(a.nx, a.ny, a.b) <= kSlSmemLimit;
}

void launchStencilLane3d(const StencilArgs& a, const double* d, double* v, cudaStream_t st)
{
    if (a.b == 2) {
        DXG_CUDA((slLaunch<2, 1>(a, d, v, st)));
        DXG_CUDA((slLaunch<2, -1>(a, d, v, st)));
    } else {
        DXG_CUDA((slLaunch<1, 1>(a, d, v, st)));
        DXG_CUDA((slLaunch<1, -1>(a, d, v, st)));
    }
}

}  // namespace dxg
