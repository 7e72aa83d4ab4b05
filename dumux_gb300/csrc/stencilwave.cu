// stencilwave.cu -- ILU(0) sweeps of the 2D 9-point stencil (MPFA-O) over a thread-block
// cluster: one thread per grid line y, 32 lines per warp, 4 warps (one per SM
// sub-partition) per CTA, as many CTAs as 128-line blocks (cluster of up to 16).
//
// Natural order: cell (x, y) sits on level L = x + 2y.  Forward, line y needs its own cell
// x-1 (level L-1) and line y-1's cells x+1, x, x-1 (levels L-1, L-2, L-3); backward, line
// y+1's cells x-1, x, x+1 (levels L+1, L+2, L+3).  Every thread keeps its last three
// results: inside a warp they pass on by shuffle; the warp's boundary lane publishes each
// result into a per-level history in the consuming warp's shared memory (in the next CTA of
// the cluster for the last warp, by a remote store), whose entries start all ones (a NaN no
// sweep produces) and are polled by the consumer until written.  No CTA barrier orders the
// levels: every warp runs ahead as far as its inputs allow.  The cells' factor entries and
// right-hand side are copied PF levels ahead into a shared-memory ring with cp.async.  The
// terms enter the accumulator oldest first (forward in ascending, backward in descending
// column order), so only the last level's two results are on the recurrence's critical path;
// the arithmetic is that of stencilApplyKernel (same operand order, explicit FMAs), so the
// results are the same bits.
//
// Every wait is bounded (the context's wait limit, measured with %globaltimer); a thread that
// gives up records DXG_ERR_TIMEOUT, stops its warp's sweep, and all CTAs leave through a final
// cluster barrier, so no CTA exits while another may still write into its shared memory.
#include <cooperative_groups.h>

#include "common.cuh"
#include "linalg_kernels.cuh"

namespace cg = cooperative_groups;

namespace dxg {
namespace {

constexpr int kSwWarps = 4;
constexpr int kSwLines = 32 * kSwWarps;
constexpr unsigned long long kSwDefaultWaitNs = 500000000ull;

__device__ __forceinline__ unsigned long long swTimer()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ uint32_t swSmem(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ uint32_t swMapa(uint32_t addr, int rank)
{
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
    return r;
}
__device__ __forceinline__ void swStCluster(uint32_t dst, double v)
{
    asm volatile("st.relaxed.cluster.shared::cluster.f64 [%0], %1;" ::"r"(dst), "d"(v) : "memory");
}
__device__ __forceinline__ double swLdShared(const double* p)
{
    double v;
    asm volatile("ld.relaxed.cluster.shared::cta.f64 %0, [%1];" : "=d"(v) : "r"(swSmem(p)) : "memory");
    return v;
}
__device__ __forceinline__ double swEmpty() { return __longlong_as_double(-1ll); }
__device__ __forceinline__ bool swIsEmpty(double v) { return __double_as_longlong(v) == -1ll; }
__device__ __forceinline__ void swCp8(uint32_t dst, const void* src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void swCommit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void swCpWait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// shared memory: histories [kSwWarps][levels] (the values each warp's boundary lane
// consumes), then the prefetch ring [PF][kSwLines][6]
__host__ __device__ inline size_t swHistBytes(int levels) { return (((size_t)kSwWarps * levels * 8) + 15) & ~(size_t)15; }
__host__ __device__ inline size_t swSmemBytes(int levels, int pf) { return swHistBytes(levels) + (size_t)pf * kSwLines * 6 * 8; }

template <int DIR, int PF>
__global__ void __launch_bounds__(kSwLines) stencilLane2dKernel(StencilArgs a, const double* __restrict__ d,
                                                                 double* __restrict__ v)
{
    constexpr int REC = DIR > 0 ? 5 : 6;
    extern __shared__ __align__(16) unsigned char swRaw[];
    __shared__ int abortFlag;
    cg::cluster_group cluster = cg::this_cluster();
    const int nx = a.nx, ny = a.ny;
    const int Lmax = (nx - 1) + 2 * (ny - 1);
    const int levels = Lmax + 1;
    double* hist = reinterpret_cast<double*>(swRaw);                            // [kSwWarps][levels]
    double* ring = reinterpret_cast<double*>(swRaw + swHistBytes(levels));      // [PF][kSwLines][REC]
    const int cta = (int)blockIdx.x;
    const int nCta = (int)gridDim.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int y = cta * kSwLines + threadIdx.x;
    const bool lineOk = y < ny;
    const int64_t N = a.N;
    const int64_t rowBase = (int64_t)y * nx;

    for (int k = threadIdx.x; k < kSwWarps * levels; k += kSwLines) hist[k] = swEmpty();
    if (threadIdx.x == 0) abortFlag = 0;
    cluster.sync();
    const bool skip = a.ks && a.ks->status != KS_RUNNING;

    // the boundary lane: producer of the next warp's (forward) / previous warp's (backward)
    // history, and its destination
    const bool producer = DIR > 0 ? lane == 31 : lane == 0;
    const bool consumer = DIR > 0 ? lane == 0 : lane == 31;
    // (a CTA-local shared address lies in the cluster window too)
    uint32_t dst = 0;
    bool hasDst = false;
    if (DIR > 0) {
        if (warp < kSwWarps - 1) { dst = swSmem(hist + (size_t)(warp + 1) * levels); hasDst = true; }
        else if (cta + 1 < nCta) { dst = swMapa(swSmem(hist), cta + 1); hasDst = true; }
    } else {
        if (warp > 0) { dst = swSmem(hist + (size_t)(warp - 1) * levels); hasDst = true; }
        else if (cta > 0) { dst = swMapa(swSmem(hist + (size_t)(kSwWarps - 1) * levels), cta - 1); hasDst = true; }
    }
    const double* myHist = hist + (size_t)warp * levels;
    // the neighbour line across the warp boundary exists
    const bool nbLine = DIR > 0 ? (lineOk && y > 0) : (y + 1 < ny);

    const uint32_t ringBase = swSmem(ring + (size_t)threadIdx.x * REC);
    constexpr uint32_t kSlotBytes = kSwLines * REC * 8u;
    auto cellX = [&](int s) -> int {
        const int L = DIR > 0 ? s : Lmax - s;
        const int x = L - 2 * y;
        return (lineOk && s <= Lmax && x >= 0 && x < nx) ? x : -1;
    };
    auto issue = [&](int s) {
        const int x = cellX(s);
        if (x >= 0) {
            const int64_t i = rowBase + x;
            const uint32_t rec = ringBase + (uint32_t)(s % PF) * kSlotBytes;
            if (DIR > 0) {
                for (int k = 0; k < 4; ++k) swCp8(rec + 8u * k, a.LU + (int64_t)k * N + i);
                swCp8(rec + 32u, d + i);
            } else {
                for (int k = 0; k < 4; ++k) swCp8(rec + 8u * k, a.LU + (int64_t)(5 + k) * N + i);
                swCp8(rec + 32u, a.Dinv + i);
                swCp8(rec + 40u, v + i);
            }
        }
        swCommit();
    };
    const unsigned long long waitNs = a.waitNs ? a.waitNs : kSwDefaultWaitNs;
    // the history entry of level L, polled until written; false when the sweep stops
    auto poll = [&](int L, double& out) -> bool {
        out = swLdShared(myHist + L);
        if (!swIsEmpty(out)) return true;
        const unsigned long long deadline = swTimer() + waitNs;
        while (swIsEmpty(out = swLdShared(myHist + L))) {
            if (*(volatile int*)&abortFlag) return false;
            if (swTimer() > deadline) {
                atomicExch(a.err, DXG_ERR_TIMEOUT);
                abortFlag = 1;
                return false;
            }
        }
        return true;
    };

    if (!skip) {
#pragma unroll
        for (int s = 0; s < PF; ++s) issue(s);
        double r1 = 0.0, r2 = 0.0, r3 = 0.0;
        for (int s = 0; s <= Lmax; ++s) {
            const int L = DIR > 0 ? s : Lmax - s;
            const int x = cellX(s);
            const int dl = DIR > 0 ? -1 : 1;
            // the neighbour line's cells two and three levels back first (available long
            // before the last level's results), so their terms are in the accumulator when
            // the freshest values arrive: forward (x, y-1) at L-2 and (x-1, y-1) at L-3,
            // backward (x, y+1) at L+2 and (x+1, y+1) at L+3
            double n3 = DIR > 0 ? __shfl_up_sync(0xffffffffu, r3, 1) : __shfl_down_sync(0xffffffffu, r3, 1);
            double n2 = DIR > 0 ? __shfl_up_sync(0xffffffffu, r2, 1) : __shfl_down_sync(0xffffffffu, r2, 1);
            bool ok = true;
            const bool across = consumer && x >= 0 && nbLine;
            if (across) {
                if (DIR > 0 ? x > 0 : x < nx - 1) ok = poll(L + 3 * dl, n3);
                if (ok) ok = poll(L + 2 * dl, n2);
            }
            if (__any_sync(0xffffffffu, !ok)) break;
            swCpWait<PF - 1>();
            const double* rec = ring + ((size_t)(s % PF) * kSwLines + threadIdx.x) * REC;
            double acc = 0.0;
            if (x >= 0) {
                if (DIR > 0) {
                    acc = rec[4];
                    if (x > 0 && y > 0) acc = fma(-rec[0], n3, acc);          // (x-1, y-1)
                    if (y > 0) acc = fma(-rec[1], n2, acc);                   // (x,   y-1)
                } else {
                    acc = rec[5];
                    if (x < nx - 1 && y < ny - 1) acc = fma(-rec[3], n3, acc);   // (x+1, y+1)
                    if (y < ny - 1) acc = fma(-rec[2], n2, acc);                 // (x,   y+1)
                }
            }
            // the last level's results: the neighbour line's (x+1, y-1) / (x-1, y+1) and this
            // line's previous cell
            double n1 = DIR > 0 ? __shfl_up_sync(0xffffffffu, r1, 1) : __shfl_down_sync(0xffffffffu, r1, 1);
            if (across && (DIR > 0 ? x < nx - 1 : x > 0)) ok = poll(L + dl, n1);
            if (__any_sync(0xffffffffu, !ok)) break;
            double res = 0.0;
            if (x >= 0) {
                const int64_t i = rowBase + x;
                if (DIR > 0) {
                    if (x < nx - 1 && y > 0) acc = fma(-rec[2], n1, acc);     // (x+1, y-1)
                    if (x > 0) acc = fma(-rec[3], r1, acc);                   // (x-1, y)
                    res = acc;
                } else {
                    if (x > 0 && y < ny - 1) acc = fma(-rec[1], n1, acc);        // (x-1, y+1)
                    if (x < nx - 1) acc = fma(-rec[0], r1, acc);                  // (x+1, y)
                    res = rec[4] * acc;
                }
                v[i] = res;
                if (producer && hasDst) swStCluster(dst + (uint32_t)L * 8u, res);
            }
            r3 = r2;
            r2 = r1;
            r1 = res;
            issue(s + PF);
        }
        swCpWait<0>();
    }
    // no CTA may leave while another can still write into its shared memory
    cluster.sync();
}

template <int DIR, int PF>
cudaError_t swLaunch(const StencilArgs& a, const double* d, double* v, int ctas, cudaStream_t st)
{
    auto kern = stencilLane2dKernel<DIR, PF>;
    const int levels = (a.nx - 1) + 2 * (a.ny - 1) + 1;
    const size_t smem = swSmemBytes(levels, PF);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)ctas);
    cfg.blockDim = dim3(kSwLines);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)ctas;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, a, d, v);
}

constexpr int kSwPf = 8;
constexpr size_t kSwSmemLimit = 200 * 1024;

}  // namespace

// The cluster sweeps take 2D 9-point stencils whose lines fit one cluster of at most 16
// CTAs and whose histories and ring fit the shared memory.
bool stencilLane2dFits(const StencilArgs& a)
{
    if (a.b != 1 || a.S != 9 || a.nz != 1 || a.ny < 1 || a.nx < 1) return false;
    const int ctas = (a.ny + kSwLines - 1) / kSwLines;
    if (ctas > 16) return false;
    const int levels = (a.nx - 1) + 2 * (a.ny - 1) + 1;
    return swSmemBytes(levels, kSwPf) <= kSwSmemLimit;
}

void launchStencilLane2d(const StencilArgs& a, const double* d, double* v, cudaStream_t st)
{
    const int ctas = (a.ny + kSwLines - 1) / kSwLines;
    DXG_CUDA((swLaunch<1, kSwPf>(a, d, v, ctas, st)));
    DXG_CUDA((swLaunch<-1, kSwPf>(a, d, v, ctas, st)));
}

}  // namespace dxg
