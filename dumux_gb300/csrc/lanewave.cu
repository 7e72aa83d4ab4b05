// lanewave.cu -- natural-order ILU(0) triangular sweeps of 3D 2x2-block systems, two lanes per
// x-line, one warp per 16 lines, one z-plane (of up to 64 lines) per CTA.
//
// On GB300 an FP64 warp instruction holds its SM sub-partition for ~64 cycles whatever the
// number of active lanes, and a dependent FP64 FMA takes as long: a wavefront level costs at
// least (dependent FP64 instructions of one step) x 64 cycles.  The two rows of a 2x2 block go
// to two lanes, so a step is one chain of 6 dependent FMAs per lane (forward; 8 backward with
// the pivot product), and a CTA holds one plane in 4 warps, one per sub-partition.  Everything
// else a step does is kept short and off that chain:
//   * the cells' factor rows and right-hand side are loaded PF steps ahead into registers (a
//     ring unrolled by PF), the entries of missing neighbours as zeros, so the chain has no
//     branches: a zero multiplier times a zero neighbour value leaves the accumulator's bits
//     unchanged, so the results are those of the sweeps that skip the term;
//   * a neighbour value from another warp or CTA is one vector load of both block rows, polled
//     after the terms that do not need it were issued;
//   * no vote and no barrier per step: a wait that expires records DXG_ERR_TIMEOUT and sets the
//     CTA's stop flag, after which every wait of the CTA returns at once (the sweep runs out on
//     stale values, which the error discards).
// A second form (laneRingKernel, below) copies the records ahead into a shared-memory ring with
// cp.async and polls before the step's FMAs; it is faster where most plane hand-offs cross
// clusters, and the context times both.  The backward sweep of either form is launched as a
// programmatic dependent of the forward one, so its prologue overlaps the forward sweep.
//
// Dependencies of cell (x, y, z) at level x+y+z: (x-1, y, z), (x, y-1, z), (x, y, z-1) at the
// level before (forward; mirrored for the backward sweep).
//   * x: the same lanes' previous cell (registers; the other row through a lane shuffle);
//   * y inside a warp: the lanes of line j-1 (shuffles); across warps: a per-level history of
//     the last line of the warp before in shared memory; across CTAs of one plane (ny > 64):
//     remote stores into the next CTA's per-level history;
//   * z: the plane before is another CTA.  Inside a thread-block cluster its results go
//     straight into this CTA's shared-memory history of the whole sweep ([x][line], no ring,
//     so no back-pressure) by remote stores.  Across clusters they go into a hand-off buffer
//     in global memory, one entry per cell.
// Every history starts filled with an all-ones bit pattern (a NaN that no arithmetic
// produces) that the consumer waits to see replaced: each entry is one aligned 4- or 8-byte
// relaxed store, seen whole, so neither side needs a fence, a flag or a barrier per level.  The
// consumer of a global hand-off puts the pattern back after reading, so every launch starts
// from it; the shared-memory histories are filled at the start of each launch.
// Warps advance on their own and wait only for the data they consume.  Producers always have
// lower CTA indices than their consumers.
//
// The arithmetic per row and cell is the one of wave.cu and of the level-scheduled kernels of
// linalg.cu (same operands, same order, explicit FMAs), so all give the same sweep results.
#include <algorithm>
#include <climits>
#include <vector>

#include <cooperative_groups.h>

#include "common.cuh"
#include "linalg.cuh"
#include "wave.cuh"

namespace cg = cooperative_groups;

namespace dxg {

namespace {

constexpr int kLwWarps = 4;
constexpr int kLwLinesPerWarp = 16;
constexpr int kLwTile = kLwWarps * kLwLinesPerWarp;   // lines of one CTA
constexpr int kLwThreads = kLwWarps * 32;
constexpr size_t kLwSmemLimit = 220 * 1024;

// both rows of a block-vector entry, or one row of a 2x2 block
template <class T>
struct LwPair;
template <>
struct LwPair<double> {
    using type = double2;
};
template <>
struct LwPair<float> {
    using type = float2;
};

struct LwSmem {
    size_t zin, ybuf, yin, total;
};
__host__ __device__ inline LwSmem lwSmem(int nx, int levels, int tsize)
{
    LwSmem s{};
    size_t o = 0;
    s.zin = o;
    o += (size_t)nx * kLwTile * 2 * tsize;
    s.ybuf = o;
    o += (size_t)kLwWarps * levels * 2 * tsize;
    s.yin = o;
    o += (size_t)levels * 2 * tsize;
    s.total = (o + 15) & ~(size_t)15;
    return s;
}

__device__ __forceinline__ unsigned long long lwTimer()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ uint32_t lwSmemAddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ uint32_t lwMapa(uint32_t addr, int rank)
{
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
    return r;
}
// The hand-off stores and polls carry no "memory" clobber: they need no order against the
// step's other memory operations (a poll issued early sees the empty pattern and repeats;
// volatile keeps every poll), so the compiler may schedule the record loads across them.
// relaxed store into the shared memory of a CTA of the cluster
template <class T>
__device__ __forceinline__ void lwStRemote(uint32_t dst, T v)
{
    if constexpr (sizeof(T) == 8)
        asm volatile("st.relaxed.cluster.shared::cluster.f64 [%0], %1;" ::"r"(dst), "d"(v));
    else
        asm volatile("st.relaxed.cluster.shared::cluster.f32 [%0], %1;" ::"r"(dst), "f"(v));
}
// The "not written yet" pattern of the hand-off histories: all bits set (a NaN that no
// arithmetic yields; cudaMemset with 0xff produces it).
template <class T>
__device__ __forceinline__ T lwEmpty()
{
    if constexpr (sizeof(T) == 8) return __longlong_as_double(-1ll);
    else return __int_as_float(-1);
}
template <class T>
__device__ __forceinline__ bool lwIsEmpty(T v)
{
    if constexpr (sizeof(T) == 8) return __double_as_longlong(v) == -1ll;
    else return __float_as_int(v) == -1;
}
template <class T>
__device__ __forceinline__ bool lwPairEmpty(typename LwPair<T>::type v)
{
    return lwIsEmpty<T>(v.x) || lwIsEmpty<T>(v.y);
}
// one relaxed vector load of a pair from this CTA's shared memory / from global memory (each
// half is one single-copy-atomic element)
template <class T>
__device__ __forceinline__ typename LwPair<T>::type lwLdPairShared(const T* p)
{
    typename LwPair<T>::type v;
    if constexpr (sizeof(T) == 8)
        asm volatile("ld.relaxed.cluster.shared::cta.v2.f64 {%0, %1}, [%2];"
                     : "=d"(v.x), "=d"(v.y)
                     : "r"(lwSmemAddr(p)));
    else
        asm volatile("ld.relaxed.cluster.shared::cta.v2.f32 {%0, %1}, [%2];"
                     : "=f"(v.x), "=f"(v.y)
                     : "r"(lwSmemAddr(p)));
    return v;
}
template <class T>
__device__ __forceinline__ typename LwPair<T>::type lwLdPairGpu(const T* p)
{
    typename LwPair<T>::type v;
    if constexpr (sizeof(T) == 8)
        asm volatile("ld.relaxed.gpu.global.v2.f64 {%0, %1}, [%2];" : "=d"(v.x), "=d"(v.y) : "l"(p));
    else
        asm volatile("ld.relaxed.gpu.global.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "l"(p));
    return v;
}
template <class T>
__device__ __forceinline__ void lwStRelaxedGpu(T* p, T v)
{
    if constexpr (sizeof(T) == 8) asm volatile("st.relaxed.gpu.global.f64 [%0], %1;" ::"l"(p), "d"(v));
    else asm volatile("st.relaxed.gpu.global.f32 [%0], %1;" ::"l"(p), "f"(v));
}
// putting the empty pattern back must stay behind the warp barrier that follows the reads
template <class T>
__device__ __forceinline__ void lwStPairGpu(T* p, T x, T y)
{
    if constexpr (sizeof(T) == 8)
        asm volatile("st.relaxed.gpu.global.v2.f64 [%0], {%1, %2};" ::"l"(p), "d"(x), "d"(y) : "memory");
    else
        asm volatile("st.relaxed.gpu.global.v2.f32 [%0], {%1, %2};" ::"l"(p), "f"(x), "f"(y) : "memory");
}
// read-only loads of the records (the factor, pivots and the sweep's input vector)
template <class T>
__device__ __forceinline__ typename LwPair<T>::type lwLdg2(const T* p)
{
    return __ldg(reinterpret_cast<const typename LwPair<T>::type*>(p));
}

// The slow path of a poll: waits, bounded, until neither half of the pair at p holds the empty
// pattern, and returns it.  Returns zeros once the CTA's sweep has stopped or when the wait
// expires (which records DXG_ERR_TIMEOUT and stops the CTA's sweep).
template <class T>
__device__ __noinline__ typename LwPair<T>::type lwWaitPair(const T* p, bool global, int* stop, int* err,
                                                          unsigned long long waitNs)
{
    using P = typename LwPair<T>::type;
    const unsigned long long deadline = lwTimer() + waitNs;
    for (;;) {
        const P v = global ? lwLdPairGpu(p) : lwLdPairShared(p);
        if (!lwPairEmpty<T>(v)) return v;
        if (*(volatile int*)stop) break;
        if (lwTimer() > deadline) {
            atomicExch(err, DXG_ERR_TIMEOUT);
            *(volatile int*)stop = 1;
            break;
        }
    }
    P zero;
    zero.x = 0;
    zero.y = 0;
    return zero;
}


// ---- the shared-memory-ring form (laneRingKernel)
template <int DIR>
struct LwRec {
    static constexpr int n = DIR > 0 ? 8 : 10;
};

struct LrSmem {
    size_t zin, ybuf, yin, ring, total;
};
__host__ __device__ inline LrSmem lrSmem(int nx, int levels, int tsize, int recElems, int pf)
{
    LrSmem s{};
    size_t o = 0;
    s.zin = o;
    o += (size_t)nx * kLwTile * 2 * tsize;
    s.ybuf = o;
    o += (size_t)kLwWarps * levels * 2 * tsize;
    s.yin = o;
    o += (size_t)levels * 2 * tsize;
    o = (o + 15) & ~(size_t)15;
    s.ring = o;
    o += (size_t)pf * kLwThreads * recElems * tsize;
    s.total = o;
    return s;
}
template <class T>
__device__ __forceinline__ T lwLdRelaxedShared(const T* p)
{
    T v;
    if constexpr (sizeof(T) == 8)
        asm volatile("ld.relaxed.cluster.shared::cta.f64 %0, [%1];" : "=d"(v) : "r"(lwSmemAddr(p)) : "memory");
    else
        asm volatile("ld.relaxed.cluster.shared::cta.f32 %0, [%1];" : "=f"(v) : "r"(lwSmemAddr(p)) : "memory");
    return v;
}
// The "not written yet" pattern of the hand-off histories: all bits set (a NaN that no
// arithmetic yields; cudaMemset with 0xff produces it).
template <class T>
__device__ __forceinline__ T lwLdRelaxedGpu(const T* p)
{
    T v;
    if constexpr (sizeof(T) == 8) asm volatile("ld.relaxed.gpu.global.f64 %0, [%1];" : "=d"(v) : "l"(p) : "memory");
    else asm volatile("ld.relaxed.gpu.global.f32 %0, [%1];" : "=f"(v) : "l"(p) : "memory");
    return v;
}
template <int BYTES>
__device__ __forceinline__ void lwCpAsync(uint32_t dst, const void* src)
{
    if constexpr (BYTES == 16) asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
    else asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(dst), "l"(src), "n"(BYTES) : "memory");
}
__device__ __forceinline__ void lwCommit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void lwCpWait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }
}  // namespace

// One sweep: DIR +1 forward (z_i = d_i - L_ix z_x - L_iy z_y - L_iz z_z), DIR -1 backward
// (y_i = D_i^-1 (v_i - U_ix y_x - U_iy y_y - U_iz y_z), in place in v).  PF: depth of the
// register ring of prefetched records.
template <class T, int DIR, int PF>
__global__ void __launch_bounds__(kLwThreads) laneWaveKernel(LaneWaveArgs<T> a)
{
    using P = typename LwPair<T>::type;
    extern __shared__ __align__(16) unsigned char lwRaw[];
    __shared__ int stopFlag;

    cg::cluster_group cluster = cg::this_cluster();
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const int levels = nx + ny + nz - 2;
    const LwSmem lay = lwSmem(nx, levels, (int)sizeof(T));
    T* zin = reinterpret_cast<T*>(lwRaw + lay.zin);     // [nx][kLwTile][2]
    T* ybuf = reinterpret_cast<T*>(lwRaw + lay.ybuf);   // [kLwWarps][levels][2]
    T* yin = reinterpret_cast<T*>(lwRaw + lay.yin);     // [levels][2]

    const int cta = (int)blockIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int j = lane >> 1, r = lane & 1;
    const int jl = warp * kLwLinesPerWarp + j;           // line within the tile
    const bool working = cta < a.ctas;
    // tile in sweep coordinates (the backward sweep mirrors x, y and z)
    const int sz = working ? cta / a.nyb : 0;
    const int syb = working ? cta % a.nyb : 0;
    const int sy0 = syb * kLwTile;
    const int sy = sy0 + jl;
    const bool lineOk = working && sy < ny;
    const int z = DIR > 0 ? sz : nz - 1 - sz;
    const int y = DIR > 0 ? sy : ny - 1 - sy;
    const int64_t N = a.N;
    const int64_t lineBase = lineOk ? ((int64_t)z * ny + y) * nx : 0;
    const int cs = a.clusterSize;
    const bool hasZUp = working && sz > 0;
    const int zUp = cta - a.nyb;
    const bool zUpLocal = hasZUp && zUp / cs == cta / cs;
    const int zDown = cta + a.nyb;
    const bool hasZDown = working && zDown < a.ctas;
    const bool zDownLocal = hasZDown && zDown / cs == cta / cs;
    const bool hasYUp = working && syb > 0;
    const bool hasYDown = working && syb + 1 < a.nyb;
    const int lastLine = min(sy0 + kLwTile, ny) - 1;
    const int Lfirst = sy0 + sz;
    const int nSteps = working ? lastLine + nx - sy0 : 0;

    // the incoming histories start empty (before any CTA of the cluster writes into them)
    if (hasZUp && zUpLocal)
        for (int k = threadIdx.x; k < nx * kLwTile * 2; k += kLwThreads) zin[k] = lwEmpty<T>();
    for (int k = threadIdx.x; k < kLwWarps * levels * 2; k += kLwThreads) ybuf[k] = lwEmpty<T>();
    if (hasYUp)
        for (int k = threadIdx.x; k < levels * 2; k += kLwThreads) yin[k] = lwEmpty<T>();
    if (threadIdx.x == 0) stopFlag = 0;
    cluster.sync();
    // The backward sweep reads the forward sweep's output.  It is launched as a programmatic
    // dependent of the forward sweep: its CTAs start and fill their histories while the forward
    // sweep runs (whose CTAs allow that right after their own start) and wait here until it has
    // completed and its writes are visible.
    if (DIR < 0) asm volatile("griddepcontrol.wait;" ::: "memory");
    else asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    const bool skip = a.ks && a.ks->status != KS_RUNNING;

    // record sources of this lane's line at x = 0 (slots: forward -x 2, -y 1, -z 0; backward
    // +x 4, +y 5, +z 6); a cell adds 4 (blocks) or 2 (vectors) elements per x
    const T* mat = DIR > 0 ? a.Lf : a.A;
    const T* srcX = mat + ((int64_t)(DIR > 0 ? 2 : 4) * N + lineBase) * 4 + 2 * r;
    const T* srcY = mat + ((int64_t)(DIR > 0 ? 1 : 5) * N + lineBase) * 4 + 2 * r;
    const T* srcZ = mat + ((int64_t)(DIR > 0 ? 0 : 6) * N + lineBase) * 4 + 2 * r;
    const T* srcD = a.Dinv + lineBase * 4 + 2 * r;
    const T* srcV = (DIR > 0 ? a.rhs : a.v) + lineBase * 2 + r;
    const bool hasY = sy > 0, hasZ = sz > 0;

    // where the neighbour values from other warps and CTAs arrive (pairs of both rows) ...
    const bool zGlobalIn = hasZUp && !zUpLocal;
    const bool zLocalIn = hasZUp && zUpLocal;
    const bool yPoll = lineOk && j == 0 && hasY;   // warp > 0: ybuf; warp 0 with sy > 0: yin
    const T* yPollSrc = warp > 0 ? ybuf + (size_t)(warp - 1) * levels * 2 : yin;   // + level * 2
    const T* zLocalSrc = zin + (size_t)jl * 2;                                       // + x * kLwTile * 2
    const T* zGlobalSrc = a.handoff + ((size_t)cta * nx * kLwTile + jl) * 2;         // + x * kLwTile * 2
    // ... and where this lane's results go (one row each)
    T* const zGlobalDst = hasZDown && !zDownLocal ? a.handoff + ((size_t)zDown * nx * kLwTile + jl) * 2 + r : nullptr;
    const uint32_t zInDownBase =
        (zDownLocal ? lwMapa(lwSmemAddr(zin), zDown % cs) : 0u) + (uint32_t)(((size_t)jl * 2 + r) * sizeof(T));
    const bool yPub = j == kLwLinesPerWarp - 1 && (warp < kLwWarps - 1 || hasYDown);
    const uint32_t yPubBase = (warp < kLwWarps - 1 ? lwSmemAddr(ybuf + (size_t)warp * levels * 2)
                                                   : (hasYDown ? lwMapa(lwSmemAddr(yin), (cta + 1) % cs) : 0u)) +
                              (uint32_t)(r * sizeof(T));

    // the register ring: records of step s in entry (s - first step) % PF
    P rX[PF], rY[PF], rZ[PF], rD[PF];
    T rV[PF];
    auto load = [&](int s, int k) {
        const int sx = s - jl;
        const bool act = lineOk && sx >= 0 && sx < nx;
        const int x = DIR > 0 ? sx : nx - 1 - sx;
        P zero;
        zero.x = 0;
        zero.y = 0;
        rX[k] = act && sx > 0 ? lwLdg2(srcX + 4 * x) : zero;
        rY[k] = act && hasY ? lwLdg2(srcY + 4 * x) : zero;
        rZ[k] = act && hasZ ? lwLdg2(srcZ + 4 * x) : zero;
        if (DIR < 0) rD[k] = act ? lwLdg2(srcD + 4 * x) : zero;
        rV[k] = act ? __ldg(srcV + 2 * x) : T(0);
    };

    const bool warpWorks = working && !skip && sy0 + warp * kLwLinesPerWarp < ny;
    if (warpWorks) {
        // line jl starts at step jl; the warp's lines are done after its last line's nx cells
        const int sBegin = warp * kLwLinesPerWarp;
        const int sEnd = min(nSteps, sBegin + kLwLinesPerWarp - 1 + nx);
        T prev = 0;
        // the inter-cluster z pair of the next step, loaded a step early (a load that still saw
        // the empty pattern is repeated by the poll)
        P gz;
        gz.x = lwEmpty<T>();
        gz.y = gz.x;
        if (zGlobalIn && lineOk && sBegin - jl >= 0) gz = lwLdPairGpu(zGlobalSrc + (size_t)(sBegin - jl) * kLwTile * 2);

        auto step = [&](int s, int k) {
            const int sx = s - jl;
            const bool act = lineOk && sx >= 0 && sx < nx;
            const int L = Lfirst + s;
            // this step's records out of the ring, whose entry is refilled right away (the
            // loads issue ahead of the step's dependent chain; measured faster than refilling
            // after the step)
            const P cX = rX[k], cY = rY[k], cZ = rZ[k];
            P cD;
            if (DIR < 0) cD = rD[k];
            const T cV = rV[k];
            load(s + PF, k);
            // x neighbour: this line's previous cell (other row from the partner lane); y
            // neighbour: line j-1 at the step before (same row two lanes down, other row from
            // lane 2j-2+(1-r)); three independent shuffles of the previous results
            const T other = __shfl_xor_sync(0xffffffffu, prev, 1);
            const T ySame = __shfl_up_sync(0xffffffffu, prev, 2);
            const T yOther = __shfl_sync(0xffffffffu, prev, (lane - 1 - 2 * r) & 31);
            T acc = cV;
            acc = fma(-cX.x, r == 0 ? prev : other, acc);
            acc = fma(-cX.y, r == 0 ? other : prev, acc);
            T zy0 = hasY ? (r == 0 ? ySame : yOther) : T(0);
            T zy1 = hasY ? (r == 0 ? yOther : ySame) : T(0);
            if (act && yPoll) {
                const T* src = yPollSrc + (size_t)(L - 1) * 2;
                P v = lwLdPairShared(src);
                if (lwPairEmpty<T>(v)) v = lwWaitPair(src, false, &stopFlag, a.err, a.waitNs);
                zy0 = v.x;
                zy1 = v.y;
            }
            acc = fma(-cY.x, zy0, acc);
            acc = fma(-cY.y, zy1, acc);
            T zz0 = 0, zz1 = 0;
            if (zLocalIn) {
                if (act) {
                    const T* src = zLocalSrc + (size_t)sx * kLwTile * 2;
                    P v = lwLdPairShared(src);
                    if (lwPairEmpty<T>(v)) v = lwWaitPair(src, false, &stopFlag, a.err, a.waitNs);
                    zz0 = v.x;
                    zz1 = v.y;
                }
            } else if (zGlobalIn) {
                const T* src = zGlobalSrc + (int64_t)sx * kLwTile * 2;
                if (act) {
                    P v = gz;
                    if (lwPairEmpty<T>(v)) v = lwWaitPair(src, true, &stopFlag, a.err, a.waitNs);
                    zz0 = v.x;
                    zz1 = v.y;
                }
                if (lineOk && sx + 1 >= 0 && sx + 1 < nx) gz = lwLdPairGpu(src + kLwTile * 2);
                // both lanes of the line hold the pair: put the empty pattern back
                __syncwarp();
                if (act && r == 0) lwStPairGpu(const_cast<T*>(src), lwEmpty<T>(), lwEmpty<T>());
            }
            acc = fma(-cZ.x, zz0, acc);
            acc = fma(-cZ.y, zz1, acc);
            T res = acc;
            if (DIR < 0) {
                const T accOther = __shfl_xor_sync(0xffffffffu, acc, 1);
                const T a0 = r == 0 ? acc : accOther, a1 = r == 0 ? accOther : acc;
                T t = cD.x * a0;
                t = fma(cD.y, a1, t);
                res = t;
            }
            if (act) {
                const int x = DIR > 0 ? sx : nx - 1 - sx;
                a.v[(lineBase + x) * 2 + r] = res;
                if (zDownLocal)
                    lwStRemote<T>(zInDownBase + (uint32_t)((size_t)sx * kLwTile * 2 * sizeof(T)), res);
                else if (hasZDown)
                    lwStRelaxedGpu(zGlobalDst + (size_t)sx * kLwTile * 2, res);
                if (yPub) lwStRemote<T>(yPubBase + (uint32_t)((size_t)L * 2 * sizeof(T)), res);
                prev = res;
            }
        };

#pragma unroll
        for (int k = 0; k < PF; ++k) load(sBegin + k, k);
        for (int s0 = sBegin; s0 < sEnd; s0 += PF) {
#pragma unroll
            for (int k = 0; k < PF; ++k) {
                step(s0 + k, k);
            }
        }
    }
    // no CTA may leave while another can still write into its shared memory
    cluster.sync();
}

// The shared-memory-ring form of the same sweeps: each step's records are copied PF steps
// ahead into a shared-memory ring with cp.async, the y and z hand-offs are polled before the
// step's FMAs, and a vote per step stops the warp on an expired wait.  Same arithmetic, same
// bits.  On grids whose z hand-offs mostly cross clusters (128x128x64 in clusters of 4: 0.97
// against 1.24 ms per apply) it is the faster form; the context times both.
template <class T, int DIR, int PF>
__global__ void __launch_bounds__(kLwThreads) laneRingKernel(LaneWaveArgs<T> a)
{
    constexpr int REC = LwRec<DIR>::n;
    constexpr int RB = 2 * (int)sizeof(T);   // bytes of one block row
    extern __shared__ __align__(16) unsigned char lwRaw[];
    __shared__ int abortFlag;

    cg::cluster_group cluster = cg::this_cluster();
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const int levels = nx + ny + nz - 2;
    const LrSmem lay = lrSmem(nx, levels, (int)sizeof(T), REC, PF);
    T* zin = reinterpret_cast<T*>(lwRaw + lay.zin);     // [nx][kLwTile][2]
    T* ybuf = reinterpret_cast<T*>(lwRaw + lay.ybuf);   // [kLwWarps][levels][2]
    T* yin = reinterpret_cast<T*>(lwRaw + lay.yin);     // [levels][2]
    T* ring = reinterpret_cast<T*>(lwRaw + lay.ring);   // [PF][kLwThreads][REC]

    const int cta = (int)blockIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int j = lane >> 1, r = lane & 1;
    const int jl = warp * kLwLinesPerWarp + j;           // line within the tile
    const bool working = cta < a.ctas;
    // tile in sweep coordinates (the backward sweep mirrors x, y and z)
    const int sz = working ? cta / a.nyb : 0;
    const int syb = working ? cta % a.nyb : 0;
    const int sy0 = syb * kLwTile;
    const int sy = sy0 + jl;
    const bool lineOk = working && sy < ny;
    const int z = DIR > 0 ? sz : nz - 1 - sz;
    const int y = DIR > 0 ? sy : ny - 1 - sy;
    const int64_t N = a.N;
    const int64_t lineBase = lineOk ? ((int64_t)z * ny + y) * nx : 0;
    const int cs = a.clusterSize;
    const bool hasZUp = working && sz > 0;
    const int zUp = cta - a.nyb;
    const bool zUpLocal = hasZUp && zUp / cs == cta / cs;
    const int zDown = cta + a.nyb;
    const bool hasZDown = working && zDown < a.ctas;
    const bool zDownLocal = hasZDown && zDown / cs == cta / cs;
    const bool hasYUp = working && syb > 0;
    const bool hasYDown = working && syb + 1 < a.nyb;
    const int lastLine = min(sy0 + kLwTile, ny) - 1;
    const int Lfirst = sy0 + sz;
    const int nSteps = working ? lastLine + nx - sy0 : 0;

    // the incoming histories start empty (before any CTA of the cluster writes into them)
    if (hasZUp && zUpLocal)
        for (int k = threadIdx.x; k < nx * kLwTile * 2; k += kLwThreads) zin[k] = lwEmpty<T>();
    for (int k = threadIdx.x; k < kLwWarps * levels * 2; k += kLwThreads) ybuf[k] = lwEmpty<T>();
    if (hasYUp)
        for (int k = threadIdx.x; k < levels * 2; k += kLwThreads) yin[k] = lwEmpty<T>();
    if (threadIdx.x == 0) abortFlag = 0;
    cluster.sync();
    // The backward sweep reads the forward sweep's output.  It is launched as a programmatic
    // dependent of the forward sweep: its CTAs start and fill their histories while the forward
    // sweep runs (whose CTAs allow that right after their own start) and wait here until it has
    // completed and its writes are visible.
    if (DIR < 0) asm volatile("griddepcontrol.wait;" ::: "memory");
    else asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    const bool skip = a.ks && a.ks->status != KS_RUNNING;

    const uint32_t zinDown = zDownLocal ? lwMapa(lwSmemAddr(zin), zDown % cs) : 0u;
    const uint32_t yinDown = hasYDown ? lwMapa(lwSmemAddr(yin), (cta + 1) % cs) : 0u;

    // cell of step s on this lane's line (sweep x), or -1
    const int sx0 = Lfirst - sy - sz;
    auto cellX = [&](int s) -> int {
        const int sx = sx0 + s;
        return (lineOk && s < nSteps && sx >= 0 && sx < nx) ? sx : -1;
    };
    auto cellIndex = [&](int sx) -> int64_t { return lineBase + (DIR > 0 ? sx : nx - 1 - sx); };
    // record sources of this lane's line at x = 0 (slots: forward -x 2, -y 1, -z 0; backward
    // +x 4, +y 5, +z 6); a cell adds 4 (blocks) or 2 (vectors) elements per x
    const T* mat = DIR > 0 ? a.Lf : a.A;
    const T* srcX = mat + ((int64_t)(DIR > 0 ? 2 : 4) * N + lineBase) * 4 + 2 * r;
    const T* srcY = mat + ((int64_t)(DIR > 0 ? 1 : 5) * N + lineBase) * 4 + 2 * r;
    const T* srcZ = mat + ((int64_t)(DIR > 0 ? 0 : 6) * N + lineBase) * 4 + 2 * r;
    const T* srcD = a.Dinv + lineBase * 4 + 2 * r;
    const T* srcV = (DIR > 0 ? a.rhs : a.v) + lineBase * 2 + r;
    const uint32_t ringBase = lwSmemAddr(ring + (size_t)threadIdx.x * REC);
    // copies of the records of step s into ring slot s % PF
    auto issue = [&](int s) {
        const int sx = cellX(s);
        if (sx >= 0) {
            const int x = DIR > 0 ? sx : nx - 1 - sx;
            const uint32_t rec = ringBase + (uint32_t)((s % PF) * kLwThreads * REC * (int)sizeof(T));
            if (sx > 0) lwCpAsync<RB>(rec + 0 * RB, srcX + 4 * x);
            if (sy > 0) lwCpAsync<RB>(rec + 1 * RB, srcY + 4 * x);
            if (sz > 0) lwCpAsync<RB>(rec + 2 * RB, srcZ + 4 * x);
            if (DIR > 0) {
                lwCpAsync<(int)sizeof(T)>(rec + 3 * RB, srcV + 2 * x);
            } else {
                lwCpAsync<RB>(rec + 3 * RB, srcD + 4 * x);
                lwCpAsync<(int)sizeof(T)>(rec + 4 * RB, srcV + 2 * x);
            }
        }
        lwCommit();
    };
    // inter-cluster hand-off entries of this lane's line
    const T* zGlobal = a.handoff + ((size_t)cta * nx * kLwTile + jl) * 2;
    // bounded wait; false when it gave up or another warp stopped the sweep
    auto waitFor = [&](auto&& ready) -> bool {
        if (ready()) return true;
        const unsigned long long deadline = lwTimer() + a.waitNs;
        while (!ready()) {
            if (*(volatile int*)&abortFlag) return false;
            if (lwTimer() > deadline) {
                atomicExch(a.err, DXG_ERR_TIMEOUT);
                abortFlag = 1;
                return false;
            }
        }
        return true;
    };

    const bool warpWorks = working && !skip && sy0 + warp * kLwLinesPerWarp < ny;
    if (warpWorks) {
#pragma unroll
        for (int s = 0; s < PF; ++s) issue(s);
        T prev = 0;
        // inter-cluster z values: loaded one step ahead, so the load's latency overlaps the
        // step before (an early load that still saw the empty pattern is repeated)
        T gz0 = lwEmpty<T>(), gz1 = lwEmpty<T>();
        const bool zGlobalIn = hasZUp && !zUpLocal;
        if (zGlobalIn && cellX(0) >= 0) {
            gz0 = lwLdRelaxedGpu(zGlobal + (size_t)cellX(0) * kLwTile * 2);
            gz1 = lwLdRelaxedGpu(zGlobal + (size_t)cellX(0) * kLwTile * 2 + 1);
        }
        for (int s = 0; s < nSteps; ++s) {
            const int L = Lfirst + s;
            const int sx = cellX(s);
            const bool active = sx >= 0;
            lwCpWait<PF - 1>();
            // x neighbour: this line's previous cell (other row from the partner lane); y
            // neighbour: line j-1 at the level before (same row two lanes down, other row from
            // lane 2j-2+(1-r)); three independent shuffles of the previous results
            const T other = __shfl_xor_sync(0xffffffffu, prev, 1);
            const T ySame = __shfl_up_sync(0xffffffffu, prev, 2);
            const T yOther = __shfl_sync(0xffffffffu, prev, (lane - 1 - 2 * r) & 31);
            const T zx0 = r == 0 ? prev : other, zx1 = r == 0 ? other : prev;
            T zy0 = r == 0 ? ySame : yOther, zy1 = r == 0 ? yOther : ySame;
            T zz0 = 0, zz1 = 0;
            bool ok = true;
            if (active && j == 0 && sy > 0 && (warp > 0 || hasYUp)) {
                const T* src = warp > 0 ? ybuf + ((size_t)(warp - 1) * levels + (L - 1)) * 2 : yin + (size_t)(L - 1) * 2;
                ok = waitFor([&] {
                    zy0 = lwLdRelaxedShared(src);
                    zy1 = lwLdRelaxedShared(src + 1);
                    return !lwIsEmpty(zy0) && !lwIsEmpty(zy1);
                });
            }
            if (hasZUp && active) {
                if (zUpLocal) {
                    const T* src = zin + ((size_t)sx * kLwTile + jl) * 2;
                    ok = waitFor([&] {
                        zz0 = lwLdRelaxedShared(src);
                        zz1 = lwLdRelaxedShared(src + 1);
                        return !lwIsEmpty(zz0) && !lwIsEmpty(zz1);
                    }) && ok;
                } else {
                    const T* src = zGlobal + (size_t)sx * kLwTile * 2;
                    zz0 = gz0;
                    zz1 = gz1;
                    if (lwIsEmpty(zz0) || lwIsEmpty(zz1))
                        ok = waitFor([&] {
                            zz0 = lwLdRelaxedGpu(src);
                            zz1 = lwLdRelaxedGpu(src + 1);
                            return !lwIsEmpty(zz0) && !lwIsEmpty(zz1);
                        }) && ok;
                }
            }
            if (zGlobalIn) {
                const int sxn = cellX(s + 1);
                if (sxn >= 0) {
                    gz0 = lwLdRelaxedGpu(zGlobal + (size_t)sxn * kLwTile * 2);
                    gz1 = lwLdRelaxedGpu(zGlobal + (size_t)sxn * kLwTile * 2 + 1);
                }
            }
            if (__any_sync(0xffffffffu, !ok)) break;
            // both lanes of the line hold the inter-cluster values: restore the pattern
            if (zGlobalIn && active && r == 0) {
                T* src = a.handoff + (((size_t)cta * nx + sx) * kLwTile + jl) * 2;
                lwStRelaxedGpu(src, lwEmpty<T>());
                lwStRelaxedGpu(src + 1, lwEmpty<T>());
            }
            const T* rec = ring + ((size_t)(s % PF) * kLwThreads + threadIdx.x) * REC;
            T acc = 0;
            if (active) {
                acc = rec[DIR > 0 ? 6 : 8];
                if (sx > 0) {
                    acc = fma(-rec[0], zx0, acc);
                    acc = fma(-rec[1], zx1, acc);
                }
                if (sy > 0) {
                    acc = fma(-rec[2], zy0, acc);
                    acc = fma(-rec[3], zy1, acc);
                }
                if (sz > 0) {
                    acc = fma(-rec[4], zz0, acc);
                    acc = fma(-rec[5], zz1, acc);
                }
            }
            T res = acc;
            if (DIR < 0) {
                const T accOther = __shfl_xor_sync(0xffffffffu, acc, 1);
                const T a0 = r == 0 ? acc : accOther, a1 = r == 0 ? accOther : acc;
                T t = rec[6] * a0;
                t = fma(rec[7], a1, t);
                res = t;
            }
            if (active) {
                const int64_t i = cellIndex(sx);
                a.v[i * 2 + r] = res;
                if (zDownLocal)
                    lwStRemote<T>(zinDown + (uint32_t)((((size_t)sx * kLwTile + jl) * 2 + r) * sizeof(T)), res);
                else if (hasZDown)
                    lwStRelaxedGpu(a.handoff + (((size_t)zDown * nx + sx) * kLwTile + jl) * 2 + r, res);
                if (j == kLwLinesPerWarp - 1) {
                    if (warp < kLwWarps - 1)
                        lwStRemote<T>(lwSmemAddr(&ybuf[((size_t)warp * levels + L) * 2 + r]), res);
                    else if (hasYDown)
                        lwStRemote<T>(yinDown + (uint32_t)(((size_t)L * 2 + r) * sizeof(T)), res);
                }
                prev = res;
            }
            issue(s + PF);
        }
        lwCpWait<0>();
    }
    // no CTA may leave while another can still write into its shared memory
    cluster.sync();
}

// ---------------------------------------------------------------- host side
namespace {

// One launch of either form (RING 0: registers, laneWaveKernel; 1: shared memory,
// laneRingKernel), or the occupancy query of its launch shape.
template <class T, int DIR, int PF, int RING>
cudaError_t lwLaunchOne(const LanePlan& p, const LaneWaveArgs<T>& a, cudaStream_t st, bool query, int* fits)
{
    void (*kern)(LaneWaveArgs<T>);
    size_t smem;
    const int levels = a.nx + a.ny + a.nz - 2;
    if constexpr (RING != 0) {
        kern = laneRingKernel<T, DIR, PF>;
        smem = lrSmem(a.nx, levels, (int)sizeof(T), LwRec<DIR>::n, PF).total;
    } else {
        kern = laneWaveKernel<T, DIR, PF>;
        smem = lwSmem(a.nx, levels, (int)sizeof(T)).total;
    }
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kLwSmemLimit);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(p.grid);
    cfg.blockDim = dim3(kLwThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[2];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = p.clusterSize;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    // the backward sweep as a programmatic dependent of the forward sweep before it
    cfg.numAttrs = (DIR < 0 && !query) ? 2 : 1;
    if (query) {
        int n = 0;
        e = cudaOccupancyMaxActiveClusters(&n, kern, &cfg);
        *fits = (e == cudaSuccess) ? n : 0;
        if (e != cudaSuccess) cudaGetLastError();
        return cudaSuccess;
    }
    return cudaLaunchKernelEx(&cfg, kern, a);
}

template <class T, int DIR>
cudaError_t lwDispatch(const LanePlan& p, int ring, const LaneWaveArgs<T>& a, cudaStream_t st, bool query, int* fits)
{
    if (ring == 0) {
        if ((DIR > 0 ? p.pfFwd : p.pfBwd) == 4) return lwLaunchOne<T, DIR, 4, 0>(p, a, st, query, fits);
    } else {
        switch (DIR > 0 ? p.pfRingFwd : p.pfRingBwd) {
            case 8: return lwLaunchOne<T, DIR, 8, 1>(p, a, st, query, fits);
            case 4: return lwLaunchOne<T, DIR, 4, 1>(p, a, st, query, fits);
            case 2: return lwLaunchOne<T, DIR, 2, 1>(p, a, st, query, fits);
            default: break;
        }
    }
    if (fits) *fits = 0;
    return query ? cudaSuccess : cudaErrorInvalidConfiguration;
}

// prefetch depth of the shared-memory ring: the deepest of {8, 4, 2} within the budget, else 0
template <class T>
int lrDepth(int nx, int levels, int dir)
{
    for (int pf : {8, 4, 2}) {
        const size_t sm = lrSmem(nx, levels, (int)sizeof(T), dir > 0 ? LwRec<1>::n : LwRec<-1>::n, pf).total;
        if (sm <= kLwSmemLimit) return pf;
    }
    return 0;
}

// every cluster of the launch shape resident at once, for both sweeps of form `ring`
template <class T>
bool lwResident(const LanePlan& p, int ring, const LaneWaveArgs<T>& dummy)
{
    int f1 = 0, f2 = 0;
    lwDispatch<T, 1>(p, ring, dummy, 0, true, &f1);
    lwDispatch<T, -1>(p, ring, dummy, 0, true, &f2);
    return f1 >= p.grid / p.clusterSize && f2 >= p.grid / p.clusterSize;
}

}  // namespace

template <class T>
LanePlan makeLanePlan(int dim, int nx, int ny, int nz, int b)
{
    LanePlan p{};
    if (dim != 3 || b != 2 || nx < 1 || ny < 1 || nz < 1) return p;
    p.nyb = (ny + kLwTile - 1) / kLwTile;
    if (p.nyb > 16) return p;
    p.ctas = nz * p.nyb;
    const int levels = nx + ny + nz - 2;
    if (lwSmem(nx, levels, (int)sizeof(T)).total > kLwSmemLimit) return p;
    // register ring depth 4: measured on GB300 at 64x64x32 (FP64, per apply): 0.195 ms with
    // depth 4, 0.194 ms with 5, 0.201 ms with 3, 0.223 ms with 6 (spills)
    p.pfFwd = 4;
    p.pfBwd = 4;
    p.pfRingFwd = lrDepth<T>(nx, levels, 1);
    p.pfRingBwd = lrDepth<T>(nx, levels, -1);
    LaneWaveArgs<T> dummy{};
    dummy.nx = nx;
    dummy.ny = ny;
    dummy.nz = nz;
    for (int cs : {16, 8, 4, 2, 1}) {
        if (cs % p.nyb != 0) continue;
        p.clusterSize = cs;
        p.grid = (p.ctas + cs - 1) / cs * cs;
        if (lwResident<T>(p, 0, dummy)) {
            p.ok = true;
            p.ringOk = p.pfRingFwd > 0 && p.pfRingBwd > 0 && lwResident<T>(p, 1, dummy);
            return p;
        }
    }
    p.ok = false;
    return p;
}

template <class T>
void launchLaneWaveApply(const LanePlan& p, const LaneWaveArgs<T>& fwd, const LaneWaveArgs<T>& bwd, cudaStream_t st)
{
    const int ring = p.ring == 1 && p.ringOk ? 1 : 0;
    DXG_CUDA((lwDispatch<T, 1>(p, ring, fwd, st, false, nullptr)));
    DXG_CUDA((lwDispatch<T, -1>(p, ring, bwd, st, false, nullptr)));
}

template LanePlan makeLanePlan<double>(int, int, int, int, int);
template LanePlan makeLanePlan<float>(int, int, int, int, int);
template void launchLaneWaveApply<double>(const LanePlan&, const LaneWaveArgs<double>&, const LaneWaveArgs<double>&,
                                          cudaStream_t);
template void launchLaneWaveApply<float>(const LanePlan&, const LaneWaveArgs<float>&, const LaneWaveArgs<float>&,
                                         cudaStream_t);

}  // namespace dxg
