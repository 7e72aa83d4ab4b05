// wave.cu -- natural-order ILU(0) factorisation and triangular solves as one
// thread-block-cluster wavefront kernel per sweep.
//
// The factor and the sweeps of SeqILU (dune-istl, bound by dumux/linear/istlsolvers.hh:
// 535-568) on the cc-TPFA stencil are recurrences over x, y and z: row i needs rows
// i-1, i-nx, i-nx*ny (forward/factor) or i+1, i+nx, i+nx*ny (backward).  Cells with equal
// ix+iy+iz ("level") are independent, so a sweep is a wavefront of nx+ny+nz-2 levels
// whose critical path is one dependent block update per level.
//
// Mapping (measured on GB300: grid barrier ~1.7 us, __syncthreads 10-40 ns, cluster
// shared-memory hand-off ~0.3 us, dependent FP64 FMA 32 ns):
//   * one thread per x-line (y, z): the x recurrence stays in registers, and the
//     cells a thread visits are consecutive in memory, so their matrix blocks are
//     prefetched PF levels ahead into shared memory with cp.async;
//   * the lines are split into contiguous slabs of whole planes (rows in 2D), one
//     slab per CTA of a single cluster of up to 16 CTAs;
//   * inside a CTA one __syncthreads per level; the y/z neighbours' values of the
//     previous level come from shared memory;
//   * the slab's boundary plane is pushed into the next CTA's shared memory with
//     st.async, completing on a per-slot mbarrier of a ring of kRing levels; the next
//     CTA waits on that mbarrier (it lags by a few levels, so it rarely waits).
//     A progress flag written back by the consumer provides back-pressure.
// Every wait has a time limit; on expiry the kernel records DXG_ERR_TIMEOUT and returns.
//
// The arithmetic per cell is the one of the level-scheduled kernels in linalg.cu (same
// operand order), so both give the same factors and sweeps.
#include <algorithm>
#include <climits>
#include <vector>

#include <cooperative_groups.h>

#include "common.cuh"
#include "linalg.cuh"
#include "wave.cuh"

namespace cg = cooperative_groups;

namespace dxg {

constexpr int kRing = 8;
constexpr unsigned long long kWaitNs = 500000000ull;   // default limit of a wait: 0.5 s
constexpr size_t kWaveSmemLimit = 200 * 1024;

__device__ __forceinline__ unsigned long long globalTimer()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ int ldAcquireCluster(const int* p)
{
    int v;
    asm volatile("ld.acquire.cluster.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
// Progress flag of the consumer.  Relaxed: the halo values it read were consumed
// before the CTA barrier that precedes this store, and a release here would make the
// storing thread wait for its own outstanding global stores and prefetches.
__device__ __forceinline__ void stRelaxedCluster(int* p, int v)
{
    asm volatile("st.relaxed.cluster.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint32_t smemAddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ uint32_t mapCluster(uint32_t addr, int rank)
{
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
    return r;
}

// ---- cp.async prefetch (each thread copies and later reads its own records)
template <int BYTES>
__device__ __forceinline__ void cpAsync(uint32_t dst, const void* src)
{
    if (BYTES == 16) asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
    else asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(dst), "l"(src), "n"(BYTES) : "memory");
}
template <class T, int NE>
__device__ __forceinline__ void copyElems(T* dst, const T* src)
{
    constexpr int BYTES = NE * (int)sizeof(T);
    constexpr int CH = (BYTES % 16 == 0) ? 16 : (BYTES % 8 == 0 ? 8 : 4);
    const uint32_t d = smemAddr(dst);
    const char* s = reinterpret_cast<const char*>(src);
#pragma unroll
    for (int o = 0; o < BYTES; o += CH) cpAsync<CH>(d + o, s + o);
}
__device__ __forceinline__ void cpCommit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cpWait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// ---- st.async into a remote CTA's shared memory, completing on its mbarrier
template <class T, int PB>
__device__ __forceinline__ void stAsync(uint32_t dst, const T* v, uint32_t bar)
{
    if constexpr (sizeof(T) == 8) {
        if constexpr (PB == 1) {
            asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.f64 [%0], %1, [%2];" ::"r"(dst),
                         "d"((double)v[0]), "r"(bar) : "memory");
        } else {
#pragma unroll
            for (int k = 0; k < PB; k += 2)
                asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v2.f64 [%0], {%1, %2}, [%3];" ::"r"(
                                 dst + 8 * k),
                             "d"((double)v[k]), "d"((double)v[k + 1]), "r"(bar) : "memory");
        }
    } else {
        if constexpr (PB == 1) {
            asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.f32 [%0], %1, [%2];" ::"r"(dst),
                         "f"((float)v[0]), "r"(bar) : "memory");
        } else if constexpr (PB == 2) {
            asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v2.f32 [%0], {%1, %2}, [%3];" ::"r"(dst),
                         "f"((float)v[0]), "f"((float)v[1]), "r"(bar) : "memory");
        } else {
            asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.f32 [%0], {%1, %2, %3, %4}, [%5];" ::"r"(
                             dst),
                         "f"((float)v[0]), "f"((float)v[1]), "f"((float)v[2]), "f"((float)v[3]), "r"(bar) : "memory");
        }
    }
}
__device__ __forceinline__ void mbarInit(uint32_t bar, int count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
// Relaxed arrive: this arrival publishes nothing; the payload bytes complete the phase.
__device__ __forceinline__ void mbarExpectTx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.relaxed.cta.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbarTryWait(uint32_t bar, uint32_t parity)
{
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    return done != 0;
}

template <int B, class T>
__device__ __forceinline__ void mmul(const T* X, const T* Y, T* Z)
{
    // explicit fused multiply-adds: every instantiation of the kernels (launch shapes,
    // single and batched) rounds the same way, whatever contraction the compiler chooses
#pragma unroll
    for (int r = 0; r < B; ++r)
#pragma unroll
        for (int c = 0; c < B; ++c) {
            T s = 0;
#pragma unroll
            for (int k = 0; k < B; ++k) s = fma(X[r * B + k], Y[k * B + c], s);
            Z[r * B + c] = s;
        }
}
template <int B, class T>
__device__ __forceinline__ bool minv(const T* A, T* inv)
{
    if (B == 1) {
        inv[0] = (T)1 / A[0];
        return A[0] != (T)0;
    } else {
        const T p12 = A[1] * A[2];
        const T det = fma(A[0], A[3], -p12);
        if (det == (T)0) return false;
        const T detInv = (T)1 / det;
        inv[0] = A[3] * detInv;
        inv[1] = -A[1] * detInv;
        inv[2] = -A[2] * detInv;
        inv[3] = A[0] * detInv;
        return true;
    }
}

// Elements per prefetched cell record (padded to 16 bytes).
template <int B, class T, int DIM, int DIR, int MODE>
struct Rec {
    static constexpr int BB = B * B;
    static constexpr int raw = MODE == 1 ? (2 * DIM + 1) * BB : (DIR > 0 ? DIM * BB + B : DIM * BB + BB + B);
    static constexpr int align = 16 / (int)sizeof(T);
    static constexpr int n = (raw + align - 1) / align * align;
};

// Cells of a hand-off plane (3D: plane zb, all y) or row (2D: row yb) that exist at
// level L.  Producer and consumer both use it to size the transfers of a level.
__host__ __device__ inline int activeCount(int L, int zb, int nx, int ny, int dim, int yb)
{
    if (dim == 3) {
        const int lo = max(0, L - zb - nx + 1), hi = min(ny - 1, L - zb);
        return hi >= lo ? hi - lo + 1 : 0;
    }
    const int x = L - yb;
    return (x >= 0 && x < nx) ? 1 : 0;
}

// byte offset of the prefetch ring behind zbuf [2][LPC] and halo [kRing][H] payloads
__host__ __device__ inline size_t pfOffset(int LPC, int H, int payloadBytes)
{
    const size_t b = (2 * (size_t)LPC + (size_t)kRing * H) * payloadBytes;
    return (b + 15) & ~(size_t)15;
}

// z -= blk * x as a chain of FMAs (row r: acc_r - b_r0 x_0 - b_r1 x_1)
template <int B, class T>
__device__ __forceinline__ void fmaSub(const T* blk, const T* x, T* acc)
{
#pragma unroll
    for (int r = 0; r < B; ++r)
#pragma unroll
        for (int c = 0; c < B; ++c) acc[r] = fma(-blk[r * B + c], x[c], acc[r]);
}

// Per-line state, computed once per launch (no divisions in the level loop).
struct LineState {
    int64_t base;      // cell index of x = 0
    int yz;            // y + z: the line's cell x sits on level x + yz
    int nbY, nbZ;      // zbuf index (>= 0) or halo index (-1 - hidx) of the y / z neighbour line, or INT_MIN
    int outIdx;        // halo index in the downstream CTA (>= 0) or -1
    int ll;            // local line index (-1: no line)
};

// MODE 0: solve (forward DIR=+1 with L, backward DIR=-1 with U=A_upper and Dinv)
// MODE 1: factorisation (DIR=+1): writes L and Dinv
//
// Batched launch (batch != nullptr): cluster k of the grid sweeps problem k; CTAs whose
// rank is at or beyond that problem's slab count only take part in the two cluster
// barriers.
template <int B, class T, int DIM, int DIR, int MODE, int PF>
__global__ void __launch_bounds__(1024) waveKernel(WaveArgs<T> a0, const WaveArgs<T>* batch)
{
    constexpr int PB = MODE == 1 ? B * B : B;
    constexpr int BB = B * B;
    constexpr int REC = Rec<B, T, DIM, DIR, MODE>::n;
    constexpr int kMaxLpt = 2;
    constexpr int kNone = INT_MIN;
    extern __shared__ __align__(16) unsigned char smemRaw[];
    __shared__ __align__(8) unsigned long long fullBar[kRing];
    __shared__ int consumerDone;    // written remotely by the downstream CTA
    __shared__ int abortFlag;

    cg::cluster_group cluster = cg::this_cluster();
    const int cta = (int)cluster.block_rank();
    const WaveArgs<T> a = batch ? batch[blockIdx.x / cluster.num_blocks()] : a0;
    if (cta >= a.ctas) {
        // idle CTA of a batched launch: nothing to sweep, no hand-off partner
        cluster.sync();
        cluster.sync();
        return;
    }
    const int C = a.ctas;
    const int LPC = a.linesPerCta;
    const int H = a.haloLines;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const int64_t N = a.N;
    const int nLines = ny * nz;
    const int nthr = blockDim.x;
    const int lpt = (LPC + nthr - 1) / nthr;

    T* zbuf = reinterpret_cast<T*>(smemRaw);                        // [2][LPC][PB]
    T* halo = zbuf + 2 * (size_t)LPC * PB;                           // [kRing][H][PB]
    // [PF][nthr*lpt][REC], 16-byte aligned for cp.async
    T* pf = reinterpret_cast<T*>(smemRaw + pfOffset(LPC, H, PB * (int)sizeof(T)));

    auto lineRange = [&](int c, int& lb, int& le) {
        lb = c * LPC;
        le = min(nLines, lb + LPC);
    };
    auto levelRange = [&](int c, int& yzMin, int& yzMax) {
        int lb, le;
        lineRange(c, lb, le);
        const int zf = lb / ny, zl = (le - 1) / ny;
        yzMin = zf + (zf == zl ? lb % ny : 0);
        yzMax = zl + (zf == zl ? (le - 1) % ny : ny - 1);
    };
    const int Lmax = nx - 1 + ny - 1 + nz - 1;
    auto gOfL = [&](int L) { return DIR > 0 ? L : Lmax - L; };
    auto firstGstep = [&](int c) {
        int mn, mx;
        levelRange(c, mn, mx);
        return DIR > 0 ? mn : Lmax - (mx + nx - 1);
    };

    int l0, l1;
    lineRange(cta, l0, l1);
    const int nLoc = l1 - l0;
    const int up = DIR > 0 ? cta - 1 : cta + 1;
    const int down = DIR > 0 ? cta + 1 : cta - 1;
    const bool hasUp = up >= 0 && up < C;
    const bool hasDown = down >= 0 && down < C;
    // hand-off plane (3D) / row (2D) received from upstream and sent downstream
    int zbIn = 0, ybIn = 0, zbOut = 0, ybOut = 0;
    if (DIM == 3) {
        zbIn = DIR > 0 ? l0 / ny - 1 : l1 / ny;
        zbOut = DIR > 0 ? (l1 - 1) / ny : l0 / ny;
    } else {
        ybIn = DIR > 0 ? l0 - 1 : l1;
        ybOut = DIR > 0 ? l1 - 1 : l0;
    }
    // first gstep with incoming data: the mbarrier phase parity counts from there
    const int gInFirst = DIR > 0 ? gOfL(DIM == 3 ? zbIn : ybIn)
                                 : gOfL((nx - 1) + (DIM == 3 ? ny - 1 + zbIn : ybIn));

    if (threadIdx.x == 0) {
        for (int k = 0; k < kRing; ++k) mbarInit(smemAddr(&fullBar[k]), 1);
        // ring slots of steps before the consumer's first step are never read
        consumerDone = hasDown ? firstGstep(down) - 1 : -1;
        abortFlag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    cluster.sync();
    const bool skip = (MODE == 0 && a.ks && a.ks->status != KS_RUNNING);
    int* upConsumed = hasUp ? cluster.map_shared_rank(&consumerDone, up) : nullptr;
    const uint32_t haloDownBase = hasDown ? mapCluster(smemAddr(halo), down) : 0u;
    const uint32_t barDownBase = hasDown ? mapCluster(smemAddr(&fullBar[0]), down) : 0u;

    int yzMin, yzMax;
    levelRange(cta, yzMin, yzMax);
    const int Lfirst = DIR > 0 ? yzMin : yzMax + nx - 1;
    const int nSteps = (yzMax + nx - 1 - yzMin) + 1;

    // slots: lower -z,-y,-x = 0..DIM-1 (column order), diag = DIM, upper +x,+y,+z
    constexpr int sDiag = DIM;
    constexpr int sMx = DIM - 1, sMy = DIM - 2, sMz = DIM - 3;
    constexpr int sPx = DIM + 1, sPy = DIM + 2, sPz = DIM + 3;
    const int64_t planeStride = (int64_t)nx * ny;

    // line states
    LineState ls[kMaxLpt];
    bool needsHalo = false;   // some line of this thread reads the incoming hand-off
#pragma unroll
    for (int k = 0; k < kMaxLpt; ++k) {
        const int ll = threadIdx.x + k * nthr;
        LineState& st = ls[k];
        st.ll = -1;
        st.nbY = st.nbZ = kNone;
        st.outIdx = -1;
        if (k >= lpt || ll >= nLoc) continue;
        const int l = l0 + ll;
        const int y = l % ny, z = l / ny;
        st.ll = ll;
        st.base = (int64_t)nx * l;
        st.yz = y + z;
        const bool hy = DIR > 0 ? y > 0 : y < ny - 1;
        const bool hz = DIM == 3 && (DIR > 0 ? z > 0 : z < nz - 1);
        const int ly = DIR > 0 ? ll - 1 : ll + 1;
        const int lz = DIR > 0 ? ll - ny : ll + ny;
        if (hy) st.nbY = (ly >= 0 && ly < nLoc) ? ly : -1 - (DIR > 0 ? ly + H : ly - nLoc);
        if (hz) st.nbZ = (lz >= 0 && lz < nLoc) ? lz : -1 - (DIR > 0 ? lz + H : lz - nLoc);
        if ((st.nbY != kNone && st.nbY < 0) || (st.nbZ != kNone && st.nbZ < 0)) needsHalo = true;
        if (hasDown && (DIR > 0 ? ll >= nLoc - H : ll < H)) st.outIdx = DIR > 0 ? ll - (nLoc - H) : ll;
    }

    T prev[kMaxLpt][PB];
#pragma unroll
    for (int k = 0; k < kMaxLpt; ++k)
#pragma unroll
        for (int e = 0; e < PB; ++e) prev[k][e] = 0;

    // The matrix blocks and vector entries of this thread's cell of step s on line k:
    // visit(offset in the record, source, number of elements) -- blocks (BB) or vectors (B)
    constexpr bool RING = PF > 0;      // PF == 0: no shared-memory ring (direct loads)
    constexpr int PFR = RING ? PF : 1;
    constexpr int PD = 8;              // direct loads: L1 prefetch distance in levels
    auto forCell = [&](int s, int k, auto&& visitBlk, auto&& visitVec) {
        if (s >= nSteps) return;
        const LineState& st = ls[k];
        if (st.ll < 0) return;
        const int L = DIR > 0 ? Lfirst + s : Lfirst - s;
        const int x = L - st.yz;
        if ((unsigned)x >= (unsigned)nx) return;
        const int64_t i = st.base + x;
        const bool vx = DIR > 0 ? x > 0 : x < nx - 1;
        const bool vy = st.nbY != kNone, vz = st.nbZ != kNone;
        if (MODE == 1) {
            if (DIM == 3 && vz) {
                visitBlk(sMz * BB, a.A + ((int64_t)sMz * N + i) * BB);
                visitBlk((DIM + 1 + sMz) * BB, a.A + ((int64_t)(2 * DIM - sMz) * N + i - planeStride) * BB);
            }
            if (vy) {
                visitBlk(sMy * BB, a.A + ((int64_t)sMy * N + i) * BB);
                visitBlk((DIM + 1 + sMy) * BB, a.A + ((int64_t)(2 * DIM - sMy) * N + i - nx) * BB);
            }
            if (vx) {
                visitBlk(sMx * BB, a.A + ((int64_t)sMx * N + i) * BB);
                visitBlk((DIM + 1 + sMx) * BB, a.A + ((int64_t)(2 * DIM - sMx) * N + i - 1) * BB);
            }
            visitBlk(DIM * BB, a.A + ((int64_t)sDiag * N + i) * BB);
        } else if (DIR > 0) {
            if (DIM == 3 && vz) visitBlk(sMz * BB, a.L + ((int64_t)sMz * N + i) * BB);
            if (vy) visitBlk(sMy * BB, a.L + ((int64_t)sMy * N + i) * BB);
            if (vx) visitBlk(sMx * BB, a.L + ((int64_t)sMx * N + i) * BB);
            visitVec(DIM * BB, a.rhs + i * B);
        } else {
            if (vx) visitBlk(0 * BB, a.A + ((int64_t)sPx * N + i) * BB);
            if (vy) visitBlk(1 * BB, a.A + ((int64_t)sPy * N + i) * BB);
            if (DIM == 3 && vz) visitBlk(2 * BB, a.A + ((int64_t)sPz * N + i) * BB);
            visitBlk(DIM * BB, a.Dinv + i * BB);
            visitVec(DIM * BB + BB, a.v + i * B);
        }
    };
    // ring: copy the cells of step s into ring slot s % PF with cp.async;
    // direct: prefetch the cells PD levels ahead into L1
    auto issue = [&](int s) {
        if constexpr (RING) {
#pragma unroll
            for (int k = 0; k < kMaxLpt; ++k) {
                T* rec = pf + ((size_t)(s & (PFR - 1)) * nthr * lpt + k * nthr + threadIdx.x) * REC;
                forCell(
                    s, k, [&](int off, const T* src) { copyElems<T, BB>(rec + off, src); },
                    [&](int off, const T* src) { copyElems<T, B>(rec + off, src); });
            }
            cpCommit();
        } else {
            // called with s = step + 1: the cells PD levels ahead of the current step
            auto pre = [&](int, const T* src) { asm volatile("prefetch.global.L1 [%0];" ::"l"(src)); };
#pragma unroll
            for (int k = 0; k < kMaxLpt; ++k) forCell(s + PD - 1, k, pre, pre);
        }
    };

    if (!skip) {
        if constexpr (RING) {
#pragma unroll
            for (int s = 0; s < PFR; ++s) issue(s);
        } else {
            // warm L1 with the first PD levels
            auto pre = [&](int, const T* src) { asm volatile("prefetch.global.L1 [%0];" ::"l"(src)); };
            for (int s = 0; s < PD; ++s)
#pragma unroll
                for (int k = 0; k < kMaxLpt; ++k) forCell(s, k, pre, pre);
        }
    }

    int roomSeen = INT_MIN;   // last consumer progress observed by this thread
    for (int step = 0; step < nSteps && !skip; ++step) {
        const int L = DIR > 0 ? Lfirst + step : Lfirst - step;
        const int gstep = gOfL(L);
        const int par = step & 1;
        T* zcur = zbuf + (size_t)par * LPC * PB;
        const T* zold = zbuf + (size_t)(par ^ 1) * LPC * PB;
        // incoming hand-off: the upstream boundary at the previous level
        const int gIn = gstep - 1;
        const T* hold = halo + (size_t)(gIn & (kRing - 1)) * H * PB;
        const uint32_t barIn = smemAddr(&fullBar[gIn & (kRing - 1)]);
        if (hasUp && threadIdx.x == 0) {
            const int cntIn = activeCount(DIR > 0 ? L - 1 : L + 1, zbIn, nx, ny, DIM, ybIn);
            if (cntIn > 0) mbarExpectTx(barIn, (uint32_t)(cntIn * PB * sizeof(T)));
        }
        bool haveHalo = !needsHalo;
        bool roomChecked = false;

        if constexpr (RING) cpWait<PFR - 1>();
#pragma unroll
        for (int k = 0; k < kMaxLpt; ++k) {
            const LineState& st = ls[k];
            if (st.ll < 0) continue;
            const int x = L - st.yz;
            if ((unsigned)x >= (unsigned)nx) continue;
            const int64_t i = st.base + x;
            T recLocal[RING ? 1 : REC];
            const T* rec;
            if constexpr (RING) {
                rec = pf + ((size_t)(step & (PFR - 1)) * nthr * lpt + k * nthr + threadIdx.x) * REC;
            } else {
                // direct loads (L1, filled by the prefetches); v is written in place by the
                // backward sweep, by this thread only, after this read
                forCell(
                    step, k,
                    [&](int off, const T* src) {
#pragma unroll
                        for (int e = 0; e < BB; ++e) recLocal[off + e] = src[e];
                    },
                    [&](int off, const T* src) {
#pragma unroll
                        for (int e = 0; e < B; ++e) recLocal[off + e] = src[e];
                    });
                rec = recLocal;
            }
            const bool hx = DIR > 0 ? x > 0 : x < nx - 1;
            if (!haveHalo && ((st.nbY != kNone && st.nbY < 0) || (st.nbZ != kNone && st.nbZ < 0))) {
                const uint32_t parity = (uint32_t)(((gIn - gInFirst) / kRing) & 1);
                if (!mbarTryWait(barIn, parity)) {
                    const unsigned long long deadline = globalTimer() + (a.waitNs ? a.waitNs : kWaitNs);
                    bool ok = false;
                    while (!(ok = mbarTryWait(barIn, parity))) {
                        if (*(volatile int*)&abortFlag) break;
                        if (globalTimer() > deadline) {
                            atomicExch(a.err, DXG_ERR_TIMEOUT);
                            abortFlag = 1;
                            break;
                        }
                    }
                    if (!ok) break;
                }
                haveHalo = true;
            }
            auto payload = [&](int nb, T* out) {
                const T* src = nb >= 0 ? zold + (size_t)nb * PB : hold + (size_t)(-1 - nb) * PB;
#pragma unroll
                for (int e = 0; e < PB; ++e) out[e] = src[e];
            };
            T res[PB];
            if (MODE == 1) {
                T D[BB];
#pragma unroll
                for (int e = 0; e < BB; ++e) D[e] = rec[DIM * BB + e];
                auto lowerTerm = [&](int s, const T* Dj) {
                    T Lij[BB], P[BB];
                    mmul<B>(rec + s * BB, Dj, Lij);
#pragma unroll
                    for (int e = 0; e < BB; ++e) a.L[((int64_t)s * N + i) * BB + e] = Lij[e];
                    mmul<B>(Lij, rec + (DIM + 1 + s) * BB, P);
#pragma unroll
                    for (int e = 0; e < BB; ++e) D[e] -= P[e];
                };
                auto zeroL = [&](int s) {
#pragma unroll
                    for (int e = 0; e < BB; ++e) a.L[((int64_t)s * N + i) * BB + e] = 0;
                };
                if (DIM == 3) {
                    if (st.nbZ != kNone) { T Dz[PB]; payload(st.nbZ, Dz); lowerTerm(sMz, Dz); }
                    else zeroL(sMz);
                }
                if (st.nbY != kNone) { T Dy[PB]; payload(st.nbY, Dy); lowerTerm(sMy, Dy); }
                else zeroL(sMy);
                if (hx) lowerTerm(sMx, prev[k]);
                else zeroL(sMx);
                if (!minv<B>(D, res)) atomicExch(a.singular, 1);
#pragma unroll
                for (int e = 0; e < BB; ++e) a.Dinv[i * BB + e] = res[e];
            } else if (DIR > 0) {
                // z_i = d_i - L_ix z_x - L_iy z_y - L_iz z_z
#pragma unroll
                for (int e = 0; e < B; ++e) res[e] = rec[DIM * BB + e];
                if (hx) fmaSub<B>(rec + sMx * BB, prev[k], res);
                if (st.nbY != kNone) { T v[PB]; payload(st.nbY, v); fmaSub<B>(rec + sMy * BB, v, res); }
                if (DIM == 3 && st.nbZ != kNone) { T v[PB]; payload(st.nbZ, v); fmaSub<B>(rec + sMz * BB, v, res); }
#pragma unroll
                for (int e = 0; e < B; ++e) a.v[i * B + e] = res[e];
            } else {
                // y_i = D_i^{-1} (z_i - U_ix y_x - U_iy y_y - U_iz y_z)
                T acc[B];
#pragma unroll
                for (int e = 0; e < B; ++e) acc[e] = rec[DIM * BB + BB + e];
                if (hx) fmaSub<B>(rec + 0 * BB, prev[k], acc);
                if (st.nbY != kNone) { T v[PB]; payload(st.nbY, v); fmaSub<B>(rec + 1 * BB, v, acc); }
                if (DIM == 3 && st.nbZ != kNone) { T v[PB]; payload(st.nbZ, v); fmaSub<B>(rec + 2 * BB, v, acc); }
                const T* Di = rec + DIM * BB;
#pragma unroll
                for (int r = 0; r < B; ++r) {
                    T t = Di[r * B] * acc[0];
#pragma unroll
                    for (int c = 1; c < B; ++c) t = fma(Di[r * B + c], acc[c], t);
                    res[r] = t;
                }
#pragma unroll
                for (int e = 0; e < B; ++e) a.v[i * B + e] = res[e];
            }
#pragma unroll
            for (int e = 0; e < PB; ++e) {
                prev[k][e] = res[e];
                zcur[(size_t)st.ll * PB + e] = res[e];
            }
            // boundary lines feed the next CTA in sweep direction
            if (st.outIdx >= 0) {
                if (!roomChecked) {
                    // slot gstep%kRing was last read by the consumer at its step gstep-kRing+1;
                    // the consumer's progress only grows, so a value seen earlier that
                    // already covers the target needs no new load
                    const int target = gstep - kRing + 1;
                    if (roomSeen < target && (roomSeen = ldAcquireCluster(&consumerDone)) < target) {
                        const unsigned long long deadline = globalTimer() + (a.waitNs ? a.waitNs : kWaitNs);
                        bool ok = true;
                        while ((roomSeen = ldAcquireCluster(&consumerDone)) < target) {
                            if (*(volatile int*)&abortFlag) { ok = false; break; }
                            if (globalTimer() > deadline) {
                                atomicExch(a.err, DXG_ERR_TIMEOUT);
                                abortFlag = 1;
                                ok = false;
                                break;
                            }
                        }
                        if (!ok) break;
                    }
                    roomChecked = true;
                }
                const uint32_t slot = (uint32_t)(gstep & (kRing - 1));
                const uint32_t dst = haloDownBase + (uint32_t)(((slot * H + st.outIdx) * PB) * sizeof(T));
                stAsync<T, PB>(dst, res, barDownBase + slot * 8u);
            }
        }
        // prefetch the cells PF levels ahead into the slot consumed by this step
        // (direct: prefetch PD levels ahead into L1)
        issue(step + PFR);
        __syncthreads();
        if (abortFlag) break;
        if (threadIdx.x == 0 && hasUp) stRelaxedCluster(upConsumed, gstep);
    }
    if constexpr (RING) cpWait<0>();
    // no CTA may leave while others can still write into its shared memory
    cluster.sync();
    if (abortFlag) {
        // in-flight hand-offs of an aborted sweep land within microseconds
        const unsigned long long until = globalTimer() + 200000ull;
        while (globalTimer() < until) {
        }
    }
}

// ---------------------------------------------------------------- bounded-wait self-test
// The waits of the sweeps, on conditions nothing ever satisfies: an mbarrier phase that
// never completes (KIND 0) or a global flag nobody sets (KIND 1).  Each waits at most
// limitNs, then records DXG_ERR_TIMEOUT and the time it waited, and returns.
__global__ void boundedWaitSelfTest(int kind, unsigned long long limitNs, const int* flag, int* status,
                                    unsigned long long* waitedNs)
{
    __shared__ __align__(8) unsigned long long bar;
    if (threadIdx.x == 0) {
        mbarInit(smemAddr(&bar), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const unsigned long long t0 = globalTimer();
    const unsigned long long deadline = t0 + limitNs;
    bool done = false;
    while (!done) {
        if (kind == 0) done = mbarTryWait(smemAddr(&bar), 0);
        else done = *(volatile const int*)flag != 0;
        if (!done && globalTimer() > deadline) break;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        *status = done ? DXG_OK : DXG_ERR_TIMEOUT;
        *waitedNs = globalTimer() - t0;
    }
}

int runBoundedWaitSelfTest(int kind, long long limitNs, int* kernelStatus, double* waitedMs)
{
    int* dStatus = nullptr;
    int* dFlag = nullptr;
    unsigned long long* dWaited = nullptr;
    int rc = DXG_OK;
    if (cudaMalloc(&dStatus, sizeof(int)) != cudaSuccess || cudaMalloc(&dFlag, sizeof(int)) != cudaSuccess ||
        cudaMalloc(&dWaited, sizeof(unsigned long long)) != cudaSuccess)
        rc = DXG_ERR_OOM;
    if (rc == DXG_OK && cudaMemset(dFlag, 0, sizeof(int)) != cudaSuccess) rc = DXG_ERR_CUDA;
    if (rc == DXG_OK && cudaMemset(dStatus, 0xff, sizeof(int)) != cudaSuccess) rc = DXG_ERR_CUDA;
    if (rc == DXG_OK) {
        boundedWaitSelfTest<<<1, 32>>>(kind, (unsigned long long)limitNs, dFlag, dStatus, dWaited);
        if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) rc = DXG_ERR_CUDA;
    }
    unsigned long long waited = 0;
    if (rc == DXG_OK &&
        (cudaMemcpy(kernelStatus, dStatus, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess ||
         cudaMemcpy(&waited, dWaited, sizeof(waited), cudaMemcpyDeviceToHost) != cudaSuccess))
        rc = DXG_ERR_CUDA;
    if (waitedMs) *waitedMs = waited / 1e6;
    cudaFree(dStatus);
    cudaFree(dFlag);
    cudaFree(dWaited);
    return rc;
}

// ---------------------------------------------------------------- host side
template <int B, class T, int DIR, int MODE>
static size_t waveSmemFor(int dim, int linesPerCta, int haloLines, int threads, int pfDepth)
{
    constexpr int PB = MODE == 1 ? B * B : B;
    const int rec = dim == 3 ? Rec<B, T, 3, DIR, MODE>::n : Rec<B, T, 2, DIR, MODE>::n;
    const int lpt = (linesPerCta + threads - 1) / threads;
    return pfOffset(linesPerCta, haloLines, PB * (int)sizeof(T)) + (size_t)pfDepth * threads * lpt * rec * sizeof(T);
}

// Uniform shape of one launch: `clusters` clusters of `ctas` CTAs.
struct WaveLaunch {
    int clusters, ctas, threads, pf;
    size_t smem;
};

template <int B, class T, int DIM, int DIR, int MODE, int PF>
static cudaError_t launchOne(const WaveLaunch& L, const WaveArgs<T>& a, const WaveArgs<T>* batch, cudaStream_t st,
                             bool query, int* fits)
{
    auto kern = waveKernel<B, T, DIM, DIR, MODE, PF>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kWaveSmemLimit);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(L.clusters * L.ctas);
    cfg.blockDim = dim3(L.threads);
    cfg.dynamicSmemBytes = L.smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = L.ctas;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (query) {
        int n = 0;
        e = cudaOccupancyMaxActiveClusters(&n, kern, &cfg);
        *fits = (e == cudaSuccess && n > 0) ? n : 0;
        if (e != cudaSuccess) cudaGetLastError();
        return cudaSuccess;
    }
    return cudaLaunchKernelEx(&cfg, kern, a, batch);
}

template <int B, class T, int DIM, int DIR, int MODE>
static cudaError_t dispatchPF(const WaveLaunch& L, const WaveArgs<T>& a, const WaveArgs<T>* batch, cudaStream_t st,
                              bool query, int* fits)
{
    switch (L.pf) {
        case 8: return launchOne<B, T, DIM, DIR, MODE, 8>(L, a, batch, st, query, fits);
        case 4: return launchOne<B, T, DIM, DIR, MODE, 4>(L, a, batch, st, query, fits);
        case 2: return launchOne<B, T, DIM, DIR, MODE, 2>(L, a, batch, st, query, fits);
        case 1: return launchOne<B, T, DIM, DIR, MODE, 1>(L, a, batch, st, query, fits);
        case 0: return launchOne<B, T, DIM, DIR, MODE, 0>(L, a, batch, st, query, fits);
        default:
            if (fits) *fits = 0;
            return query ? cudaSuccess : cudaErrorInvalidConfiguration;
    }
}

template <int B, class T, int DIR, int MODE>
static cudaError_t dispatch(const WaveLaunch& L, int dim, const WaveArgs<T>& a, const WaveArgs<T>* batch,
                            cudaStream_t st, bool query, int* fits)
{
    return dim == 3 ? dispatchPF<B, T, 3, DIR, MODE>(L, a, batch, st, query, fits)
                    : dispatchPF<B, T, 2, DIR, MODE>(L, a, batch, st, query, fits);
}

// prefetch depth of a single-problem launch: the deepest of {8, 4, 2, 1} within the
// shared-memory budget, else 0 (no ring); pf stays -1 (refused by the dispatch) when not
// even the ring-free layout fits
template <int B, class T, int DIR, int MODE>
static WaveLaunch singleLaunch(const WavePlan& p, int dim)
{
    WaveLaunch L{1, p.ctas, p.threads, -1, 0};
    for (int d : {8, 4, 2, 1, 0}) {
        const size_t sm = waveSmemFor<B, T, DIR, MODE>(dim, p.linesPerCta, p.haloLines, p.threads, d);
        if (sm <= kWaveSmemLimit) {
            L.pf = d;
            L.smem = sm;
            break;
        }
    }
    return L;
}

template <int B, class T>
static bool planFits(const WavePlan& p, int dim)
{
    WaveArgs<T> dummy{};
    int f1 = 0, f2 = 0, f3 = 0;
    dispatch<B, T, 1, 0>(singleLaunch<B, T, 1, 0>(p, dim), dim, dummy, nullptr, 0, true, &f1);
    dispatch<B, T, -1, 0>(singleLaunch<B, T, -1, 0>(p, dim), dim, dummy, nullptr, 0, true, &f2);
    dispatch<B, T, 1, 1>(singleLaunch<B, T, 1, 1>(p, dim), dim, dummy, nullptr, 0, true, &f3);
    return f1 && f2 && f3;
}

WaveGeom waveGeom(int dim, int nx, int ny, int nz, int maxCtas)
{
    WaveGeom g{};
    const int unit = dim == 3 ? ny : 1;                 // lines per plane of the slab axis
    const int units = dim == 3 ? nz : ny;
    if (units <= 0 || nx <= 0 || maxCtas <= 0) return g;
    int ctas = std::min(maxCtas, units);
    const int per = (units + ctas - 1) / ctas;
    ctas = (units + per - 1) / per;
    g.ctas = ctas;
    g.linesPerCta = per * unit;
    g.haloLines = dim == 3 ? ny : 1;
    return g;
}

static WavePlan planFor(int dim, int nx, int ny, int nz, int maxCtas)
{
    WavePlan p{};
    const WaveGeom g = waveGeom(dim, nx, ny, nz, maxCtas);
    if (g.ctas == 0) return p;
    p.ctas = g.ctas;
    p.linesPerCta = g.linesPerCta;
    p.haloLines = g.haloLines;
    const int threads = std::min(1024, ((p.linesPerCta + 31) / 32) * 32);
    p.lpt = (p.linesPerCta + threads - 1) / threads;
    p.threads = threads;
    p.ok = p.lpt <= 2;
    return p;
}

std::vector<WavePlan> wavePlanCandidates(int dim, int nx, int ny, int nz, int b, bool fp64)
{
    std::vector<WavePlan> out;
    for (int maxCtas = 16; maxCtas >= 1; maxCtas /= 2) {
        WavePlan p = planFor(dim, nx, ny, nz, maxCtas);
        if (!p.ok) continue;
        bool fits;
        if (b == 1) fits = fp64 ? planFits<1, double>(p, dim) : planFits<1, float>(p, dim);
        else fits = fp64 ? planFits<2, double>(p, dim) : planFits<2, float>(p, dim);
        if (!fits) continue;
        bool dup = false;
        for (const WavePlan& q : out) dup = dup || q.ctas == p.ctas;
        if (!dup) out.push_back(p);
    }
    return out;
}

WavePlan makeWavePlan(int dim, int nx, int ny, int nz, int b, bool fp64)
{
    const std::vector<WavePlan> c = wavePlanCandidates(dim, nx, ny, nz, b, fp64);
    return c.empty() ? WavePlan{} : c.front();
}

template <class T>
void launchWaveFactor(const WavePlan& plan, const WaveArgs<T>& a, int b, cudaStream_t st)
{
    const cudaError_t e = b == 1 ? dispatch<1, T, 1, 1>(singleLaunch<1, T, 1, 1>(plan, a.dim), a.dim, a, nullptr, st,
                                                        false, nullptr)
                                 : dispatch<2, T, 1, 1>(singleLaunch<2, T, 1, 1>(plan, a.dim), a.dim, a, nullptr, st,
                                                        false, nullptr);
    DXG_CUDA(e);
}
template <class T>
void launchWaveApply(const WavePlan& plan, const WaveArgs<T>& fwd, const WaveArgs<T>& bwd, int b, cudaStream_t st)
{
    const int dim = fwd.dim;
    if (b == 1) {
        DXG_CUDA((dispatch<1, T, 1, 0>(singleLaunch<1, T, 1, 0>(plan, dim), dim, fwd, nullptr, st, false, nullptr)));
        DXG_CUDA((dispatch<1, T, -1, 0>(singleLaunch<1, T, -1, 0>(plan, dim), dim, bwd, nullptr, st, false, nullptr)));
    } else {
        DXG_CUDA((dispatch<2, T, 1, 0>(singleLaunch<2, T, 1, 0>(plan, dim), dim, fwd, nullptr, st, false, nullptr)));
        DXG_CUDA((dispatch<2, T, -1, 0>(singleLaunch<2, T, -1, 0>(plan, dim), dim, bwd, nullptr, st, false, nullptr)));
    }
}

// ---------------------------------------------------------------- batched launches
// Shared memory of a batched launch of kernel (DIR, MODE): the largest problem's need.
template <int B, class T, int DIR, int MODE>
static size_t batchSmem(const WaveBatchPlan& p, const std::vector<WaveGeom>& geoms, int dim)
{
    size_t mx = 0;
    for (const WaveGeom& g : geoms)
        mx = std::max(mx, waveSmemFor<B, T, DIR, MODE>(dim, g.linesPerCta, g.haloLines, p.threads, p.pf));
    return mx;
}

template <int B, class T>
static int batchFits(WaveBatchPlan& p, const std::vector<WaveGeom>& geoms, int dim, int count)
{
    p.smemFwd = batchSmem<B, T, 1, 0>(p, geoms, dim);
    p.smemBwd = batchSmem<B, T, -1, 0>(p, geoms, dim);
    p.smemFactor = batchSmem<B, T, 1, 1>(p, geoms, dim);
    if (std::max(p.smemFwd, std::max(p.smemBwd, p.smemFactor)) > kWaveSmemLimit) return 0;
    WaveArgs<T> dummy{};
    int f1 = 0, f2 = 0, f3 = 0;
    dispatch<B, T, 1, 0>(WaveLaunch{count, p.ctas, p.threads, p.pf, p.smemFwd}, dim, dummy, nullptr, 0, true, &f1);
    dispatch<B, T, -1, 0>(WaveLaunch{count, p.ctas, p.threads, p.pf, p.smemBwd}, dim, dummy, nullptr, 0, true, &f2);
    dispatch<B, T, 1, 1>(WaveLaunch{count, p.ctas, p.threads, p.pf, p.smemFactor}, dim, dummy, nullptr, 0, true, &f3);
    return std::min(f1, std::min(f2, f3));
}

// Completes p (smem sizes) for problems of the given geometries under p.ctas CTAs per
// cluster; returns the number of clusters that can be resident at once (0: invalid).
int completeWaveBatchPlan(WaveBatchPlan& p, const std::vector<WaveGeom>& geoms, int dim, int b, bool fp64)
{
    if (p.ctas < 1 || p.ctas > 16 || p.threads < 32 || p.threads > 1024 || p.threads % 32) return 0;
    if (p.pf != 0 && p.pf != 1 && p.pf != 2 && p.pf != 4 && p.pf != 8) return 0;
    for (const WaveGeom& g : geoms) {
        if (g.ctas < 1 || g.ctas > p.ctas) return 0;
        if ((g.linesPerCta + p.threads - 1) / p.threads > 2) return 0;
    }
    const int count = (int)geoms.size();
    if (b == 1) return fp64 ? batchFits<1, double>(p, geoms, dim, count) : batchFits<1, float>(p, geoms, dim, count);
    return fp64 ? batchFits<2, double>(p, geoms, dim, count) : batchFits<2, float>(p, geoms, dim, count);
}

template <class T>
void launchWaveFactorBatch(const WaveBatchPlan& p, const WaveArgs<T>* batch, int count, int dim, int b,
                           cudaStream_t st)
{
    const WaveLaunch L{count, p.ctas, p.threads, p.pf, p.smemFactor};
    const cudaError_t e = b == 1 ? dispatch<1, T, 1, 1>(L, dim, WaveArgs<T>{}, batch, st, false, nullptr)
                                 : dispatch<2, T, 1, 1>(L, dim, WaveArgs<T>{}, batch, st, false, nullptr);
    DXG_CUDA(e);
}
template <class T>
void launchWaveApplyBatch(const WaveBatchPlan& p, const WaveArgs<T>* fwd, const WaveArgs<T>* bwd, int count, int dim,
                          int b, cudaStream_t st)
{
    const WaveLaunch Lf{count, p.ctas, p.threads, p.pf, p.smemFwd};
    const WaveLaunch Lb{count, p.ctas, p.threads, p.pf, p.smemBwd};
    if (b == 1) {
        DXG_CUDA((dispatch<1, T, 1, 0>(Lf, dim, WaveArgs<T>{}, fwd, st, false, nullptr)));
        DXG_CUDA((dispatch<1, T, -1, 0>(Lb, dim, WaveArgs<T>{}, bwd, st, false, nullptr)));
    } else {
        DXG_CUDA((dispatch<2, T, 1, 0>(Lf, dim, WaveArgs<T>{}, fwd, st, false, nullptr)));
        DXG_CUDA((dispatch<2, T, -1, 0>(Lb, dim, WaveArgs<T>{}, bwd, st, false, nullptr)));
    }
}

template void launchWaveFactor<double>(const WavePlan&, const WaveArgs<double>&, int, cudaStream_t);
template void launchWaveFactor<float>(const WavePlan&, const WaveArgs<float>&, int, cudaStream_t);
template void launchWaveApply<double>(const WavePlan&, const WaveArgs<double>&, const WaveArgs<double>&, int,
                                      cudaStream_t);
template void launchWaveApply<float>(const WavePlan&, const WaveArgs<float>&, const WaveArgs<float>&, int,
                                     cudaStream_t);
template void launchWaveFactorBatch<double>(const WaveBatchPlan&, const WaveArgs<double>*, int, int, int,
                                            cudaStream_t);
template void launchWaveFactorBatch<float>(const WaveBatchPlan&, const WaveArgs<float>*, int, int, int, cudaStream_t);
template void launchWaveApplyBatch<double>(const WaveBatchPlan&, const WaveArgs<double>*, const WaveArgs<double>*, int,
                                           int, int, cudaStream_t);
template void launchWaveApplyBatch<float>(const WaveBatchPlan&, const WaveArgs<float>*, const WaveArgs<float>*, int,
                                          int, int, cudaStream_t);

}  // namespace dxg
