// linesweep.cu -- natural-order ILU(0) sweeps of 2D cc-TPFA systems (1x1 or 2x2 blocks) in one
// CTA: one thread per grid line y holding both block rows, one CTA barrier per level (up to
// 512 lines).
//
// Cell (x, y) sits on level x + y; forward it needs its own line's cell x-1 and line y-1's cell
// x, both of the level before (backward mirrored: x+1 and y+1).  Line y handles cell x = s - y
// at step s; its previous result stays in registers, line y-1's comes by warp shuffle (from the
// warp before through a double-buffered shared-memory slot).  Each cell's factor rows,
// right-hand side (backward: and pivot inverse) are loaded PF steps ahead into a register ring
// whose entry is refilled at the start of the step that empties it.  The arithmetic per cell is
// that of the cluster wavefront (wave.cu) and of the level-scheduled kernels: the x term, then
// the y term, each block row a chain of explicit FMAs; backward the pivot-inverse product as
// there.  So all give the same bits.
#include <algorithm>

#include "common.cuh"
#include "linalg.cuh"
#include "wave.cuh"

namespace dxg {
namespace {

// records: forward L_x, L_y blocks and d; backward U_x, U_y, Dinv blocks and v
template <int B, int DIR>
struct L2Rec {
    static constexpr int n = DIR > 0 ? 2 * B * B + B : 3 * B * B + B;
};

template <int B, class T, int DIR, int PF, int MAXT>
__global__ void __launch_bounds__(MAXT) tpfaLine2dKernel(LaneWaveArgs<T> a)
{
    constexpr int BB = B * B;
    constexpr int REC = L2Rec<B, DIR>::n;
    __shared__ T hist[32][2][B];   // per warp and step parity: its last line's result
    if (a.ks && a.ks->status != KS_RUNNING) return;
    const int nx = a.nx, ny = a.ny;
    const int64_t N = a.N;
    const int sy = threadIdx.x;                        // sweep line (backward: mirrored y)
    const bool lineOk = sy < ny;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int y = DIR > 0 ? sy : ny - 1 - sy;
    const int64_t lineBase = lineOk ? (int64_t)y * nx : 0;
    const int nSteps = nx + ny - 1;
    // TPFA slots of a 2D grid: -y 0, -x 1, centre 2, +x 3, +y 4
    const T* srcX = (DIR > 0 ? a.Lf + (int64_t)1 * N * BB : a.A + (int64_t)3 * N * BB) + lineBase * BB;
    const T* srcY = (DIR > 0 ? a.Lf : a.A + (int64_t)4 * N * BB) + lineBase * BB;
    const T* srcD = a.Dinv + lineBase * BB;
    const T* srcV = (DIR > 0 ? a.rhs : a.v) + lineBase * B;

    T ring[PF][REC];
    auto load = [&](int s, int k) {
        const int sx = s - sy;
        const bool act = lineOk && sx >= 0 && sx < nx;
        const int x = DIR > 0 ? sx : nx - 1 - sx;
        const int xx = act ? x : 0;
#pragma unroll
        for (int e = 0; e < BB; ++e) {
            ring[k][e] = act ? __ldg(srcX + (int64_t)xx * BB + e) : T(0);
            ring[k][BB + e] = act ? __ldg(srcY + (int64_t)xx * BB + e) : T(0);
            if (DIR < 0) ring[k][2 * BB + e] = act ? __ldg(srcD + (int64_t)xx * BB + e) : T(0);
        }
#pragma unroll
        for (int e = 0; e < B; ++e) ring[k][REC - B + e] = act ? __ldg(srcV + (int64_t)xx * B + e) : T(0);
    };
#pragma unroll
    for (int k = 0; k < PF; ++k) load(k, k);
    T prev[B];
#pragma unroll
    for (int e = 0; e < B; ++e) prev[e] = 0;
    for (int s0 = 0; s0 < nSteps; s0 += PF) {
#pragma unroll
        for (int k = 0; k < PF; ++k) {
            const int s = s0 + k;
            T rec[REC];
#pragma unroll
            for (int e = 0; e < REC; ++e) rec[e] = ring[k][e];
            load(s + PF, k);
            // line sy-1's result of the step before (its cell at this x)
            T nb[B];
#pragma unroll
            for (int e = 0; e < B; ++e) nb[e] = __shfl_up_sync(0xffffffffu, prev[e], 1);
            if (lane == 0 && warp > 0 && s > 0)
#pragma unroll
                for (int e = 0; e < B; ++e) nb[e] = hist[warp - 1][(s - 1) & 1][e];
            const int sx = s - sy;
            const bool act = lineOk && sx >= 0 && sx < nx;
            T res[B];
#pragma unroll
            for (int e = 0; e < B; ++e) res[e] = 0;
            if (act) {
                const int x = DIR > 0 ? sx : nx - 1 - sx;
                T acc[B];
#pragma unroll
                for (int e = 0; e < B; ++e) acc[e] = rec[REC - B + e];
                if (sx > 0)
#pragma unroll
                    for (int r = 0; r < B; ++r)
#pragma unroll
                        for (int c = 0; c < B; ++c) acc[r] = fma(-rec[r * B + c], prev[c], acc[r]);
                if (sy > 0)
#pragma unroll
                    for (int r = 0; r < B; ++r)
#pragma unroll
                        for (int c = 0; c < B; ++c) acc[r] = fma(-rec[BB + r * B + c], nb[c], acc[r]);
                if (DIR > 0) {
#pragma unroll
                    for (int e = 0; e < B; ++e) res[e] = acc[e];
                } else {
                    const T* Di = rec + 2 * BB;
#pragma unroll
                    for (int r = 0; r < B; ++r) {
                        T t = Di[r * B] * acc[0];
#pragma unroll
                        for (int c = 1; c < B; ++c) t = fma(Di[r * B + c], acc[c], t);
                        res[r] = t;
                    }
                }
#pragma unroll
                for (int e = 0; e < B; ++e) a.v[(lineBase + x) * B + e] = res[e];
            }
#pragma unroll
            for (int e = 0; e < B; ++e) prev[e] = res[e];
            if (lane == 31)
#pragma unroll
                for (int e = 0; e < B; ++e) hist[warp][s & 1][e] = res[e];
            __syncthreads();
        }
    }
}

template <int B, class T, int DIR>
void l2Launch(const LaneWaveArgs<T>& a, unsigned threads, cudaStream_t st)
{
    // ring depth by CTA size and block size (the registers a thread has at that size)
    if (threads <= 256) tpfaLine2dKernel<B, T, DIR, (B == 1 ? 8 : 4), 256><<<1, threads, 0, st>>>(a);
    else tpfaLine2dKernel<B, T, DIR, (B == 1 ? 4 : 2), 512><<<1, threads, 0, st>>>(a);
}

}  // namespace

// up to 512 lines: one CTA of at most 512 threads keeps the ring in registers without spills
bool tpfaLine2dFits(int dim, int nx, int ny, int b)
{
    return dim == 2 && (b == 1 || b == 2) && nx >= 1 && ny >= 1 && ny <= 512;
}

template <class T>
void launchTpfaLine2d(const LaneWaveArgs<T>& fwd, const LaneWaveArgs<T>& bwd, int b, cudaStream_t st)
{
    const unsigned threads = (unsigned)((fwd.ny + 31) / 32 * 32);
    if (b == 2) {
        l2Launch<2, T, 1>(fwd, threads, st);
        l2Launch<2, T, -1>(bwd, threads, st);
    } else {
        l2Launch<1, T, 1>(fwd, threads, st);
        l2Launch<1, T, -1>(bwd, threads, st);
    }
    DXG_CUDA(cudaGetLastError());
}

template void launchTpfaLine2d<double>(const LaneWaveArgs<double>&, const LaneWaveArgs<double>&, int, cudaStream_t);
template void launchTpfaLine2d<float>(const LaneWaveArgs<float>&, const LaneWaveArgs<float>&, int, cudaStream_t);

}  // namespace dxg
