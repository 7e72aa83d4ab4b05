// linalg.cu -- block SpMV, natural-order ILU(0) and BiCGSTAB on the device.
//
// Replaces the dune-istl path bound by ILUBiCGSTABIstlSolver
// (dumux/linear/istlsolvers.hh:635-642): SeqILU with n = 0, relaxation 1 (block ILU(0)
// of the assembled matrix in its natural, lexicographic order) and BiCGSTABSolver.
//
// ILU(0) on the cc-TPFA stencil: for row i every lower neighbour j = i - stride has,
// in its own row, exactly one upper block inside row i's pattern -- the one pointing
// back at i -- so the factorisation only rewrites pivots:
//     L_ij = A_ij * D_j^{-1},   D_i = A_ii - sum_j L_ij * A_ji   (j in increasing order)
// and the upper factor is the upper part of A itself.  Row i depends on rows i-1,
// i-nx, i-nx*ny, so all cells with equal ix+iy+iz (one "level") are independent.
//
// BiCGSTAB keeps its scalars on the device (KrylovState); every kernel returns at
// once when the solve has stopped, so a fixed sequence of launches can be queued or
// captured without a host round trip per half step.  Reductions are deterministic:
// per-block partial sums in a fixed grid, combined in block order by the last block.
#include <cuda/atomic>
#include <type_traits>

#include "common.cuh"
#include "linalg.cuh"
#include "linalg_kernels.cuh"

namespace dxg {

// ---------------------------------------------------------------- reductions
__device__ __forceinline__ double warpSum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warpMax(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Block-wide sum of NV values per thread; result valid in thread 0.
template <int NV>
__device__ __forceinline__ void blockSum(double (&v)[NV])
{
    __shared__ double sh[NV][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = warpSum(v[k]);
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; ++k) sh[k][wid] = v[k];
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double t = lane < nw ? sh[k][lane] : 0.0;
            v[k] = warpSum(t);
        }
    }
}

// Blocks a vector kernel over M entries uses (host: reduceBlocks): kReducePerThread
// entries per thread, at most kMaxReduceBlocks blocks.
__host__ __device__ __forceinline__ int reduceBlocksFor(int64_t M)
{
    int64_t b = (M + kReduceThreads * kReducePerThread - 1) / (kReduceThreads * kReducePerThread);
    if (b > kMaxReduceBlocks) b = kMaxReduceBlocks;
    if (b < 1) b = 1;
    return (int)b;
}
// Blocks of the SpMV over N cells: one cell per thread, at most kMaxReduceBlocks blocks.
__host__ __device__ __forceinline__ int cellBlocksFor(int64_t N)
{
    int64_t b = (N + kReduceThreads - 1) / kReduceThreads;
    if (b > kMaxReduceBlocks) b = kMaxReduceBlocks;
    if (b < 1) b = 1;
    return (int)b;
}

// The problem and problem-local block of this block: single launch (a0), batched
// launch with blockIdx.y = problem, or batched launch through a block map.
template <class ARGT>
__device__ __forceinline__ ARGT problemOf(const ARGT& a0, const ARGT* batch, const uint2* map, unsigned& lb)
{
    if (map) {
        const uint2 m = map[blockIdx.x];
        lb = m.y;
        return batch[m.x];
    }
    lb = blockIdx.x;
    return batch ? batch[blockIdx.y] : a0;
}

// Writes this block's partials; returns true in thread 0 of the last of the nblk
// participating blocks to finish, which then holds the totals (summed in block
// order) in v.
template <int NV>
__device__ __forceinline__ bool gridSum(double (&v)[NV], double* partials, unsigned* counter, unsigned nblk,
                                        unsigned lb)
{
    blockSum<NV>(v);
    __shared__ bool amLast;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) partials[k * kMaxReduceBlocks + lb] = v[k];
        __threadfence();
        const unsigned t = atomicAdd(counter, 1u);
        amLast = (t == nblk - 1);
    }
    __syncthreads();
    if (!amLast) return false;
    __threadfence();
    // the last block combines the partials in block order
    if (threadIdx.x < 32) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double s = 0.0;
            for (unsigned bI = threadIdx.x; bI < nblk; bI += 32)
                s += ((volatile double*)partials)[k * kMaxReduceBlocks + bI];
            v[k] = warpSum(s);
        }
    }
    if (threadIdx.x == 0) *counter = 0u;
    return threadIdx.x == 0;
}

// ---------------------------------------------------------------- block helpers
template <int B, class MT, class VT>
__device__ __forceinline__ void blkMv(const MT* __restrict__ blk, const VT* x, VT* acc)
{
#pragma unroll
    for (int r = 0; r < B; ++r)
#pragma unroll
        for (int c = 0; c < B; ++c) acc[r] += (VT)blk[r * B + c] * x[c];
}
template <int B, class MT, class VT>
__device__ __forceinline__ void blkMvSub(const MT* __restrict__ blk, const VT* x, VT* acc)
{
#pragma unroll
    for (int r = 0; r < B; ++r) {
        VT s = 0;
#pragma unroll
        for (int c = 0; c < B; ++c) s += (VT)blk[r * B + c] * x[c];
        acc[r] -= s;
    }
}

template <int B, class T>
__device__ __forceinline__ void loadVec(const T* p, int64_t i, T* v)
{
#pragma unroll
    for (int e = 0; e < B; ++e) v[e] = p[i * B + e];
}
template <int B, class T>
__device__ __forceinline__ void storeVec(T* p, int64_t i, const T* v)
{
#pragma unroll
    for (int e = 0; e < B; ++e) p[i * B + e] = v[e];
}

// Read-only vector loads of one b x b block / one b-vector (16-byte loads for 2 x 2 FP32
// blocks and FP64 pairs; every block and vector entry starts on a multiple of its size
// from a cudaMalloc base).  Only for data no kernel writes while the reader runs.
template <int B, class T>
__device__ __forceinline__ void ldgBlock(const T* p, T* o)
{
    if constexpr (B == 2 && sizeof(T) == 4) {
        const float4 v = __ldg(reinterpret_cast<const float4*>(p));
        o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
    } else if constexpr (B == 2 && sizeof(T) == 8) {
        const double2 v0 = __ldg(reinterpret_cast<const double2*>(p));
        const double2 v1 = __ldg(reinterpret_cast<const double2*>(p) + 1);
        o[0] = v0.x; o[1] = v0.y; o[2] = v1.x; o[3] = v1.y;
    } else {
#pragma unroll
        for (int e = 0; e < B * B; ++e) o[e] = __ldg(p + e);
    }
}
template <int B, class T>
__device__ __forceinline__ void ldgVec(const T* p, T* o)
{
    if constexpr (B == 2 && sizeof(T) == 4) {
        const float2 v = __ldg(reinterpret_cast<const float2*>(p));
        o[0] = v.x; o[1] = v.y;
    } else if constexpr (B == 2 && sizeof(T) == 8) {
        const double2 v = __ldg(reinterpret_cast<const double2*>(p));
        o[0] = v.x; o[1] = v.y;
    } else {
#pragma unroll
        for (int e = 0; e < B; ++e) o[e] = __ldg(p + e);
    }
}

__device__ __forceinline__ bool slotValid(unsigned mask, int dim, int s)
{
    if (s == dim) return true;
    const int f = s < dim ? 2 * (dim - 1 - s) : 2 * (s - dim - 1) + 1;
    return (mask >> f) & 1u;
}

// ---------------------------------------------------------------- SpMV
// y = A x; MODE 0: plain; MODE 1: also dot(w, y) -> h, alpha; MODE 2: dots (y,w),(y,y) -> omega
template <int B, int DIM, class MT, class VT, class XT, int MODE>
__global__ void __launch_bounds__(kReduceThreads) spmvKernel(SpmvArgs<MT, VT, XT> a0,
                                                              const SpmvArgs<MT, VT, XT>* batch, const uint2* map)
{
    // accumulation: FP32 when both operands are FP32, else the output type
    using AT = typename std::conditional<sizeof(MT) == 4 && sizeof(XT) == 4, float, VT>::type;
    unsigned lb;
    const SpmvArgs<MT, VT, XT> a = problemOf(a0, batch, map, lb);
    const unsigned nblk = cellBlocksFor(a.N);
    if (lb >= nblk) return;
    if (a.ks && a.ks->status != KS_RUNNING) return;
    constexpr int S = 2 * DIM + 1;
    constexpr int BB = B * B;
    double part[2] = {0.0, 0.0};
    for (int64_t i = lb * (int64_t)blockDim.x + threadIdx.x; i < a.N; i += (int64_t)nblk * blockDim.x) {
        const unsigned m = __ldg(a.nbmask + i);
        AT sum[B];
#pragma unroll
        for (int e = 0; e < B; ++e) sum[e] = 0;
        // straight-line code: every slot's block (always allocated) and x entry (the
        // cell's own for a missing neighbour) is loaded without a branch, so all loads of
        // the row are in flight together; a missing neighbour's block enters as zero
#pragma unroll
        for (int s = 0; s < S; ++s) {
            const bool valid = slotValid(m, DIM, s);
            MT blk[BB];
            XT xs[B];
            ldgBlock<B>(a.A + ((int64_t)s * a.N + i) * BB, blk);
            ldgVec<B>(a.x + (i + (valid ? a.off[s] : 0)) * B, xs);
            AT xj[B];
#pragma unroll
            for (int e = 0; e < B; ++e) xj[e] = valid ? (AT)xs[e] : (AT)0;
#pragma unroll
            for (int e = 0; e < BB; ++e) blk[e] = valid ? blk[e] : (MT)0;
            blkMv<B>(blk, xj, sum);
        }
        VT acc[B];
#pragma unroll
        for (int e = 0; e < B; ++e) acc[e] = (VT)sum[e];
        storeVec<B>(a.y, i, acc);
        if (MODE == 1) {
            VT w[B];
            loadVec<B>(a.w, i, w);
#pragma unroll
            for (int e = 0; e < B; ++e) part[0] += (double)w[e] * (double)acc[e];
        } else if (MODE == 2) {
            VT w[B];
            loadVec<B>(a.w, i, w);
#pragma unroll
            for (int e = 0; e < B; ++e) {
                part[0] += (double)acc[e] * (double)w[e];
                part[1] += (double)acc[e] * (double)acc[e];
            }
        }
    }
    if (MODE == 0) return;
    if (gridSum<2>(part, a.scratch.partials, a.scratch.counter + MODE, nblk, lb)) {
        KrylovState& ks = *a.ks;
        if (MODE == 1) {
            ks.h = part[0];
            if (fabs(ks.h) < 1e-80) ks.status = KS_BREAKDOWN;
            else ks.alpha = ks.rho_new / ks.h;
        } else {
            ks.tr = part[0];
            ks.tt = part[1];
            ks.omega = ks.tr / ks.tt;
        }
    }
}

// ---------------------------------------------------------------- ILU(0)
template <int B, class T>
__device__ __forceinline__ bool blkInvert(const T* A, T* inv)
{
    if (B == 1) {
        inv[0] = (T)1 / A[0];
        return A[0] != (T)0;
    } else {
        const T det = A[0] * A[3] - A[1] * A[2];
        if (det == (T)0) return false;
        const T detInv = (T)1 / det;
        inv[0] = A[3] * detInv;
        inv[1] = -A[1] * detInv;
        inv[2] = -A[2] * detInv;
        inv[3] = A[0] * detInv;
        return true;
    }
}
template <int B, class T>
__device__ __forceinline__ void blkMul(const T* X, const T* Y, T* Z)
{
#pragma unroll
    for (int r = 0; r < B; ++r)
#pragma unroll
        for (int c = 0; c < B; ++c) {
            T s = 0;
#pragma unroll
            for (int k = 0; k < B; ++k) s += X[r * B + k] * Y[k * B + c];
            Z[r * B + c] = s;
        }
}

template <int B, int DIM, class MT>
__global__ void iluFactorLevel(IluArgs<MT, MT> a, int begin, int count)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    constexpr int BB = B * B;
    const int64_t i = a.perm[begin + k];
    const unsigned m = a.nbmask[i];
    MT D[BB];
#pragma unroll
    for (int e = 0; e < BB; ++e) D[e] = a.A[((int64_t)DIM * a.N + i) * BB + e];
#pragma unroll
    for (int s = 0; s < DIM; ++s) {
        MT* Ls = a.L + ((int64_t)s * a.N + i) * BB;
        if (!slotValid(m, DIM, s)) {
#pragma unroll
            for (int e = 0; e < BB; ++e) Ls[e] = 0;
            continue;
        }
        const int64_t j = i + a.off[s];
        MT Aij[BB], Dj[BB], Lij[BB], Uji[BB], P[BB];
#pragma unroll
        for (int e = 0; e < BB; ++e) {
            Aij[e] = a.A[((int64_t)s * a.N + i) * BB + e];
            Dj[e] = a.Dinv[j * BB + e];
            Uji[e] = a.A[((int64_t)(2 * DIM - s) * a.N + j) * BB + e];
        }
        blkMul<B>(Aij, Dj, Lij);
#pragma unroll
        for (int e = 0; e < BB; ++e) Ls[e] = Lij[e];
        blkMul<B>(Lij, Uji, P);
#pragma unroll
        for (int e = 0; e < BB; ++e) D[e] -= P[e];
    }
    MT inv[BB];
    if (!blkInvert<B>(D, inv)) *a.singular = 1;
#pragma unroll
    for (int e = 0; e < BB; ++e) a.Dinv[i * BB + e] = inv[e];
}

// z -= blk * x as a chain of FMAs, the operation order of the wavefront kernels (wave.cu)
template <int B, class MT, class VT>
__device__ __forceinline__ void blkFmaSub(const MT* __restrict__ blk, const VT* x, VT* acc)
{
#pragma unroll
    for (int r = 0; r < B; ++r)
#pragma unroll
        for (int c = 0; c < B; ++c) acc[r] = fma(-(VT)blk[r * B + c], x[c], acc[r]);
}

// ---------------------------------------------------------------- red-black ILU(0)
// Cell k of colour c (0 red: x+y+z even) in row-major order of the half rows; -1 past the end.
__device__ __forceinline__ int64_t rbCell(int64_t k, int c, int nx, int ny, int64_t rows)
{
    const int h = (nx + 1) / 2;
    const int64_t row = k / h;
    if (row >= rows) return -1;
    const int j = (int)(k - row * h);
    const int y = (int)(row % ny), z = (int)(row / ny);
    const int x = 2 * j + ((c + y + z) & 1);
    return x < nx ? row * nx + x : -1;
}

// red cells: D_r^-1 = A_rr^-1
template <int B, int DIM, class T>
__global__ void rbFactorRed(RbArgs<T> a0, const RbArgs<T>* batch, const uint2* map)
{
    unsigned lb;
    const RbArgs<T> a = problemOf(a0, batch, map, lb);
    constexpr int BB = B * B;
    const int64_t rows = (int64_t)a.ny * a.nz, total = rows * ((a.nx + 1) / 2);
    const unsigned nblk = cellBlocksFor(total);
    if (lb >= nblk) return;
    for (int64_t k = lb * (int64_t)blockDim.x + threadIdx.x; k < total; k += (int64_t)nblk * blockDim.x) {
        const int64_t i = rbCell(k, 0, a.nx, a.ny, rows);
        if (i < 0) continue;
        T D[BB], inv[BB];
        ldgBlock<B>(a.A + ((int64_t)DIM * a.N + i) * BB, D);
        if (!blkInvert<B>(D, inv)) *a.singular = 1;
#pragma unroll
        for (int e = 0; e < BB; ++e) a.Dinv[i * BB + e] = inv[e];
    }
}

// black cells: D_b^-1 = (A_bb - sum_r A_br D_r^-1 A_rb)^-1, neighbours in slot order
template <int B, int DIM, class T>
__global__ void rbFactorBlack(RbArgs<T> a0, const RbArgs<T>* batch, const uint2* map)
{
    unsigned lb;
    const RbArgs<T> a = problemOf(a0, batch, map, lb);
    constexpr int BB = B * B, S = 2 * DIM + 1;
    const int64_t rows = (int64_t)a.ny * a.nz, total = rows * ((a.nx + 1) / 2);
    const unsigned nblk = cellBlocksFor(total);
    if (lb >= nblk) return;
    for (int64_t k = lb * (int64_t)blockDim.x + threadIdx.x; k < total; k += (int64_t)nblk * blockDim.x) {
        const int64_t i = rbCell(k, 1, a.nx, a.ny, rows);
        if (i < 0) continue;
        const unsigned m = a.nbmask[i];
        T D[BB];
        ldgBlock<B>(a.A + ((int64_t)DIM * a.N + i) * BB, D);
#pragma unroll
        for (int s = 0; s < S; ++s) {
            if (s == DIM || !slotValid(m, DIM, s)) continue;
            const int64_t j = i + a.off[s];
            T Aij[BB], Dj[BB], Aji[BB], Lij[BB], P[BB];
            ldgBlock<B>(a.A + ((int64_t)s * a.N + i) * BB, Aij);
            ldgBlock<B>(a.Dinv + j * BB, Dj);
            ldgBlock<B>(a.A + ((int64_t)(2 * DIM - s) * a.N + j) * BB, Aji);
            blkMul<B>(Aij, Dj, Lij);
            blkMul<B>(Lij, Aji, P);
#pragma unroll
            for (int e = 0; e < BB; ++e) D[e] -= P[e];
        }
        T inv[BB];
        if (!blkInvert<B>(D, inv)) *a.singular = 1;
#pragma unroll
        for (int e = 0; e < BB; ++e) a.Dinv[i * BB + e] = inv[e];
    }
}

// black pass: v_b = D_b^-1 (d_b - sum_r A_br (D_r^-1 d_r))
template <int B, int DIM, class T>
__global__ void rbApplyBlack(RbArgs<T> a0, const RbArgs<T>* batch, const uint2* map)
{
    unsigned lb;
    const RbArgs<T> a = problemOf(a0, batch, map, lb);
    if (a.ks && a.ks->status != KS_RUNNING) return;
    const T* __restrict__ d = a.d;
    T* __restrict__ v = a.v;
    constexpr int BB = B * B, S = 2 * DIM + 1;
    const int64_t rows = (int64_t)a.ny * a.nz, total = rows * ((a.nx + 1) / 2);
    const unsigned nblk = cellBlocksFor(total);
    if (lb >= nblk) return;
    for (int64_t k = lb * (int64_t)blockDim.x + threadIdx.x; k < total; k += (int64_t)nblk * blockDim.x) {
        const int64_t i = rbCell(k, 1, a.nx, a.ny, rows);
        if (i < 0) continue;
        const unsigned m = __ldg(a.nbmask + i);
        T acc[B];
        ldgVec<B>(d + i * B, acc);
        // FP32: straight-line loads of every neighbour slot (the cell's own entries stand in
        // for a missing neighbour, whose block enters as zero), so all gathers are in flight
        // together; FP64 skips missing neighbours (its zero products would cost FP64 issue)
#pragma unroll
        for (int s = 0; s < S; ++s) {
            if (s == DIM) continue;
            const bool valid = slotValid(m, DIM, s);
            if (sizeof(T) == 8 && !valid) continue;
            const int64_t j = i + (valid ? a.off[s] : 0);
            T Aij[BB], Dj[BB], dj[B], w[B];
            ldgBlock<B>(a.A + ((int64_t)s * a.N + i) * BB, Aij);
            ldgBlock<B>(a.Dinv + j * BB, Dj);
            ldgVec<B>(d + j * B, dj);
#pragma unroll
            for (int e = 0; e < BB; ++e) Aij[e] = valid ? Aij[e] : (T)0;
#pragma unroll
            for (int e = 0; e < B; ++e) {
                dj[e] = valid ? dj[e] : (T)0;
                w[e] = 0;
            }
            blkMv<B>(Dj, dj, w);
            blkFmaSub<B>(Aij, w, acc);
        }
        T Di[BB], out[B];
        ldgBlock<B>(a.Dinv + i * BB, Di);
#pragma unroll
        for (int e = 0; e < B; ++e) out[e] = 0;
        blkMv<B>(Di, acc, out);
        storeVec<B>(v, i, out);
    }
}

// red pass: v_r = D_r^-1 (d_r - sum_b A_rb v_b)
template <int B, int DIM, class T>
__global__ void rbApplyRed(RbArgs<T> a0, const RbArgs<T>* batch, const uint2* map)
{
    unsigned lb;
    const RbArgs<T> a = problemOf(a0, batch, map, lb);
    if (a.ks && a.ks->status != KS_RUNNING) return;
    const T* __restrict__ d = a.d;
    T* v = a.v;
    constexpr int BB = B * B, S = 2 * DIM + 1;
    const int64_t rows = (int64_t)a.ny * a.nz, total = rows * ((a.nx + 1) / 2);
    const unsigned nblk = cellBlocksFor(total);
    if (lb >= nblk) return;
    for (int64_t k = lb * (int64_t)blockDim.x + threadIdx.x; k < total; k += (int64_t)nblk * blockDim.x) {
        const int64_t i = rbCell(k, 0, a.nx, a.ny, rows);
        if (i < 0) continue;
        const unsigned m = __ldg(a.nbmask + i);
        T acc[B];
        ldgVec<B>(d + i * B, acc);
#pragma unroll
        for (int s = 0; s < S; ++s) {
            if (s == DIM) continue;
            const bool valid = slotValid(m, DIM, s);
            if (sizeof(T) == 8 && !valid) continue;   // as in the black pass
            const int64_t j = i + (valid ? a.off[s] : 0);
            T Aij[BB], vj[B];
            ldgBlock<B>(a.A + ((int64_t)s * a.N + i) * BB, Aij);
            loadVec<B>(v, j, vj);   // written by the black pass (previous launch)
#pragma unroll
            for (int e = 0; e < BB; ++e) Aij[e] = valid ? Aij[e] : (T)0;
            // a missing neighbour reads this cell's own (not yet written) entry: zero it
#pragma unroll
            for (int e = 0; e < B; ++e) vj[e] = valid ? vj[e] : (T)0;
            blkFmaSub<B>(Aij, vj, acc);
        }
        T Di[BB], out[B];
        ldgBlock<B>(a.Dinv + i * BB, Di);
#pragma unroll
        for (int e = 0; e < B; ++e) out[e] = 0;
        blkMv<B>(Di, acc, out);
        storeVec<B>(v, i, out);
    }
}

// forward sweep of one level: z_i = d_i - L_ix z_x - L_iy z_y - L_iz z_z
template <int B, int DIM, class MT, class VT>
__global__ void iluForwardLevel(IluArgs<MT, VT> a, const VT* __restrict__ d, VT* v, int begin, int count)
{
    if (a.ks && a.ks->status != KS_RUNNING) return;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    constexpr int BB = B * B;
    const int64_t i = a.perm[begin + k];
    const unsigned m = a.nbmask[i];
    VT rhs[B];
    loadVec<B>(d, i, rhs);
#pragma unroll
    for (int s = DIM - 1; s >= 0; --s) {
        if (!slotValid(m, DIM, s)) continue;
        const int64_t j = i + a.off[s];
        VT vj[B];
        loadVec<B>(v, j, vj);
        blkFmaSub<B>(a.L + ((int64_t)s * a.N + i) * BB, vj, rhs);
    }
    storeVec<B>(v, i, rhs);
}

// backward sweep of one level: y_i = D_i^{-1} (z_i - U_ix y_x - U_iy y_y - U_iz y_z)
template <int B, int DIM, class MT, class VT>
__global__ void iluBackwardLevel(IluArgs<MT, VT> a, VT* v, int begin, int count)
{
    if (a.ks && a.ks->status != KS_RUNNING) return;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    constexpr int BB = B * B;
    const int64_t i = a.perm[begin + k];
    const unsigned m = a.nbmask[i];
    VT acc[B];
    loadVec<B>(v, i, acc);
#pragma unroll
    for (int s = DIM + 1; s < 2 * DIM + 1; ++s) {
        if (!slotValid(m, DIM, s)) continue;
        const int64_t j = i + a.off[s];
        VT vj[B];
        loadVec<B>(v, j, vj);
        blkFmaSub<B>(a.A + ((int64_t)s * a.N + i) * BB, vj, acc);
    }
    const MT* Di = a.Dinv + i * BB;
    VT out[B];
#pragma unroll
    for (int r = 0; r < B; ++r) {
        VT t = (VT)Di[r * B] * acc[0];
#pragma unroll
        for (int c = 1; c < B; ++c) t = fma((VT)Di[r * B + c], acc[c], t);
        out[r] = t;
    }
    storeVec<B>(v, i, out);
}

// ---------------------------------------------------------------- BiCGSTAB vector kernels
// Each kernel takes a single argument block, or (batch != nullptr) one per problem,
// selected by blockIdx.y or by a block map; a problem always works with its own
// reduceBlocksFor(M) blocks, as in a single launch.
#define DXG_PROBLEM_BLOCKS(ARGT, LEN)                             \
    unsigned lb;                                                  \
    const ARGT a = problemOf(a0, batch, map, lb);                 \
    const unsigned nblk = reduceBlocksFor(a.LEN);                 \
    if (lb >= nblk) return;                                       \
    const int64_t stride = (int64_t)nblk * blockDim.x;            \
    const int64_t k0 = lb * (int64_t)blockDim.x + threadIdx.x;

// The rho step that opens an iteration, taken by the kernel that closed the previous one
// (the last block of bicgInit or of the stage-1 update, with rhoNew = <rt, r>): iteration
// limit, breakdown checks and beta.
__device__ __forceinline__ void rhoStep(KrylovState& ks, double rhoNew)
{
    if (ks.halfsteps + 1 >= ks.maxHalf) { ks.status = KS_MAXIT; return; }
    ks.rho_new = rhoNew;
    if (fabs(ks.rho) <= 1e-80 || fabs(ks.omega) <= 1e-80) { ks.status = KS_BREAKDOWN; return; }
    if (ks.halfsteps > 0) ks.beta = (ks.rho_new / ks.rho) * (ks.alpha / ks.omega);
}

template <class VT>
__global__ void __launch_bounds__(kReduceThreads) bicgInit(BicgArgs<VT> a0, const BicgArgs<VT>* batch, const uint2* map)
{
    DXG_PROBLEM_BLOCKS(BicgArgs<VT>, M)
    double part[1] = {0.0};
    for (int64_t k = k0; k < a.M; k += stride) {
        const VT rv = (VT)a.rhs[k];
        a.r[k] = rv;
        a.rt[k] = rv;
        a.x[k] = 0;
        a.p[k] = 0;
        a.v[k] = 0;
        part[0] += (double)rv * (double)rv;
    }
    if (gridSum<1>(part, a.scratch.partials, a.scratch.counter + 4, nblk, lb)) {
        KrylovState& ks = *a.ks;
        if (a.maxHalf > 0) {
            ks.reduction = a.reduction;
            ks.maxHalf = a.maxHalf;
        }
        ks.def0 = ks.def = sqrt(part[0]);
        ks.rho = ks.alpha = ks.omega = 1.0;
        ks.halfsteps = 0;
        if (!isfinite(ks.def)) ks.status = KS_NAN;
        else if (ks.def < 1e-30) ks.status = KS_CONVERGED;
        else {
            ks.status = KS_RUNNING;
            // first rho step: rt = r, so <rt, r> is the defect sum just formed
            rhoStep(ks, part[0]);
        }
    }
}

// p = r (first iteration) or p = (p - omega v) * beta + r
template <class VT>
__global__ void bicgUpdateP(BicgArgs<VT> a0, const BicgArgs<VT>* batch, const uint2* map)
{
    DXG_PROBLEM_BLOCKS(BicgArgs<VT>, M)
    const KrylovState& ks = *a.ks;
    if (ks.status != KS_RUNNING) return;
    const bool first = ks.halfsteps == 0;
    const VT omega = (VT)ks.omega, beta = (VT)ks.beta;
    for (int64_t k = k0; k < a.M; k += stride) {
        VT pk;
        if (first) pk = a.r[k];
        else {
            pk = a.p[k];
            pk += -omega * a.v[k];
            pk *= beta;
            pk += a.r[k];
        }
        a.p[k] = pk;
        if (a.pLow) a.pLow[k] = (float)pk;
    }
}

// x += s*y; r -= s*q; def = ||r||; STAGE 0: s = alpha, q = v; STAGE 1: s = omega, q = t,
// and the next iteration's rho step on <rt, r>
template <class VT, int STAGE>
__global__ void __launch_bounds__(kReduceThreads) bicgAxpyNorm(BicgArgs<VT> a0, const BicgArgs<VT>* batch, const uint2* map)
{
    DXG_PROBLEM_BLOCKS(BicgArgs<VT>, M)
    const KrylovState& ksr = *a.ks;
    if (ksr.status != KS_RUNNING) return;
    const double sd = STAGE == 0 ? ksr.alpha : ksr.omega;
    const VT s = (VT)sd;
    const VT* q = STAGE == 0 ? a.v : a.t;
    constexpr int NP = STAGE == 1 ? 2 : 1;
    double part[NP];
#pragma unroll
    for (int e = 0; e < NP; ++e) part[e] = 0.0;
    float* rLow = STAGE == 0 ? a.rLow : nullptr;
    for (int64_t k = k0; k < a.M; k += stride) {
        const VT yk = a.yLow ? (VT)a.yLow[k] : a.y[k];
        a.x[k] += s * yk;
        const VT rk = a.r[k] + (-s) * q[k];
        a.r[k] = rk;
        if (rLow) rLow[k] = (float)rk;
        part[0] += (double)rk * (double)rk;
        if (STAGE == 1) part[NP - 1] += (double)a.rt[k] * (double)rk;
    }
    if (gridSum<NP>(part, a.scratch.partials, a.scratch.counter + 6, nblk, lb)) {
        KrylovState& ks = *a.ks;
        ks.def = sqrt(part[0]);
        ks.halfsteps += 1;
        if (STAGE == 1) ks.rho = ks.rho_new;
        if (!isfinite(ks.def)) ks.status = KS_NAN;
        else if (ks.def < ks.def0 * ks.reduction || ks.def < 1e-30) ks.status = KS_CONVERGED;
        else if (STAGE == 1) rhoStep(ks, part[NP - 1]);
    }
}

// ---------------------------------------------------------------- Newton helpers
// u = uLast - lambda*delta (uLast keeps the iterate), shift = max relative shift
// (maxRelativeShift, dumux/nonlinear/newtonsolver.hh:110-128)
__global__ void __launch_bounds__(kReduceThreads) newtonUpdateKernel(NewtonUpdArgs a0, const NewtonUpdArgs* batch, const uint2* map)
{
    DXG_PROBLEM_BLOCKS(NewtonUpdArgs, M)
    double mx = 0.0;
    for (int64_t k = k0; k < a.M; k += stride) {
        const double x = a.uLast[k];
        const double y = x + (-a.lambda) * a.delta[k];
        a.u[k] = y;
        const double s = fabs(x - y) / fmax(1.0, fabs(x + y) * 0.5);
        mx = fmax(mx, s);
    }
    // block max
    __shared__ double sh[32];
    mx = warpMax(mx);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sh[wid] = mx;
    __syncthreads();
    __shared__ bool amLast;
    double* partials = a.scratch.partials;
    unsigned* counter = a.scratch.counter + 7;
    if (threadIdx.x == 0) {
        double bm = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) bm = fmax(bm, sh[k]);
        partials[lb] = bm;
        __threadfence();
        amLast = atomicAdd(counter, 1u) == nblk - 1;
    }
    __syncthreads();
    if (amLast && threadIdx.x == 0) {
        __threadfence();
        double g = 0.0;
        for (unsigned bI = 0; bI < nblk; ++bI) g = fmax(g, ((volatile double*)partials)[bI]);
        *a.shiftOut = g;
        *counter = 0u;
    }
}

__global__ void __launch_bounds__(kReduceThreads) norm2Kernel(NormArgs a0, const NormArgs* batch, const uint2* map)
{
    DXG_PROBLEM_BLOCKS(NormArgs, M)
    double part[1] = {0.0};
    for (int64_t k = k0; k < a.M; k += stride)
        part[0] += a.x[k] * a.x[k];
    if (gridSum<1>(part, a.scratch.partials, a.scratch.counter + 3, nblk, lb)) *a.out = sqrt(part[0]);
}

template <class VT>
__global__ void copyToDouble(const VT* __restrict__ x, double* y, int64_t M)
{
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < M; k += (int64_t)gridDim.x * blockDim.x)
        y[k] = (double)x[k];
}

// ---------------------------------------------------------------- partial reassembly
// newtonUpdate's partial-reassembly block (newtonsolver.hh:590-602, 1257-1280) and
// PartialReassemblerEngine<CCTpfa>::computeColors (partialreassembler.hh:313-343): add the
// cell's relative shift to its distance from the last linearisation, color it red when
// the distance exceeds the threshold, and reset the distance of red cells.
__global__ void partialColorKernel(const double* __restrict__ uLast, const double* __restrict__ u, double* dist,
                                   uint8_t* color, int64_t N, int b, double threshold)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int e = 0; e < b; ++e) {
            const double x = uLast[i * b + e], y = u[i * b + e];
            s = fmax(s, fabs(x - y) / fmax(1.0, fabs(x + y) * 0.5));
        }
        const double d = dist[i] + s;
        const bool red = d > threshold;
        color[i] = red ? 1 : 0;
        dist[i] = red ? 0.0 : d;
    }
}

// ---------------------------------------------------------------- mixed-precision helpers
__global__ void toFloatKernel(ToFloatArgs a0, const ToFloatArgs* batch)
{
    const ToFloatArgs a = batch ? batch[blockIdx.y] : a0;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < a.n; k += (int64_t)gridDim.x * blockDim.x)
        a.dst[k] = (float)a.src[k];
}
__global__ void toDoubleKernel(ToDoubleArgs a0, const ToDoubleArgs* batch, const uint2* map)
{
    DXG_PROBLEM_BLOCKS(ToDoubleArgs, n)
    for (int64_t k = k0; k < a.n; k += stride) a.dst[k] = (double)a.src[k];
}
__global__ void accumKernel(AccumArgs a0, const AccumArgs* batch)
{
    const AccumArgs a = batch ? batch[blockIdx.y] : a0;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < a.n; k += (int64_t)gridDim.x * blockDim.x)
        a.y[k] += (double)a.x[k];
}
// defect = rhs - A*x in FP64 (iterative refinement of the mixed-precision solve)
template <int B, int DIM>
__global__ void defectKernel(DefectArgs a0, const DefectArgs* batch)
{
    const DefectArgs a = batch ? batch[blockIdx.y] : a0;
    constexpr int BB = B * B;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.N; i += (int64_t)gridDim.x * blockDim.x) {
        const unsigned m = a.nbmask[i];
        double acc[B];
#pragma unroll
        for (int e = 0; e < B; ++e) acc[e] = 0.0;
#pragma unroll
        for (int s = 0; s < 2 * DIM + 1; ++s) {
            if (!slotValid(m, DIM, s)) continue;
            const int64_t j = i + a.off[s];
            const double* blk = a.A + ((int64_t)s * a.N + i) * BB;
#pragma unroll
            for (int rr = 0; rr < B; ++rr)
#pragma unroll
                for (int cc = 0; cc < B; ++cc) acc[rr] += blk[rr * B + cc] * a.x[j * B + cc];
        }
#pragma unroll
        for (int rr = 0; rr < B; ++rr) a.y[i * B + rr] = a.rhs[i * B + rr] - acc[rr];
    }
}

// ---------------------------------------------------------------- host launchers
int reduceBlocks(int64_t M) { return reduceBlocksFor(M); }
int cellBlocks(int64_t N) { return cellBlocksFor(N); }

void buildBlockMap(const std::vector<int64_t>& lengths, bool cells, std::vector<uint2>& out)
{
    out.clear();
    for (size_t p = 0; p < lengths.size(); ++p) {
        const int nb = cells ? cellBlocksFor(lengths[p]) : reduceBlocksFor(lengths[p]);
        for (int j = 0; j < nb; ++j) out.push_back(make_uint2((unsigned)p, (unsigned)j));
    }
}

// grid of a batched grid-stride launch: x covers the largest problem (capped), y = problems
static dim3 batchGrid(int64_t maxN, int count, int threads, int cap)
{
    int64_t gx = (maxN + threads - 1) / threads;
    if (gx > cap) gx = cap;
    if (gx < 1) gx = 1;
    return dim3((unsigned)gx, (unsigned)count);
}

template <int B, int DIM, class MT, class VT, class XT>
static void spmvT(const SpmvArgs<MT, VT, XT>& a, const SpmvArgs<MT, VT, XT>* batch, const uint2* map, dim3 g,
                  int mode, cudaStream_t st)
{
    if (mode == 0) spmvKernel<B, DIM, MT, VT, XT, 0><<<g, kReduceThreads, 0, st>>>(a, batch, map);
    else if (mode == 1) spmvKernel<B, DIM, MT, VT, XT, 1><<<g, kReduceThreads, 0, st>>>(a, batch, map);
    else spmvKernel<B, DIM, MT, VT, XT, 2><<<g, kReduceThreads, 0, st>>>(a, batch, map);
}
template <class MT, class VT, class XT>
static void spmvDispatch(const SpmvArgs<MT, VT, XT>& a, const SpmvArgs<MT, VT, XT>* batch, const uint2* map, dim3 g,
                         int b, int dim, int mode, cudaStream_t st)
{
    if (b == 1) {
        if (dim == 2) spmvT<1, 2>(a, batch, map, g, mode, st);
        else spmvT<1, 3>(a, batch, map, g, mode, st);
    } else {
        if (dim == 2) spmvT<2, 2>(a, batch, map, g, mode, st);
        else spmvT<2, 3>(a, batch, map, g, mode, st);
    }
    DXG_CUDA(cudaGetLastError());
}

template <class MT, class VT, class XT>
void launchSpmv(const SpmvArgs<MT, VT, XT>& a, int b, int dim, int mode, cudaStream_t st)
{
    spmvDispatch<MT, VT, XT>(a, nullptr, nullptr, dim3(cellBlocksFor(a.N)), b, dim, mode, st);
}
template <class MT, class VT, class XT>
void launchSpmvBatch(const SpmvArgs<MT, VT, XT>* batch, const BlockMap& cellMap, int b, int dim, int mode,
                     cudaStream_t st)
{
    spmvDispatch<MT, VT, XT>(SpmvArgs<MT, VT, XT>{}, batch, cellMap.map, dim3(cellMap.blocks), b, dim, mode, st);
}

template <class MT>
int64_t launchIluFactor(const IluArgs<MT, MT>& a, const LevelSchedule& ls, int b, int dim, cudaStream_t st)
{
    int64_t launches = 0;
    for (int L = 0; L < ls.numLevels; ++L) {
        const int begin = ls.ptr[L], count = ls.ptr[L + 1] - ls.ptr[L];
        const int g = (count + 127) / 128;
        if (b == 1) {
            if (dim == 2) iluFactorLevel<1, 2, MT><<<g, 128, 0, st>>>(a, begin, count);
            else iluFactorLevel<1, 3, MT><<<g, 128, 0, st>>>(a, begin, count);
        } else {
            if (dim == 2) iluFactorLevel<2, 2, MT><<<g, 128, 0, st>>>(a, begin, count);
            else iluFactorLevel<2, 3, MT><<<g, 128, 0, st>>>(a, begin, count);
        }
        ++launches;
    }
    DXG_CUDA(cudaGetLastError());
    return launches;
}

template <int B, int DIM, class MT, class VT>
static int64_t iluApplyT(const IluArgs<MT, VT>& a, const LevelSchedule& ls, const VT* d, VT* v, cudaStream_t st)
{
    for (int L = 0; L < ls.numLevels; ++L) {
        const int begin = ls.ptr[L], count = ls.ptr[L + 1] - ls.ptr[L];
        iluForwardLevel<B, DIM, MT, VT><<<(count + 127) / 128, 128, 0, st>>>(a, d, v, begin, count);
    }
    for (int L = ls.numLevels - 1; L >= 0; --L) {
        const int begin = ls.ptr[L], count = ls.ptr[L + 1] - ls.ptr[L];
        iluBackwardLevel<B, DIM, MT, VT><<<(count + 127) / 128, 128, 0, st>>>(a, v, begin, count);
    }
    return 2 * (int64_t)ls.numLevels;
}

template <class MT, class VT>
int64_t launchIluApply(const IluArgs<MT, VT>& a, const LevelSchedule& ls, int b, int dim, const VT* d, VT* v,
                       cudaStream_t st)
{
    int64_t n;
    if (b == 1) n = dim == 2 ? iluApplyT<1, 2>(a, ls, d, v, st) : iluApplyT<1, 3>(a, ls, d, v, st);
    else n = dim == 2 ? iluApplyT<2, 2>(a, ls, d, v, st) : iluApplyT<2, 3>(a, ls, d, v, st);
    DXG_CUDA(cudaGetLastError());
    return n;
}

template <class T, int B, int DIM>
static void rbFactorPasses(const RbArgs<T>& a, const RbArgs<T>* batch, const uint2* map, unsigned g, cudaStream_t st)
{
    rbFactorRed<B, DIM, T><<<g, kReduceThreads, 0, st>>>(a, batch, map);
    rbFactorBlack<B, DIM, T><<<g, kReduceThreads, 0, st>>>(a, batch, map);
}
template <class T, int B, int DIM>
static void rbApplyPasses(const RbArgs<T>& a, const RbArgs<T>* batch, const uint2* map, unsigned g, cudaStream_t st)
{
    rbApplyBlack<B, DIM, T><<<g, kReduceThreads, 0, st>>>(a, batch, map);
    rbApplyRed<B, DIM, T><<<g, kReduceThreads, 0, st>>>(a, batch, map);
}
template <class T>
static void rbDispatch(bool factor, const RbArgs<T>& a, const RbArgs<T>* batch, const uint2* map, unsigned g, int b,
                       int dim, cudaStream_t st)
{
    if (factor) {
        if (b == 1) dim == 2 ? rbFactorPasses<T, 1, 2>(a, batch, map, g, st) : rbFactorPasses<T, 1, 3>(a, batch, map, g, st);
        else dim == 2 ? rbFactorPasses<T, 2, 2>(a, batch, map, g, st) : rbFactorPasses<T, 2, 3>(a, batch, map, g, st);
    } else {
        if (b == 1) dim == 2 ? rbApplyPasses<T, 1, 2>(a, batch, map, g, st) : rbApplyPasses<T, 1, 3>(a, batch, map, g, st);
        else dim == 2 ? rbApplyPasses<T, 2, 2>(a, batch, map, g, st) : rbApplyPasses<T, 2, 3>(a, batch, map, g, st);
    }
    DXG_CUDA(cudaGetLastError());
}

template <class T>
int64_t launchRbFactor(const RbArgs<T>& a, int b, int dim, cudaStream_t st)
{
    rbDispatch<T>(true, a, nullptr, nullptr, (unsigned)cellBlocksFor(rbSlots(a.nx, a.ny, a.nz)), b, dim, st);
    return 2;
}

template <class T>
int64_t launchRbApply(const RbArgs<T>& a, int b, int dim, const T* d, T* v, cudaStream_t st)
{
    RbArgs<T> aa = a;
    aa.d = d;
    aa.v = v;
    rbDispatch<T>(false, aa, nullptr, nullptr, (unsigned)cellBlocksFor(rbSlots(a.nx, a.ny, a.nz)), b, dim, st);
    return 2;
}

template <class T>
void launchRbFactorBatch(const RbArgs<T>* batch, const BlockMap& m, int b, int dim, cudaStream_t st)
{
    rbDispatch<T>(true, RbArgs<T>{}, batch, m.map, m.blocks, b, dim, st);
}
template <class T>
void launchRbApplyBatch(const RbArgs<T>* batch, const BlockMap& m, int b, int dim, cudaStream_t st)
{
    rbDispatch<T>(false, RbArgs<T>{}, batch, m.map, m.blocks, b, dim, st);
}

template <class VT>
void launchBicgInit(const BicgArgs<VT>& a, const double* rhs, cudaStream_t st)
{
    BicgArgs<VT> aa = a;
    aa.rhs = rhs;
    bicgInit<VT><<<reduceBlocks(a.M), kReduceThreads, 0, st>>>(aa, nullptr, nullptr);
    DXG_CUDA(cudaGetLastError());
}
template <class VT>
void launchBicgUpdateP(const BicgArgs<VT>& a, cudaStream_t st)
{
    bicgUpdateP<VT><<<reduceBlocks(a.M), kReduceThreads, 0, st>>>(a, nullptr, nullptr);
}
template <class VT>
void launchBicgAxpyNorm(const BicgArgs<VT>& a, int stage, cudaStream_t st)
{
    if (stage == 0) bicgAxpyNorm<VT, 0><<<reduceBlocks(a.M), kReduceThreads, 0, st>>>(a, nullptr, nullptr);
    else bicgAxpyNorm<VT, 1><<<reduceBlocks(a.M), kReduceThreads, 0, st>>>(a, nullptr, nullptr);
}
template <class VT>
void launchBicgInitBatch(const BicgArgs<VT>* batch, const BlockMap& m, cudaStream_t st)
{
    bicgInit<VT><<<m.blocks, kReduceThreads, 0, st>>>(BicgArgs<VT>{}, batch, m.map);
    DXG_CUDA(cudaGetLastError());
}
template <class VT>
void launchBicgUpdatePBatch(const BicgArgs<VT>* batch, const BlockMap& m, cudaStream_t st)
{
    bicgUpdateP<VT><<<m.blocks, kReduceThreads, 0, st>>>(BicgArgs<VT>{}, batch, m.map);
}
template <class VT>
void launchBicgAxpyNormBatch(const BicgArgs<VT>* batch, const BlockMap& m, int stage, cudaStream_t st)
{
    if (stage == 0) bicgAxpyNorm<VT, 0><<<m.blocks, kReduceThreads, 0, st>>>(BicgArgs<VT>{}, batch, m.map);
    else bicgAxpyNorm<VT, 1><<<m.blocks, kReduceThreads, 0, st>>>(BicgArgs<VT>{}, batch, m.map);
}
template <class VT>
void launchCopyToDouble(const VT* x, double* y, int64_t M, cudaStream_t st)
{
    copyToDouble<VT><<<reduceBlocks(M), kReduceThreads, 0, st>>>(x, y, M);
}

void launchNewtonUpdate(const double* uLast, const double* delta, double* u, double lambda, int64_t M,
                        const ReduceScratch& sc, double* shiftOut, cudaStream_t st)
{
    const NewtonUpdArgs a{uLast, delta, u, lambda, M, sc, shiftOut};
    newtonUpdateKernel<<<reduceBlocks(M), kReduceThreads, 0, st>>>(a, nullptr, nullptr);
    DXG_CUDA(cudaGetLastError());
}
void launchNewtonUpdateBatch(const NewtonUpdArgs* batch, const BlockMap& m, cudaStream_t st)
{
    newtonUpdateKernel<<<m.blocks, kReduceThreads, 0, st>>>(NewtonUpdArgs{}, batch, m.map);
    DXG_CUDA(cudaGetLastError());
}
void launchNorm2(const double* x, int64_t M, const ReduceScratch& sc, double* out, cudaStream_t st)
{
    const NormArgs a{x, M, sc, out};
    norm2Kernel<<<reduceBlocks(M), kReduceThreads, 0, st>>>(a, nullptr, nullptr);
    DXG_CUDA(cudaGetLastError());
}
void launchNorm2Batch(const NormArgs* batch, const BlockMap& m, cudaStream_t st)
{
    norm2Kernel<<<m.blocks, kReduceThreads, 0, st>>>(NormArgs{}, batch, m.map);
    DXG_CUDA(cudaGetLastError());
}
void launchPartialColors(const double* uLast, const double* u, double* dist, uint8_t* color, int64_t N, int b,
                         double threshold, cudaStream_t st)
{
    partialColorKernel<<<reduceBlocks(N), kReduceThreads, 0, st>>>(uLast, u, dist, color, N, b, threshold);
    DXG_CUDA(cudaGetLastError());
}
void launchToFloat(const ToFloatArgs& a, cudaStream_t st)
{
    toFloatKernel<<<reduceBlocks(a.n), kReduceThreads, 0, st>>>(a, nullptr);
    DXG_CUDA(cudaGetLastError());
}
void launchToFloatBatch(const ToFloatArgs* batch, int count, int64_t maxN, cudaStream_t st)
{
    toFloatKernel<<<batchGrid(maxN, count, kReduceThreads, 1184), kReduceThreads, 0, st>>>(ToFloatArgs{}, batch);
    DXG_CUDA(cudaGetLastError());
}
void launchToDouble(const ToDoubleArgs& a, cudaStream_t st)
{
    toDoubleKernel<<<reduceBlocks(a.n), kReduceThreads, 0, st>>>(a, nullptr, nullptr);
    DXG_CUDA(cudaGetLastError());
}
void launchToDoubleBatch(const ToDoubleArgs* batch, const BlockMap& m, cudaStream_t st)
{
    toDoubleKernel<<<m.blocks, kReduceThreads, 0, st>>>(ToDoubleArgs{}, batch, m.map);
    DXG_CUDA(cudaGetLastError());
}
void launchAccum(const AccumArgs& a, cudaStream_t st)
{
    accumKernel<<<reduceBlocks(a.n), kReduceThreads, 0, st>>>(a, nullptr);
    DXG_CUDA(cudaGetLastError());
}
void launchAccumBatch(const AccumArgs* batch, int count, int64_t maxN, cudaStream_t st)
{
    accumKernel<<<batchGrid(maxN, count, kReduceThreads, 1184), kReduceThreads, 0, st>>>(AccumArgs{}, batch);
    DXG_CUDA(cudaGetLastError());
}
static void defectDispatch(const DefectArgs& a, const DefectArgs* batch, dim3 g, int b, int dim, cudaStream_t st)
{
    if (b == 1) {
        if (dim == 2) defectKernel<1, 2><<<g, kReduceThreads, 0, st>>>(a, batch);
        else defectKernel<1, 3><<<g, kReduceThreads, 0, st>>>(a, batch);
    } else {
        if (dim == 2) defectKernel<2, 2><<<g, kReduceThreads, 0, st>>>(a, batch);
        else defectKernel<2, 3><<<g, kReduceThreads, 0, st>>>(a, batch);
    }
    DXG_CUDA(cudaGetLastError());
}
void launchDefect(const DefectArgs& a, int b, int dim, cudaStream_t st)
{
    defectDispatch(a, nullptr, dim3(reduceBlocks(a.N * b)), b, dim, st);
}
void launchDefectBatch(const DefectArgs* batch, int count, int64_t maxN, int b, int dim, cudaStream_t st)
{
    defectDispatch(DefectArgs{}, batch, batchGrid(maxN, count, kReduceThreads, 1184), b, dim, st);
}

// explicit instantiations
template void launchSpmv<double, double, double>(const SpmvArgs<double, double, double>&, int, int, int,
                                                cudaStream_t);
template void launchSpmv<float, double, float>(const SpmvArgs<float, double, float>&, int, int, int, cudaStream_t);
template void launchSpmv<double, double, float>(const SpmvArgs<double, double, float>&, int, int, int, cudaStream_t);
template void launchSpmvBatch<double, double, double>(const SpmvArgs<double, double, double>*, const BlockMap&, int,
                                                      int, int, cudaStream_t);
template void launchSpmvBatch<float, double, float>(const SpmvArgs<float, double, float>*, const BlockMap&, int, int,
                                                    int, cudaStream_t);
template void launchSpmvBatch<double, double, float>(const SpmvArgs<double, double, float>*, const BlockMap&, int, int,
                                                     int, cudaStream_t);
template void launchBicgInitBatch<double>(const BicgArgs<double>*, const BlockMap&, cudaStream_t);
template void launchBicgInitBatch<float>(const BicgArgs<float>*, const BlockMap&, cudaStream_t);
template void launchBicgUpdatePBatch<double>(const BicgArgs<double>*, const BlockMap&, cudaStream_t);
template void launchBicgUpdatePBatch<float>(const BicgArgs<float>*, const BlockMap&, cudaStream_t);
template void launchBicgAxpyNormBatch<double>(const BicgArgs<double>*, const BlockMap&, int, cudaStream_t);
template void launchBicgAxpyNormBatch<float>(const BicgArgs<float>*, const BlockMap&, int, cudaStream_t);
template int64_t launchRbFactor<double>(const RbArgs<double>&, int, int, cudaStream_t);
template int64_t launchRbFactor<float>(const RbArgs<float>&, int, int, cudaStream_t);
template int64_t launchRbApply<double>(const RbArgs<double>&, int, int, const double*, double*, cudaStream_t);
template int64_t launchRbApply<float>(const RbArgs<float>&, int, int, const float*, float*, cudaStream_t);
template void launchRbFactorBatch<double>(const RbArgs<double>*, const BlockMap&, int, int, cudaStream_t);
template void launchRbFactorBatch<float>(const RbArgs<float>*, const BlockMap&, int, int, cudaStream_t);
template void launchRbApplyBatch<double>(const RbArgs<double>*, const BlockMap&, int, int, cudaStream_t);
template void launchRbApplyBatch<float>(const RbArgs<float>*, const BlockMap&, int, int, cudaStream_t);
template int64_t launchIluFactor<double>(const IluArgs<double, double>&, const LevelSchedule&, int, int, cudaStream_t);
template int64_t launchIluFactor<float>(const IluArgs<float, float>&, const LevelSchedule&, int, int, cudaStream_t);
template int64_t launchIluApply<double, double>(const IluArgs<double, double>&, const LevelSchedule&, int, int,
                                                const double*, double*, cudaStream_t);
template int64_t launchIluApply<float, float>(const IluArgs<float, float>&, const LevelSchedule&, int, int,
                                              const float*, float*, cudaStream_t);
template void launchBicgInit<double>(const BicgArgs<double>&, const double*, cudaStream_t);
template void launchBicgInit<float>(const BicgArgs<float>&, const double*, cudaStream_t);
template void launchBicgUpdateP<double>(const BicgArgs<double>&, cudaStream_t);
template void launchBicgUpdateP<float>(const BicgArgs<float>&, cudaStream_t);
template void launchBicgAxpyNorm<double>(const BicgArgs<double>&, int, cudaStream_t);
template void launchBicgAxpyNorm<float>(const BicgArgs<float>&, int, cudaStream_t);
template void launchCopyToDouble<double>(const double*, double*, int64_t, cudaStream_t);
template void launchCopyToDouble<float>(const float*, double*, int64_t, cudaStream_t);

// ---------------------------------------------------------------- scalar stencil operators
// Rows of one unknown over the 3^dim neighbourhood of a cell (the MPFA-O Jacobian): values
// A[slot][row], slot s = (ox+1) + 3(oy+1) + 9(oz+1) in ascending column order, valid for row
// i when bit s of mask[i] is set.

// y = A x; MODE 1: also dot(w, y) -> h, alpha; MODE 2: dots (y,w),(y,y) -> omega (the
// Krylov-state updates of spmvKernel)
template <int S, int MODE>
__global__ void __launch_bounds__(kReduceThreads) stencilSpmvKernel(StencilArgs a, const double* __restrict__ x,
                                                                     double* __restrict__ y, const double* __restrict__ w)
{
    const unsigned nblk = cellBlocksFor(a.N);
    const unsigned lb = blockIdx.x;
    if (a.ks && a.ks->status != KS_RUNNING) return;
    double part[2] = {0.0, 0.0};
    for (int64_t i = lb * (int64_t)blockDim.x + threadIdx.x; i < a.N; i += (int64_t)nblk * blockDim.x) {
        const uint32_t m = __ldg(a.mask + i);
        double sum = 0.0;
#pragma unroll
        for (int s = 0; s < S; ++s) {
            const bool valid = (m >> s) & 1u;
            const double aij = __ldg(a.A + (int64_t)s * a.N + i);
            const double xj = __ldg(x + i + (valid ? a.off[s] : 0));
            sum += valid ? aij * xj : 0.0;
        }
        y[i] = sum;
        if (MODE == 1) {
            part[0] += w[i] * sum;
        } else if (MODE == 2) {
            part[0] += sum * w[i];
            part[1] += sum * sum;
        }
    }
    if (MODE == 0) return;
    if (gridSum<2>(part, a.scratch.partials, a.scratch.counter + MODE, nblk, lb)) {
        KrylovState& ks = *a.ks;
        if (MODE == 1) {
            ks.h = part[0];
            if (fabs(ks.h) < 1e-80) ks.status = KS_BREAKDOWN;
            else ks.alpha = ks.rho_new / ks.h;
        } else {
            ks.tr = part[0];
            ks.tt = part[1];
            ks.omega = ks.tr / ks.tt;
        }
    }
}

// Rows of hyperplane level L of the natural ordering: x + 2y + 4z = L.  Every lower
// neighbour of a row (dz = -1; dz = 0, dy = -1; dz = dy = 0, dx = -1) sits on a lower
// level, so the rows of one level are independent.
template <class F>
__device__ __forceinline__ void forLevelRows(const StencilArgs& a, int L, F&& body)
{
    const int lines = a.ny * a.nz;
    for (int q = threadIdx.x; q < lines; q += blockDim.x) {
        const int yy = q % a.ny, zz = q / a.ny;
        const int xx = L - 2 * yy - 4 * zz;
        if (xx >= 0 && xx < a.nx) body(((int64_t)zz * a.ny + yy) * a.nx + xx);
    }
}

// ILU(0) of the stencil matrix in one CTA, level by level (Saad's row-wise IKJ variant as
// the block ILU(0) of the linear solver: for each lower entry j of row i in column order,
// l_ij = a_ij / u_jj, then a_ik -= l_ij u_jk for every later entry k of row i that row j
// holds; pivots stored inverted).  LU keeps the multipliers in the lower slots and U in the
// upper slots.
__global__ void __launch_bounds__(1024) stencilFactorKernel(StencilArgs a)
{
    const int levels = (a.nx - 1) + 2 * (a.ny - 1) + 4 * (a.nz - 1) + 1;
    for (int L = 0; L < levels; ++L) {
        forLevelRows(a, L, [&](int64_t i) {
            const uint32_t m = a.mask[i];
            for (int s = 0; s < a.S; ++s) a.LU[(int64_t)s * a.N + i] = a.A[(int64_t)s * a.N + i];
            int t0 = 0;
            for (int s = 0; s < a.center; ++s) {
                if (!((m >> s) & 1u)) continue;
                const int64_t j = i + a.off[s];
                const double l = a.LU[(int64_t)s * a.N + i] * a.Dinv[j];
                a.LU[(int64_t)s * a.N + i] = l;
                const uint32_t mj = a.mask[j];
                // the update triples (s, t, u) of this s, t ascending
                while (t0 < a.nTri && a.tri[t0][0] < s) ++t0;
                for (int k = t0; k < a.nTri && a.tri[k][0] == s; ++k) {
                    const int t = a.tri[k][1], u = a.tri[k][2];
                    if (!((m >> t) & 1u) || !((mj >> u) & 1u)) continue;
                    a.LU[(int64_t)t * a.N + i] = fma(-l, a.LU[(int64_t)u * a.N + j], a.LU[(int64_t)t * a.N + i]);
                }
            }
            const double piv = a.LU[(int64_t)a.center * a.N + i];
            if (piv == 0.0) atomicExch(a.singular, 1);
            a.Dinv[i] = 1.0 / piv;
        });
        __syncthreads();
    }
}

// v = (LU)^-1 d: forward sweep with the multipliers, backward sweep with U and the inverted
// pivots, both level by level in one CTA.
__global__ void __launch_bounds__(1024) stencilApplyKernel(StencilArgs a, const double* __restrict__ d,
                                                            double* __restrict__ v)
{
    if (a.ks && a.ks->status != KS_RUNNING) return;
    const int levels = (a.nx - 1) + 2 * (a.ny - 1) + 4 * (a.nz - 1) + 1;
    for (int L = 0; L < levels; ++L) {
        forLevelRows(a, L, [&](int64_t i) {
            const uint32_t m = a.mask[i];
            double rhs = d[i];
            for (int s = 0; s < a.center; ++s)
                if ((m >> s) & 1u) rhs = fma(-a.LU[(int64_t)s * a.N + i], v[i + a.off[s]], rhs);
            v[i] = rhs;
        });
        __syncthreads();
    }
    for (int L = levels - 1; L >= 0; --L) {
        forLevelRows(a, L, [&](int64_t i) {
            const uint32_t m = a.mask[i];
            // descending column order: the entries of the latest levels come last
            double rhs = v[i];
            for (int s = a.S - 1; s > a.center; --s)
                if ((m >> s) & 1u) rhs = fma(-a.LU[(int64_t)s * a.N + i], v[i + a.off[s]], rhs);
            v[i] = a.Dinv[i] * rhs;
        });
        __syncthreads();
    }
}

// The sweeps of a 2D 9-point stencil with one thread per grid line y (levels L = x + 2y):
// line y needs, besides its own previous cell, line y-1's cells x+1, x, x-1, which that line
// computed at levels L-1, L-2, L-3 (backward: line y+1's cells x-1, x, x+1 at L+1, L+2,
// L+3).  Every thread keeps its last three results; a warp passes them on by shuffle, the
// boundary lane of each warp through a double-buffered shared-memory slot, and one CTA
// barrier ends each level.  The cells' factor entries, right-hand side (and pivot) are
// loaded PF levels ahead into a register ring (a shared-memory ring filled with cp.async took
// 1.09-1.11 ms per apply at 256 x 256).  The arithmetic is that of stencilApplyKernel (same
// operand order, explicit FMAs), so both give the same bits.

template <int DIR, int PF, int MAXT>
__global__ void __launch_bounds__(MAXT) stencilWave2dKernel(StencilArgs a, const double* __restrict__ d,
                                                             double* __restrict__ v)
{
    // record per cell: forward L0..L3 (slots 0..3), d; backward U5..U8 (slots 5..8), Dinv, v;
    // held PF steps ahead in a register ring whose entry is refilled at the start of the step
    // that empties it (the loads issue ahead of the step's chain); the ring's depth follows the
    // registers a thread has at MAXT threads
    constexpr int REC = DIR > 0 ? 5 : 6;
    __shared__ double hist[32][2][3];                  // per warp, level parity: boundary lane's r1..r3
    if (a.ks && a.ks->status != KS_RUNNING) return;
    const int nx = a.nx, ny = a.ny;
    const int y = threadIdx.x;
    const bool lineOk = y < ny;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int Lmax = (nx - 1) + 2 * (ny - 1);
    const int64_t N = a.N;
    const int64_t rowBase = (int64_t)y * nx;
    // sweep step s: level L = s (forward) or Lmax - s (backward)
    auto cellX = [&](int s) -> int {
        const int L = DIR > 0 ? s : Lmax - s;
        const int x = L - 2 * y;
        return (lineOk && s <= Lmax && x >= 0 && x < nx) ? x : -1;
    };
    double ring[PF][REC];
    auto load = [&](int s, int k) {
        const int x = cellX(s);
        const int64_t i = rowBase + (x >= 0 ? x : 0);
#pragma unroll
        for (int e = 0; e < 4; ++e) ring[k][e] = x >= 0 ? __ldg(a.LU + (int64_t)((DIR > 0 ? 0 : 5) + e) * N + i) : 0.0;
        if (DIR > 0) {
            ring[k][4] = x >= 0 ? __ldg(d + i) : 0.0;
        } else {
            ring[k][4] = x >= 0 ? __ldg(a.Dinv + i) : 0.0;
            ring[k][5] = x >= 0 ? __ldg(v + i) : 0.0;
        }
    };
#pragma unroll
    for (int k = 0; k < PF; ++k) load(k, k);
    double r1 = 0.0, r2 = 0.0, r3 = 0.0;
    for (int s0 = 0; s0 <= Lmax; s0 += PF) {
#pragma unroll
        for (int k = 0; k < PF; ++k) {
            const int s = s0 + k;
            double rec[REC];
#pragma unroll
            for (int e = 0; e < REC; ++e) rec[e] = ring[k][e];
            load(s + PF, k);
            // the neighbour line's results of two and three levels back first, then the last
            // level's (see stencilLane2dKernel): the same operand order as stencilApplyKernel
            double n3 = DIR > 0 ? __shfl_up_sync(0xffffffffu, r3, 1) : __shfl_down_sync(0xffffffffu, r3, 1);
            double n2 = DIR > 0 ? __shfl_up_sync(0xffffffffu, r2, 1) : __shfl_down_sync(0xffffffffu, r2, 1);
            double n1 = DIR > 0 ? __shfl_up_sync(0xffffffffu, r1, 1) : __shfl_down_sync(0xffffffffu, r1, 1);
            const int par = (s - 1) & 1;
            if (DIR > 0 && lane == 0 && warp > 0 && s > 0) {
                n1 = hist[warp - 1][par][0];
                n2 = hist[warp - 1][par][1];
                n3 = hist[warp - 1][par][2];
            } else if (DIR < 0 && lane == 31 && s > 0 && (warp + 1) * 32 < (int)blockDim.x) {
                n1 = hist[warp + 1][par][0];
                n2 = hist[warp + 1][par][1];
                n3 = hist[warp + 1][par][2];
            }
            const int x = cellX(s);
            double res = 0.0;
            if (x >= 0) {
                const int64_t i = rowBase + x;
                if (DIR > 0) {
                    double acc = rec[4];
                    if (x > 0 && y > 0) acc = fma(-rec[0], n3, acc);        // (x-1, y-1)
                    if (y > 0) acc = fma(-rec[1], n2, acc);                 // (x,   y-1)
                    if (x < nx - 1 && y > 0) acc = fma(-rec[2], n1, acc);   // (x+1, y-1)
                    if (x > 0) acc = fma(-rec[3], r1, acc);                 // (x-1, y)
                    res = acc;
                } else {
                    double acc = rec[5];
                    if (x < nx - 1 && y < ny - 1) acc = fma(-rec[3], n3, acc);   // (x+1, y+1)
                    if (y < ny - 1) acc = fma(-rec[2], n2, acc);                 // (x,   y+1)
                    if (x > 0 && y < ny - 1) acc = fma(-rec[1], n1, acc);        // (x-1, y+1)
                    if (x < nx - 1) acc = fma(-rec[0], r1, acc);                  // (x+1, y)
                    res = rec[4] * acc;
                }
                v[i] = res;
            }
            r3 = r2;
            r2 = r1;
            r1 = res;
            if ((DIR > 0 && lane == 31) || (DIR < 0 && lane == 0)) {
                hist[warp][s & 1][0] = r1;
                hist[warp][s & 1][1] = r2;
                hist[warp][s & 1][2] = r3;
            }
            __syncthreads();
        }
    }
}


// 2x2 blocks over the same stencil (the 2p MPFA-O Jacobian, A[slot][row][4] row-major
// blocks): SpMV with the same fused dots, and the block ILU(0) factor and sweeps level by
// level (block products with explicit FMAs, pivot blocks inverted as in the wavefront factor)
template <int S, int MODE>
__global__ void __launch_bounds__(kReduceThreads) stencilSpmv2Kernel(StencilArgs a, const double* __restrict__ x,
                                                                      double* __restrict__ y, const double* __restrict__ w)
{
    const unsigned nblk = cellBlocksFor(a.N);
    const unsigned lb = blockIdx.x;
    if (a.ks && a.ks->status != KS_RUNNING) return;
    double part[2] = {0.0, 0.0};
    for (int64_t i = lb * (int64_t)blockDim.x + threadIdx.x; i < a.N; i += (int64_t)nblk * blockDim.x) {
        const uint32_t m = __ldg(a.mask + i);
        double sum[2] = {0.0, 0.0};
#pragma unroll
        for (int s = 0; s < S; ++s) {
            const bool valid = (m >> s) & 1u;
            double blk[4], xs[2];
            ldgBlock<2>(a.A + ((int64_t)s * a.N + i) * 4, blk);
            ldgVec<2>(x + (i + (valid ? a.off[s] : 0)) * 2, xs);
#pragma unroll
            for (int e = 0; e < 2; ++e) xs[e] = valid ? xs[e] : 0.0;
#pragma unroll
            for (int e = 0; e < 4; ++e) blk[e] = valid ? blk[e] : 0.0;
            blkMv<2>(blk, xs, sum);
        }
        y[i * 2] = sum[0];
        y[i * 2 + 1] = sum[1];
        if (MODE == 1) {
            for (int e = 0; e < 2; ++e) part[0] += w[i * 2 + e] * sum[e];
        } else if (MODE == 2) {
            for (int e = 0; e < 2; ++e) {
                part[0] += sum[e] * w[i * 2 + e];
                part[1] += sum[e] * sum[e];
            }
        }
    }
    if (MODE == 0) return;
    if (gridSum<2>(part, a.scratch.partials, a.scratch.counter + MODE, nblk, lb)) {
        KrylovState& ks = *a.ks;
        if (MODE == 1) {
            ks.h = part[0];
            if (fabs(ks.h) < 1e-80) ks.status = KS_BREAKDOWN;
            else ks.alpha = ks.rho_new / ks.h;
        } else {
            ks.tr = part[0];
            ks.tt = part[1];
            ks.omega = ks.tr / ks.tt;
        }
    }
}

__device__ __forceinline__ void st2Mul(const double* X, const double* Y, double* Z)
{
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            double t = 0.0;
            t = fma(X[r * 2 + 0], Y[0 * 2 + c], t);
            t = fma(X[r * 2 + 1], Y[1 * 2 + c], t);
            Z[r * 2 + c] = t;
        }
}

__global__ void __launch_bounds__(1024) stencilFactor2Kernel(StencilArgs a)
{
    const int levels = (a.nx - 1) + 2 * (a.ny - 1) + 4 * (a.nz - 1) + 1;
    for (int L = 0; L < levels; ++L) {
        forLevelRows(a, L, [&](int64_t i) {
            const uint32_t m = a.mask[i];
            for (int s = 0; s < a.S; ++s)
                for (int e = 0; e < 4; ++e) a.LU[((int64_t)s * a.N + i) * 4 + e] = a.A[((int64_t)s * a.N + i) * 4 + e];
            int t0 = 0;
            for (int s = 0; s < a.center; ++s) {
                if (!((m >> s) & 1u)) continue;
                const int64_t j = i + a.off[s];
                double* Lis = a.LU + ((int64_t)s * a.N + i) * 4;
                double l[4];
                st2Mul(Lis, a.Dinv + j * 4, l);
                for (int e = 0; e < 4; ++e) Lis[e] = l[e];
                const uint32_t mj = a.mask[j];
                while (t0 < a.nTri && a.tri[t0][0] < s) ++t0;
                for (int k = t0; k < a.nTri && a.tri[k][0] == s; ++k) {
                    const int t = a.tri[k][1], u = a.tri[k][2];
                    if (!((m >> t) & 1u) || !((mj >> u) & 1u)) continue;
                    double pr[4];
                    st2Mul(l, a.LU + ((int64_t)u * a.N + j) * 4, pr);
                    double* Lit = a.LU + ((int64_t)t * a.N + i) * 4;
                    for (int e = 0; e < 4; ++e) Lit[e] -= pr[e];
                }
            }
            const double* D = a.LU + ((int64_t)a.center * a.N + i) * 4;
            const double p12 = D[1] * D[2];
            const double det = fma(D[0], D[3], -p12);
            if (det == 0.0) atomicExch(a.singular, 1);
            const double di = 1.0 / det;
            a.Dinv[i * 4 + 0] = D[3] * di;
            a.Dinv[i * 4 + 1] = -D[1] * di;
            a.Dinv[i * 4 + 2] = -D[2] * di;
            a.Dinv[i * 4 + 3] = D[0] * di;
        });
        __syncthreads();
    }
}

__global__ void __launch_bounds__(1024) stencilApply2Kernel(StencilArgs a, const double* __restrict__ d,
                                                             double* __restrict__ v)
{
    if (a.ks && a.ks->status != KS_RUNNING) return;
    const int levels = (a.nx - 1) + 2 * (a.ny - 1) + 4 * (a.nz - 1) + 1;
    for (int L = 0; L < levels; ++L) {
        forLevelRows(a, L, [&](int64_t i) {
            const uint32_t m = a.mask[i];
            double r0 = d[i * 2], r1 = d[i * 2 + 1];
            for (int s = 0; s < a.center; ++s)
                if ((m >> s) & 1u) {
                    const double* B = a.LU + ((int64_t)s * a.N + i) * 4;
                    const double* vj = v + (i + a.off[s]) * 2;
                    r0 = fma(-B[0], vj[0], r0);
                    r0 = fma(-B[1], vj[1], r0);
                    r1 = fma(-B[2], vj[0], r1);
                    r1 = fma(-B[3], vj[1], r1);
                }
            v[i * 2] = r0;
            v[i * 2 + 1] = r1;
        });
        __syncthreads();
    }
    for (int L = levels - 1; L >= 0; --L) {
        forLevelRows(a, L, [&](int64_t i) {
            const uint32_t m = a.mask[i];
            double r0 = v[i * 2], r1 = v[i * 2 + 1];
            for (int s = a.S - 1; s > a.center; --s)
                if ((m >> s) & 1u) {
                    const double* B = a.LU + ((int64_t)s * a.N + i) * 4;
                    const double* vj = v + (i + a.off[s]) * 2;
                    r0 = fma(-B[0], vj[0], r0);
                    r0 = fma(-B[1], vj[1], r0);
                    r1 = fma(-B[2], vj[0], r1);
                    r1 = fma(-B[3], vj[1], r1);
                }
            const double* D = a.Dinv + i * 4;
            double t0 = D[0] * r0;
            t0 = fma(D[1], r1, t0);
            double t1 = D[2] * r0;
            t1 = fma(D[3], r1, t1);
            v[i * 2] = t0;
            v[i * 2 + 1] = t1;
        });
        __syncthreads();
    }
}

void launchStencilSpmv(const StencilArgs& a, const double* x, double* y, const double* w, int mode, cudaStream_t st)
{
    const dim3 g((unsigned)cellBlocksFor(a.N));
    if (a.b == 2) {
        if (a.S == 9) {
            if (mode == 0) stencilSpmv2Kernel<9, 0><<<g, kReduceThreads, 0, st>>>(a, x, y, w);
            else if (mode == 1) stencilSpmv2Kernel<9, 1><<<g, kReduceThreads, 0, st>>>(a, x, y, w);
            else stencilSpmv2Kernel<9, 2><<<g, kReduceThreads, 0, st>>>(a, x, y, w);
        } else {
            if (mode == 0) stencilSpmv2Kernel<27, 0><<<g, kReduceThreads, 0, st>>>(a, x, y, w);
            else if (mode == 1) stencilSpmv2Kernel<27, 1><<<g, kReduceThreads, 0, st>>>(a, x, y, w);
            else stencilSpmv2Kernel<27, 2><<<g, kReduceThreads, 0, st>>>(a, x, y, w);
        }
        DXG_CUDA(cudaGetLastError());
        return;
    }
    if (a.S == 9) {
        if (mode == 0) stencilSpmvKernel<9, 0><<<g, kReduceThreads, 0, st>>>(a, x, y, w);
        else if (mode == 1) stencilSpmvKernel<9, 1><<<g, kReduceThreads, 0, st>>>(a, x, y, w);
        else stencilSpmvKernel<9, 2><<<g, kReduceThreads, 0, st>>>(a, x, y, w);
    } else {
        if (mode == 0) stencilSpmvKernel<27, 0><<<g, kReduceThreads, 0, st>>>(a, x, y, w);
        else if (mode == 1) stencilSpmvKernel<27, 1><<<g, kReduceThreads, 0, st>>>(a, x, y, w);
        else stencilSpmvKernel<27, 2><<<g, kReduceThreads, 0, st>>>(a, x, y, w);
    }
    DXG_CUDA(cudaGetLastError());
}

static unsigned stencilThreads(const StencilArgs& a)
{
    const int lines = a.ny * a.nz;
    const int t = ((lines + 31) / 32) * 32;
    return (unsigned)std::min(1024, std::max(32, t));
}

// 3D (27-point) stencils: the cluster factorisation (the rows carry up to 101 update triples;
// one CTA level by level took 23 ms for a 2p 32x32x16 factor on GB300, the cluster version
// with one warp per row spreads a level over 16 SMs); 2D stencils (12 triples): the cluster
// factorisation from 4096 cells, one CTA below
void launchStencilFactor(const StencilArgs& a, cudaStream_t st)
{
    if (a.S == 27 || a.N >= 4096) {
        launchStencilFactorCluster(a, st);
        return;
    }
    if (a.b == 2) stencilFactor2Kernel<<<1, stencilThreads(a), 0, st>>>(a);
    else stencilFactorKernel<<<1, stencilThreads(a), 0, st>>>(a);
    DXG_CUDA(cudaGetLastError());
}

bool stencilWave2dFits(const StencilArgs& a) { return a.b == 1 && a.S == 9 && a.ny >= 1 && a.ny <= 1024; }

void launchStencilWave2d(const StencilArgs& a, const double* d, double* v, cudaStream_t st)
{
    // ring depth by CTA size: 8 steps up to 256 lines, 4 up to 512, 2 up to 1024
    const unsigned threads = (unsigned)((a.ny + 31) / 32 * 32);
    if (threads <= 256) {
        stencilWave2dKernel<1, 8, 256><<<1, threads, 0, st>>>(a, d, v);
        stencilWave2dKernel<-1, 8, 256><<<1, threads, 0, st>>>(a, d, v);
    } else if (threads <= 512) {
        stencilWave2dKernel<1, 4, 512><<<1, threads, 0, st>>>(a, d, v);
        stencilWave2dKernel<-1, 4, 512><<<1, threads, 0, st>>>(a, d, v);
    } else {
        stencilWave2dKernel<1, 2, 1024><<<1, threads, 0, st>>>(a, d, v);
        stencilWave2dKernel<-1, 2, 1024><<<1, threads, 0, st>>>(a, d, v);
    }
    DXG_CUDA(cudaGetLastError());
}

void launchStencilApplyLevels(const StencilArgs& a, const double* d, double* v, cudaStream_t st)
{
    if (a.b == 2) stencilApply2Kernel<<<1, stencilThreads(a), 0, st>>>(a, d, v);
    else stencilApplyKernel<<<1, stencilThreads(a), 0, st>>>(a, d, v);
    DXG_CUDA(cudaGetLastError());
}

}  // namespace dxg
