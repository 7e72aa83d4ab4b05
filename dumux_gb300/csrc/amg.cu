// amg.cu -- aggregation AMG kernels (setup and V-cycle) on the structured stencil.
#include "amg.cuh"

#include <cooperative_groups.h>

namespace cg = cooperative_groups;

namespace dxg {

namespace {

constexpr int kAmgThreads = 256;

// neighbour of (x, y, z) through slot s (3D: -z,-y,-x,diag,+x,+y,+z; 2D: -y,-x,diag,+x,+y):
// false when it leaves the grid; *d = index offset
template <int DIM>
__device__ __forceinline__ bool neighbour(int s, int x, int y, int z, int nx, int ny, int nz, int64_t* d)
{
    const int axis = s < DIM ? DIM - 1 - s : s - DIM - 1;
    const int sign = s < DIM ? -1 : 1;
    const int c = axis == 0 ? x : (axis == 1 ? y : z);
    const int n = axis == 0 ? nx : (axis == 1 ? ny : nz);
    const int64_t stride = axis == 0 ? 1 : (axis == 1 ? (int64_t)nx : (int64_t)nx * ny);
    *d = sign * stride;
    return sign < 0 ? c > 0 : c < n - 1;
}

template <int B, class T>
__device__ __forceinline__ void ldBlk(const T* p, T* o)
{
#pragma unroll
    for (int e = 0; e < B * B; ++e) o[e] = p[e];
}
template <int B, class T>
__device__ __forceinline__ bool invBlk(const T* A, T* inv)
{
    if (B == 1) {
        inv[0] = (T)1 / A[0];
        return A[0] != (T)0;
    } else {
        const T det = A[0] * A[3] - A[1] * A[2];
        if (det == (T)0) return false;
        const T r = (T)1 / det;
        inv[0] = A[3] * r;
        inv[1] = -A[1] * r;
        inv[2] = -A[2] * r;
        inv[3] = A[0] * r;
        return true;
    }
}
// y = M v (B x B block times B-vector)
template <int B, class T>
__device__ __forceinline__ void mv(const T* M, const T* v, T* y)
{
#pragma unroll
    for (int r = 0; r < B; ++r) {
        T t = M[r * B] * v[0];
#pragma unroll
        for (int c = 1; c < B; ++c) t = fma(M[r * B + c], v[c], t);
        y[r] = t;
    }
}

#define AMG_LOOP(L)                                                                                 \
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (L).N;                   \
         i += (int64_t)gridDim.x * blockDim.x)

__device__ __forceinline__ void coordOf(int64_t i, int nx, int ny, int& x, int& y, int& z)
{
    x = (int)(i % nx);
    y = (int)((i / nx) % ny);
    z = (int)(i / ((int64_t)nx * ny));
}

template <int B, class T>
__device__ __forceinline__ void diagInvCell(const AmgLevel<T>& L, int64_t i, int dim, int* singular)
{
    constexpr int BB = B * B;
    T D[BB], inv[BB];
    ldBlk<B>(L.A + ((int64_t)dim * L.N + i) * BB, D);
    if (!invBlk<B>(D, inv)) *singular = 1;
#pragma unroll
    for (int e = 0; e < BB; ++e) L.Dinv[i * BB + e] = inv[e];
}

template <int B, class T>
__global__ void amgDiagInvKernel(AmgLevel<T> L, int dim, int* singular)
{
    AMG_LOOP(L) diagInvCell<B, T>(L, i, dim, singular);
}

// coarse cell C = block sums over its aggregate's fine cells (fixed order: z, y, x, slot)
template <int B, int DIM, class T>
__device__ __forceinline__ void coarsenCell(const AmgLevel<T>& F, const AmgLevel<T>& C, int64_t i, int* singular)
{
    constexpr int BB = B * B, S = 2 * DIM + 1;
    T* Ac = const_cast<T*>(C.A);
    {
        int cx, cy, cz;
        coordOf(i, C.nx, C.ny, cx, cy, cz);
        T acc[S][BB];
#pragma unroll
        for (int s = 0; s < S; ++s)
#pragma unroll
            for (int e = 0; e < BB; ++e) acc[s][e] = 0;
        for (int dz = 0; dz < (DIM == 3 ? 2 : 1); ++dz) {
            const int z = 2 * cz + dz;
            if (z >= F.nz) continue;
            for (int dy = 0; dy < 2; ++dy) {
                const int y = 2 * cy + dy;
                if (y >= F.ny) continue;
                for (int dx = 0; dx < 2; ++dx) {
                    const int x = 2 * cx + dx;
                    if (x >= F.nx) continue;
                    const int64_t f = x + (int64_t)F.nx * (y + (int64_t)F.ny * z);
#pragma unroll
                    for (int s = 0; s < S; ++s) {
                        int target = DIM;
                        if (s != DIM) {
                            int64_t d;
                            if (!neighbour<DIM>(s, x, y, z, F.nx, F.ny, F.nz, &d)) continue;
                            // leaves the aggregate when the neighbour's coarse coordinate differs
                            const int axis = s < DIM ? DIM - 1 - s : s - DIM - 1;
                            const int c = axis == 0 ? x : (axis == 1 ? y : z);
                            const int cn = c + (s < DIM ? -1 : 1);
                            if ((cn >> 1) != (c >> 1)) target = s;
                        }
                        const T* blk = F.A + ((int64_t)s * F.N + f) * BB;
#pragma unroll
                        for (int e = 0; e < BB; ++e) acc[target][e] += blk[e];
                    }
                }
            }
        }
#pragma unroll
        for (int s = 0; s < S; ++s)
#pragma unroll
            for (int e = 0; e < BB; ++e) Ac[((int64_t)s * C.N + i) * BB + e] = acc[s][e];
        T inv[BB];
        if (!invBlk<B>(acc[DIM], inv)) *singular = 1;
#pragma unroll
        for (int e = 0; e < BB; ++e) C.Dinv[i * BB + e] = inv[e];
    }
}

template <int B, int DIM, class T>
__global__ void amgCoarsenKernel(AmgLevel<T> F, AmgLevel<T> C, int* singular)
{
    AMG_LOOP(C) coarsenCell<B, DIM, T>(F, C, i, singular);
}

// sum_s A_is x_j over the existing neighbours and the diagonal
template <int B, int DIM, class T>
__device__ __forceinline__ void rowTimes(const AmgLevel<T>& L, int64_t i, const T* xv, const T* xc, int cnx, int cny,
                                         T* out)
{
    constexpr int BB = B * B, S = 2 * DIM + 1;
    int x, y, z;
    coordOf(i, L.nx, L.ny, x, y, z);
#pragma unroll
    for (int e = 0; e < B; ++e) out[e] = 0;
#pragma unroll
    for (int s = 0; s < S; ++s) {
        int64_t d = 0;
        int jx = x, jy = y, jz = z;
        if (s != DIM) {
            if (!neighbour<DIM>(s, x, y, z, L.nx, L.ny, L.nz, &d)) continue;
            const int axis = s < DIM ? DIM - 1 - s : s - DIM - 1;
            const int sg = s < DIM ? -1 : 1;
            if (axis == 0) jx += sg;
            else if (axis == 1) jy += sg;
            else jz += sg;
        }
        const int64_t j = i + d;
        T v[B];
#pragma unroll
        for (int e = 0; e < B; ++e) v[e] = xv[j * B + e];
        if (xc) {   // prolongation on the fly: x~_j = x_j + xc[aggregate of j]
            const int64_t C = (jx >> 1) + (int64_t)cnx * ((jy >> 1) + (int64_t)cny * (jz >> 1));
#pragma unroll
            for (int e = 0; e < B; ++e) v[e] += xc[C * B + e];
        }
        T blk[BB], t[B];
        ldBlk<B>(L.A + ((int64_t)s * L.N + i) * BB, blk);
        mv<B>(blk, v, t);
#pragma unroll
        for (int e = 0; e < B; ++e) out[e] += t[e];
    }
}

template <class T>
__device__ __forceinline__ bool stopped(const KrylovState* ks)
{
    return ks && ks->status != KS_RUNNING;
}

// ---- per-cell bodies of the V-cycle passes (shared by the per-level kernels and the
// cluster kernel of the small levels)

// out = omega D^-1 b
template <int B, class T>
__device__ __forceinline__ void firstCell(const AmgLevel<T>& L, int64_t i, T* out, T omega)
{
    constexpr int BB = B * B;
    T D[BB], bi[B], y[B];
    ldBlk<B>(L.Dinv + i * BB, D);
#pragma unroll
    for (int e = 0; e < B; ++e) bi[e] = L.b[i * B + e];
    mv<B>(D, bi, y);
#pragma unroll
    for (int e = 0; e < B; ++e) out[i * B + e] = omega * y[e];
}

// out = x~ + omega D^-1 (b - A x~), x~ = xin (+ prolongated xc when given)
template <int B, int DIM, class T>
__device__ __forceinline__ void jacobiCell(const AmgLevel<T>& L, int64_t i, const T* xin, const T* xc, int cnx, int cny,
                                           T* out, T omega)
{
    constexpr int BB = B * B;
    T ax[B], res[B], D[BB], y[B];
    rowTimes<B, DIM, T>(L, i, xin, xc, cnx, cny, ax);
#pragma unroll
    for (int e = 0; e < B; ++e) res[e] = L.b[i * B + e] - ax[e];
    ldBlk<B>(L.Dinv + i * BB, D);
    mv<B>(D, res, y);
    int x, yy, z;
    coordOf(i, L.nx, L.ny, x, yy, z);
    const int64_t C = xc ? (x >> 1) + (int64_t)cnx * ((yy >> 1) + (int64_t)cny * (z >> 1)) : 0;
#pragma unroll
    for (int e = 0; e < B; ++e) {
        T xi = xin[i * B + e];
        if (xc) xi += xc[C * B + e];
        out[i * B + e] = xi + omega * y[e];
    }
}

// r = b - A x
template <int B, int DIM, class T>
__device__ __forceinline__ void residualCell(const AmgLevel<T>& L, int64_t i, const T* xin)
{
    T ax[B];
    rowTimes<B, DIM, T>(L, i, xin, nullptr, 0, 0, ax);
#pragma unroll
    for (int e = 0; e < B; ++e) L.r[i * B + e] = L.b[i * B + e] - ax[e];
}

// coarse b = sum of the aggregate's fine residuals (fixed order)
template <int B, int DIM, class T>
__device__ __forceinline__ void restrictCell(const AmgLevel<T>& F, const AmgLevel<T>& C, int64_t i)
{
    int cx, cy, cz;
    coordOf(i, C.nx, C.ny, cx, cy, cz);
    T acc[B];
#pragma unroll
    for (int e = 0; e < B; ++e) acc[e] = 0;
    for (int dz = 0; dz < (DIM == 3 ? 2 : 1); ++dz) {
        const int z = 2 * cz + dz;
        if (z >= F.nz) continue;
        for (int dy = 0; dy < 2; ++dy) {
            const int y = 2 * cy + dy;
            if (y >= F.ny) continue;
            for (int dx = 0; dx < 2; ++dx) {
                const int x = 2 * cx + dx;
                if (x >= F.nx) continue;
                const int64_t f = x + (int64_t)F.nx * (y + (int64_t)F.ny * z);
#pragma unroll
                for (int e = 0; e < B; ++e) acc[e] += F.r[f * B + e];
            }
        }
    }
#pragma unroll
    for (int e = 0; e < B; ++e) C.b[i * B + e] = acc[e];
}

// row i of x = Ainv b on the last level
template <class T>
__device__ __forceinline__ void coarseRow(const AmgLevel<T>& L, int n, int i)
{
    T t = 0;
    for (int j = 0; j < n; ++j) t = fma(L.Ainv[(int64_t)i * n + j], L.b[j], t);
    L.x[i] = t;
}

template <int B, class T>
__global__ void amgFirstKernel(AmgLevel<T> L, T* out, T omega, const KrylovState* ks)
{
    if (stopped<T>(ks)) return;
    AMG_LOOP(L) firstCell<B, T>(L, i, out, omega);
}

template <int B, int DIM, class T>
__global__ void amgJacobiKernel(AmgLevel<T> L, const T* xin, const T* xc, int cnx, int cny, T* out, T omega,
                                const KrylovState* ks)
{
    if (stopped<T>(ks)) return;
    AMG_LOOP(L) jacobiCell<B, DIM, T>(L, i, xin, xc, cnx, cny, out, omega);
}

template <int B, int DIM, class T>
__global__ void amgResidualKernel(AmgLevel<T> L, const T* xin, const KrylovState* ks)
{
    if (stopped<T>(ks)) return;
    AMG_LOOP(L) residualCell<B, DIM, T>(L, i, xin);
}

template <int B, int DIM, class T>
__global__ void amgRestrictKernel(AmgLevel<T> F, AmgLevel<T> C, const KrylovState* ks)
{
    if (stopped<T>(ks)) return;
    AMG_LOOP(C) restrictCell<B, DIM, T>(F, C, i);
}

// The V-cycle below a level of at most kAmgClusterLevel cells as one launch of one thread
// block cluster: every pass is a loop over the level's cells across the cluster's threads,
// followed by a cluster barrier (release/acquire at cluster scope orders the passes' global
// memory traffic).  Same per-cell arithmetic and pass order as the per-level kernels.
constexpr int kAmgMaxClusterLevels = 12;
constexpr int kAmgClusterCtas = 16;
constexpr int kAmgClusterThreads = 512;
template <class T>
struct AmgCycle {
    AmgLevel<T> lv[kAmgMaxClusterLevels];
    int count;
};

template <int B, int DIM, class T>
__global__ void __launch_bounds__(kAmgClusterThreads) amgClusterCycle(AmgCycle<T> cy, const KrylovState* ks)
{
    if (stopped<T>(ks)) return;   // uniform: the status does not change during the launch
    cg::cluster_group cl = cg::this_cluster();
    const int64_t gid = (int64_t)cl.block_rank() * blockDim.x + threadIdx.x;
    const int64_t gstride = (int64_t)cl.num_blocks() * blockDim.x;
    const T omega = (T)kAmgOmega;
    const T* pre[kAmgMaxClusterLevels];
    const int last = cy.count - 1;
    for (int l = 0; l < last; ++l) {
        const AmgLevel<T>& L = cy.lv[l];
        T* buf[2] = {L.tmp, L.x};
        int w = 0;
        for (int64_t i = gid; i < L.N; i += gstride) firstCell<B, T>(L, i, buf[0], omega);
        cl.sync();
        for (int k = 1; k < L.sweeps; ++k, ++w) {
            for (int64_t i = gid; i < L.N; i += gstride)
                jacobiCell<B, DIM, T>(L, i, buf[w & 1], nullptr, 0, 0, buf[(w + 1) & 1], omega);
            cl.sync();
        }
        pre[l] = buf[w & 1];
        for (int64_t i = gid; i < L.N; i += gstride) residualCell<B, DIM, T>(L, i, pre[l]);
        cl.sync();
        for (int64_t i = gid; i < cy.lv[l + 1].N; i += gstride) restrictCell<B, DIM, T>(L, cy.lv[l + 1], i);
        cl.sync();
    }
    {
        const AmgLevel<T>& L = cy.lv[last];
        const int n = (int)L.N * B;
        for (int64_t i = gid; i < n; i += gstride) coarseRow<T>(L, n, (int)i);
        cl.sync();
    }
    for (int l = last - 1; l >= 0; --l) {
        const AmgLevel<T>& L = cy.lv[l];
        const AmgLevel<T>& C = cy.lv[l + 1];
        T* buf[2] = {L.tmp, L.x};
        int w = L.sweeps - 1;   // index of the last pre-smoothing write
        for (int64_t i = gid; i < L.N; i += gstride)
            jacobiCell<B, DIM, T>(L, i, pre[l], C.x, C.nx, C.ny, buf[(w + 1) & 1], omega);
        ++w;
        cl.sync();
        for (int k = 1; k < L.sweeps; ++k, ++w) {
            for (int64_t i = gid; i < L.N; i += gstride)
                jacobiCell<B, DIM, T>(L, i, buf[w & 1], nullptr, 0, 0, buf[(w + 1) & 1], omega);
            cl.sync();
        }
    }
}

// Dense inverse of a level of at most kAmgCoarsest cells: the block stencil is expanded
// into an n x n matrix (n = N*b) in shared memory and inverted in place by Gauss-Jordan
// elimination with partial pivoting (row exchanges, undone as column exchanges in reverse
// order at the end); one CTA.
template <int B, int DIM, class T>
__device__ void coarseInvertCta(const AmgLevel<T>& L, int* singular, unsigned char* smemRaw)
{
    constexpr int BB = B * B, S = 2 * DIM + 1;
    const int n = (int)L.N * B;
    T* a = reinterpret_cast<T*>(smemRaw);   // [n][n]
    T* f = a + n * n;                       // column k before the elimination
    int* swapRow = reinterpret_cast<int*>(f + n);
    __shared__ int piv;
    __shared__ bool bad;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) a[e] = 0;
    if (threadIdx.x == 0) bad = false;
    __syncthreads();
    for (int i = threadIdx.x; i < (int)L.N; i += blockDim.x) {
        int x, y, z;
        coordOf(i, L.nx, L.ny, x, y, z);
        for (int s = 0; s < S; ++s) {
            int64_t d = 0;
            if (s != DIM && !neighbour<DIM>(s, x, y, z, L.nx, L.ny, L.nz, &d)) continue;
            const int j = i + (int)d;
            const T* blk = L.A + ((int64_t)s * L.N + i) * BB;
            for (int r = 0; r < B; ++r)
                for (int c = 0; c < B; ++c) a[(i * B + r) * n + j * B + c] = blk[r * B + c];
        }
    }
    __syncthreads();
    for (int k = 0; k < n; ++k) {
        if (threadIdx.x < 32) {
            // pivot: the largest magnitude in column k at or below row k (lowest row on ties)
            T best = -1;
            int row = k;
            for (int i = k + threadIdx.x; i < n; i += 32) {
                const T v = fabs(a[i * n + k]);
                if (v > best) { best = v; row = i; }
            }
            for (int o = 16; o > 0; o >>= 1) {
                const T ob = __shfl_down_sync(0xffffffffu, best, o);
                const int orow = __shfl_down_sync(0xffffffffu, row, o);
                if (ob > best || (ob == best && orow < row)) { best = ob; row = orow; }
            }
            if (threadIdx.x == 0) {
                piv = row;
                swapRow[k] = row;
                if (!(best > 0)) bad = true;
            }
        }
        __syncthreads();
        if (bad) break;
        if (piv != k)
            for (int c = threadIdx.x; c < n; c += blockDim.x) {
                const T t = a[k * n + c];
                a[k * n + c] = a[piv * n + c];
                a[piv * n + c] = t;
            }
        __syncthreads();
        const T dinv = (T)1 / a[k * n + k];
        __syncthreads();
        for (int c = threadIdx.x; c < n; c += blockDim.x) a[k * n + c] = c == k ? dinv : a[k * n + c] * dinv;
        for (int i = threadIdx.x; i < n; i += blockDim.x) f[i] = i == k ? (T)0 : a[i * n + k];
        __syncthreads();
        for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
            const int i = e / n, c = e % n;
            if (i == k) continue;
            a[e] = c == k ? -f[i] * a[k * n + k] : a[e] - f[i] * a[k * n + c];
        }
        __syncthreads();
    }
    if (bad) {
        if (threadIdx.x == 0) *singular = 1;
        return;
    }
    for (int k = n - 1; k >= 0; --k) {
        const int p = swapRow[k];
        if (p != k)
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                const T t = a[i * n + k];
                a[i * n + k] = a[i * n + p];
                a[i * n + p] = t;
            }
        __syncthreads();
    }
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) L.Ainv[e] = a[e];
}

template <int B, int DIM, class T>
__global__ void amgCoarseInvertKernel(AmgLevel<T> L, int* singular)
{
    extern __shared__ __align__(16) unsigned char smemRaw[];
    coarseInvertCta<B, DIM, T>(L, singular, smemRaw);
}

// x = Ainv b on the last level (one row per thread, fixed order)
template <class T>
__global__ void amgCoarseSolveKernel(AmgLevel<T> L, int n, const KrylovState* ks)
{
    if (stopped<T>(ks)) return;
    for (int i = threadIdx.x; i < n; i += blockDim.x) coarseRow<T>(L, n, i);
}

// ---- batched passes: one launch runs one pass for several problems, block k of the
// grid working on problem map[k].x as its block map[k].y of amgPassBlocks(items)
__host__ __device__ __forceinline__ int64_t passItems(int kind, int64_t LN, int64_t CN, int b)
{
    return (kind == AMG_RESTRICT || kind == AMG_COARSEN) ? CN : (kind == AMG_COARSE ? LN * b : LN);
}

template <int B, int DIM, class T, int KIND>
__global__ void __launch_bounds__(kAmgThreads) amgPassBatch(const AmgPass<T>* passes, const uint2* map)
{
    const uint2 m = map[blockIdx.x];
    const AmgPass<T>& P = passes[m.x];
    if (stopped<T>(P.ks)) return;
    const int64_t n = passItems(KIND, P.L.N, P.C.N, B);
    const unsigned nblk = amgPassBlocks(n);
    if (m.y >= nblk) return;
    for (int64_t i = m.y * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)nblk * blockDim.x) {
        if constexpr (KIND == AMG_FIRST) firstCell<B, T>(P.L, i, P.out, P.omega);
        else if constexpr (KIND == AMG_JACOBI)
            jacobiCell<B, DIM, T>(P.L, i, P.in, P.prolong ? P.C.x : nullptr, P.C.nx, P.C.ny, P.out, P.omega);
        else if constexpr (KIND == AMG_RESIDUAL) residualCell<B, DIM, T>(P.L, i, P.in);
        else if constexpr (KIND == AMG_RESTRICT) restrictCell<B, DIM, T>(P.L, P.C, i);
        else if constexpr (KIND == AMG_COARSE) coarseRow<T>(P.L, (int)n, (int)i);
        else if constexpr (KIND == AMG_DIAGINV) diagInvCell<B, T>(P.L, i, DIM, P.singular);
        else coarsenCell<B, DIM, T>(P.L, P.C, i, P.singular);
    }
}

// one CTA per problem: dense inverse of its last level
template <int B, int DIM, class T>
__global__ void amgInvertBatch(const AmgPass<T>* passes)
{
    extern __shared__ __align__(16) unsigned char smemRaw[];
    const AmgPass<T>& P = passes[blockIdx.x];
    coarseInvertCta<B, DIM, T>(P.L, P.singular, smemRaw);
}

unsigned gridFor(int64_t n)
{
    int64_t g = (n + kAmgThreads - 1) / kAmgThreads;
    if (g > 4096) g = 4096;
    return (unsigned)(g < 1 ? 1 : g);
}

template <class T, int B, int DIM>
int64_t vcycle(const std::vector<AmgLevel<T>>& Ls, size_t l, const KrylovState* ks, cudaStream_t st)
{
    const AmgLevel<T>& L = Ls[l];
    const unsigned g = gridFor(L.N);
    if (L.N <= kAmgClusterLevel && Ls.size() - l <= (size_t)kAmgMaxClusterLevels) {
        // this level and all below: one cluster launch
        AmgCycle<T> cy{};
        cy.count = (int)(Ls.size() - l);
        for (int k = 0; k < cy.count; ++k) cy.lv[k] = Ls[l + k];
        auto kern = amgClusterCycle<B, DIM, T>;
        DXG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(kAmgClusterCtas);
        cfg.blockDim = dim3(kAmgClusterThreads);
        cfg.stream = st;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = kAmgClusterCtas;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        DXG_CUDA(cudaLaunchKernelEx(&cfg, kern, cy, ks));
        return 1;
    }
    if (l + 1 == Ls.size()) {
        amgCoarseSolveKernel<T><<<1, kAmgThreads, 0, st>>>(L, (int)L.N * B, ks);   // exact solve
        return 1;
    }
    const AmgLevel<T>& C = Ls[l + 1];
    const T omega = (T)kAmgOmega;
    int64_t n = 0;
    // 2*sweeps writes alternate between tmp and x, the last one into x
    T* buf[2] = {L.tmp, L.x};
    int w = 0;
    amgFirstKernel<B, T><<<g, kAmgThreads, 0, st>>>(L, buf[w & 1], omega, ks);
    ++n;
    for (int k = 1; k < L.sweeps; ++k, ++w, ++n)
        amgJacobiKernel<B, DIM, T><<<g, kAmgThreads, 0, st>>>(L, buf[w & 1], nullptr, 0, 0, buf[(w + 1) & 1], omega,
                                                              ks);
    const T* pre = buf[w & 1];
    amgResidualKernel<B, DIM, T><<<g, kAmgThreads, 0, st>>>(L, pre, ks);
    amgRestrictKernel<B, DIM, T><<<gridFor(C.N), kAmgThreads, 0, st>>>(L, C, ks);
    n += 2;
    n += vcycle<T, B, DIM>(Ls, l + 1, ks, st);
    // prolongation fused into the first post-sweep
    amgJacobiKernel<B, DIM, T><<<g, kAmgThreads, 0, st>>>(L, pre, C.x, C.nx, C.ny, buf[(w + 1) & 1], omega, ks);
    ++w;
    ++n;
    for (int k = 1; k < L.sweeps; ++k, ++w, ++n)
        amgJacobiKernel<B, DIM, T><<<g, kAmgThreads, 0, st>>>(L, buf[w & 1], nullptr, 0, 0, buf[(w + 1) & 1], omega,
                                                              ks);
    return n;
}

}  // namespace

std::vector<std::array<int, 3>> amgLevelDims(int dim, int nx, int ny, int nz)
{
    std::vector<std::array<int, 3>> out;
    int n[3] = {nx, ny, dim == 3 ? nz : 1};
    while (n[0] * (int64_t)n[1] * n[2] > kAmgCoarsest) {
        for (int a = 0; a < 3; ++a) n[a] = (n[a] + 1) / 2;
        out.push_back({n[0], n[1], n[2]});
    }
    return out;
}

template <class T>
void launchAmgDiagInv(const AmgLevel<T>& L, int dim, int b, int* singular, cudaStream_t st)
{
    const unsigned g = gridFor(L.N);
    if (b == 1) amgDiagInvKernel<1, T><<<g, kAmgThreads, 0, st>>>(L, dim, singular);
    else amgDiagInvKernel<2, T><<<g, kAmgThreads, 0, st>>>(L, dim, singular);
    DXG_CUDA(cudaGetLastError());
}

template <class T>
void launchAmgCoarsen(const AmgLevel<T>& fine, AmgLevel<T>& coarse, int dim, int b, int* singular, cudaStream_t st)
{
    const unsigned g = gridFor(coarse.N);
    if (b == 1) {
        if (dim == 2) amgCoarsenKernel<1, 2, T><<<g, kAmgThreads, 0, st>>>(fine, coarse, singular);
        else amgCoarsenKernel<1, 3, T><<<g, kAmgThreads, 0, st>>>(fine, coarse, singular);
    } else {
        if (dim == 2) amgCoarsenKernel<2, 2, T><<<g, kAmgThreads, 0, st>>>(fine, coarse, singular);
        else amgCoarsenKernel<2, 3, T><<<g, kAmgThreads, 0, st>>>(fine, coarse, singular);
    }
    DXG_CUDA(cudaGetLastError());
}

template <class T>
void launchAmgCoarseInvert(const AmgLevel<T>& L, int dim, int b, int* singular, cudaStream_t st)
{
    const int n = (int)L.N * b;
    const size_t smem = (size_t)n * n * sizeof(T) + (size_t)n * sizeof(T) + (size_t)n * sizeof(int);
    auto go = [&](auto kern) {
        DXG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kern<<<1, kAmgThreads, smem, st>>>(L, singular);
    };
    if (b == 1) dim == 2 ? go(amgCoarseInvertKernel<1, 2, T>) : go(amgCoarseInvertKernel<1, 3, T>);
    else dim == 2 ? go(amgCoarseInvertKernel<2, 2, T>) : go(amgCoarseInvertKernel<2, 3, T>);
    DXG_CUDA(cudaGetLastError());
}

template <class T>
int64_t launchAmgVcycle(const std::vector<AmgLevel<T>>& levels, int dim, int b, const KrylovState* ks,
                        cudaStream_t st)
{
    int64_t n;
    if (b == 1) n = dim == 2 ? vcycle<T, 1, 2>(levels, 0, ks, st) : vcycle<T, 1, 3>(levels, 0, ks, st);
    else n = dim == 2 ? vcycle<T, 2, 2>(levels, 0, ks, st) : vcycle<T, 2, 3>(levels, 0, ks, st);
    DXG_CUDA(cudaGetLastError());
    return n;
}

template <class T, int B, int DIM>
static void passDispatch(int kind, const AmgPass<T>* p, const uint2* map, unsigned blocks, cudaStream_t st)
{
    switch (kind) {
        case AMG_FIRST: amgPassBatch<B, DIM, T, AMG_FIRST><<<blocks, kAmgThreads, 0, st>>>(p, map); break;
        case AMG_JACOBI: amgPassBatch<B, DIM, T, AMG_JACOBI><<<blocks, kAmgThreads, 0, st>>>(p, map); break;
        case AMG_RESIDUAL: amgPassBatch<B, DIM, T, AMG_RESIDUAL><<<blocks, kAmgThreads, 0, st>>>(p, map); break;
        case AMG_RESTRICT: amgPassBatch<B, DIM, T, AMG_RESTRICT><<<blocks, kAmgThreads, 0, st>>>(p, map); break;
        case AMG_COARSE: amgPassBatch<B, DIM, T, AMG_COARSE><<<blocks, kAmgThreads, 0, st>>>(p, map); break;
        case AMG_DIAGINV: amgPassBatch<B, DIM, T, AMG_DIAGINV><<<blocks, kAmgThreads, 0, st>>>(p, map); break;
        default: amgPassBatch<B, DIM, T, AMG_COARSEN><<<blocks, kAmgThreads, 0, st>>>(p, map); break;
    }
}

template <class T>
void launchAmgPassBatch(int kind, const AmgPass<T>* passes, const uint2* map, unsigned blocks, int dim, int b,
                        cudaStream_t st)
{
    if (b == 1) dim == 2 ? passDispatch<T, 1, 2>(kind, passes, map, blocks, st)
                         : passDispatch<T, 1, 3>(kind, passes, map, blocks, st);
    else dim == 2 ? passDispatch<T, 2, 2>(kind, passes, map, blocks, st)
                  : passDispatch<T, 2, 3>(kind, passes, map, blocks, st);
    DXG_CUDA(cudaGetLastError());
}

template <class T>
void launchAmgInvertBatch(const AmgPass<T>* passes, int count, int maxN, int dim, int b, cudaStream_t st)
{
    const int n = maxN * b;
    const size_t smem = (size_t)n * n * sizeof(T) + (size_t)n * sizeof(T) + (size_t)n * sizeof(int);
    auto go = [&](auto kern) {
        DXG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kern<<<count, kAmgThreads, smem, st>>>(passes);
    };
    if (b == 1) dim == 2 ? go(amgInvertBatch<1, 2, T>) : go(amgInvertBatch<1, 3, T>);
    else dim == 2 ? go(amgInvertBatch<2, 2, T>) : go(amgInvertBatch<2, 3, T>);
    DXG_CUDA(cudaGetLastError());
}

template void launchAmgPassBatch<double>(int, const AmgPass<double>*, const uint2*, unsigned, int, int, cudaStream_t);
template void launchAmgPassBatch<float>(int, const AmgPass<float>*, const uint2*, unsigned, int, int, cudaStream_t);
template void launchAmgInvertBatch<double>(const AmgPass<double>*, int, int, int, int, cudaStream_t);
template void launchAmgInvertBatch<float>(const AmgPass<float>*, int, int, int, int, cudaStream_t);
template void launchAmgDiagInv<double>(const AmgLevel<double>&, int, int, int*, cudaStream_t);
template void launchAmgDiagInv<float>(const AmgLevel<float>&, int, int, int*, cudaStream_t);
template void launchAmgCoarseInvert<double>(const AmgLevel<double>&, int, int, int*, cudaStream_t);
template void launchAmgCoarseInvert<float>(const AmgLevel<float>&, int, int, int*, cudaStream_t);
template void launchAmgCoarsen<double>(const AmgLevel<double>&, AmgLevel<double>&, int, int, int*, cudaStream_t);
template void launchAmgCoarsen<float>(const AmgLevel<float>&, AmgLevel<float>&, int, int, int*, cudaStream_t);
template int64_t launchAmgVcycle<double>(const std::vector<AmgLevel<double>>&, int, int, const KrylovState*,
                                         cudaStream_t);
template int64_t launchAmgVcycle<float>(const std::vector<AmgLevel<float>>&, int, int, const KrylovState*,
                                        cudaStream_t);

}  // namespace dxg
