// amg.cuh -- aggregation algebraic multigrid on the structured cc-TPFA stencil, the
// preconditioner of the AMG-BiCGSTAB solver variant (AMGBiCGSTABIstlSolver,
// dumux/linear/istlsolvers.hh:729-736, whose AMG is dune-istl's Amg::AMG).
//
// GB300 restatement of aggregation AMG (Blatt & Bastian's aggregation with piecewise
// constant prolongation, Galerkin coarse operators, smoothed V-cycle):
//   * aggregates are 2x2(x2) boxes of the structured grid, so every coarse operator
//     P^T A P is again a block 5/7-point stencil on a grid of half the extent (block
//     sums: couplings inside an aggregate add to its diagonal, couplings across a face
//     to the coarse neighbour in that direction); coarsening stops at 64 cells or fewer;
//   * the smoother is damped block Jacobi (omega = 0.8): the fully parallel counterpart
//     of the reference's SSOR; one pre- and one post-sweep per level, two each on
//     levels of at most 4096 cells;
//   * the last level is solved exactly: its dense inverse (Gauss-Jordan elimination
//     with partial pivoting in one CTA's shared memory) is formed at setup and applied
//     as one dense matrix-vector product;
//   * the V-cycle is a fixed linear operator, so it preconditions BiCGSTAB;
//   * the levels of at most 4096 cells run as one launch of a 16-CTA thread block
//     cluster (passes separated by cluster barriers) instead of a few-microsecond
//     launch per pass.
// Every kernel is a pass over one level's cells (bandwidth bound); the setup (pivot
// inverses, coarse operators) runs once per Jacobian.
#pragma once

#include <array>
#include <cstdint>
#include <vector>

#include "common.cuh"
#include "linalg.cuh"

namespace dxg {

template <class T>
struct AmgLevel {
    int nx = 1, ny = 1, nz = 1;
    int64_t N = 0;
    const T* A = nullptr;     // slot matrix [2*dim+1][N][b*b]
    T* Dinv = nullptr;        // inverted diagonal blocks [N][b*b]
    T* b = nullptr;           // right-hand side (level 0: the preconditioner input)
    T* x = nullptr;           // result (level 0: the preconditioner output)
    T* tmp = nullptr;         // Jacobi ping-pong partner of x
    T* r = nullptr;           // residual
    int sweeps = 1;           // pre- and post-smoothing sweeps
    T* Ainv = nullptr;        // last level: dense inverse [(N*b)^2]
};

constexpr double kAmgOmega = 0.8;
constexpr int64_t kAmgSmallLevel = 4096;
constexpr int kAmgSmallSweeps = 2;
constexpr int64_t kAmgCoarsest = 64;   // cells of the directly solved last level (at most)
constexpr int64_t kAmgClusterLevel = 4096;    // levels this small and below: one cluster launch

// One pass of a V-cycle or of the setup for one problem of a batch.
enum { AMG_FIRST = 0, AMG_JACOBI = 1, AMG_RESIDUAL = 2, AMG_RESTRICT = 3, AMG_COARSE = 4, AMG_DIAGINV = 5,
       AMG_COARSEN = 6 };
template <class T>
struct AmgPass {
    AmgLevel<T> L;            // the level of the pass (restrict, coarsen: the finer level)
    AmgLevel<T> C;            // the coarser level (restrict, coarsen, prolongation)
    const T* in = nullptr;    // Jacobi / residual input
    T* out = nullptr;         // first / Jacobi output
    int prolong = 0;          // Jacobi: the input is in + the prolongated C.x
    T omega = 0;
    int* singular = nullptr;
    const KrylovState* ks = nullptr;   // V-cycle passes skip once the solve has stopped
};
// blocks a batched pass gives one problem with `items` work items (256 threads each)
__host__ __device__ inline unsigned amgPassBlocks(int64_t items)
{
    int64_t g = (items + 255) / 256;
    if (g > 1024) g = 1024;
    return (unsigned)(g < 1 ? 1 : g);
}
template <class T>
void launchAmgPassBatch(int kind, const AmgPass<T>* passes, const uint2* map, unsigned blocks, int dim, int b,
                        cudaStream_t st);
// one CTA per problem: the dense inverse of each problem's last level (maxN: its largest cell count)
template <class T>
void launchAmgInvertBatch(const AmgPass<T>* passes, int count, int maxN, int dim, int b, cudaStream_t st);

// Grid extents of the levels below a fine grid (2D: nz = 1), the last one of at most
// kAmgCoarsest cells (none when the fine grid is that small).
std::vector<std::array<int, 3>> amgLevelDims(int dim, int nx, int ny, int nz);

template <class T>
void launchAmgDiagInv(const AmgLevel<T>& L, int dim, int b, int* singular, cudaStream_t st);
template <class T>
void launchAmgCoarsen(const AmgLevel<T>& fine, AmgLevel<T>& coarse, int dim, int b, int* singular,
                      cudaStream_t st);
// dense inverse of the last level into L.Ainv
template <class T>
void launchAmgCoarseInvert(const AmgLevel<T>& L, int dim, int b, int* singular, cudaStream_t st);
// x = V-cycle(b) from level l down; returns the number of kernels launched
template <class T>
int64_t launchAmgVcycle(const std::vector<AmgLevel<T>>& levels, int dim, int b, const KrylovState* ks,
                        cudaStream_t st);

}  // namespace dxg
