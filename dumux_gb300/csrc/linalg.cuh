// linalg.cuh -- structured block-sparse linear algebra on the device.
//
// Matrix layout ("slot BCRS"): the pattern of a cc-TPFA Jacobian on a structured grid
// is the 5-point (2D) / 7-point (3D) stencil, so every block row has the same slots,
// ordered by column: 3D -z,-y,-x,diag,+x,+y,+z (2D -y,-x,diag,+x,+y).  Values are
// stored slot-major, A[slot][row][b*b] with row-major b x b blocks, so a warp reading
// one slot of 32 consecutive rows reads one contiguous segment.  Slots that fall
// outside the grid hold zero blocks and are skipped through the per-cell neighbour
// mask.  Host export converts to the plain BCRS layout of Dune::BCRSMatrix.
#pragma once

#include <vector>

#include "common.cuh"

namespace dxg {

// Device-resident scalars of one BiCGSTAB solve (dune-istl BiCGSTABSolver::apply).
struct KrylovState {
    double rho, rho_new, alpha, omega, beta, h;
    double def, def0, reduction;
    double tr, tt;
    int status;         // 0 running, 1 converged, 2 breakdown, 3 non-finite defect, 4 maxit
    int halfsteps;      // 2*it of dune-istl's half-step counter
    int maxHalf;        // 2*maxit
    int pad;
};

enum { KS_RUNNING = 0, KS_CONVERGED = 1, KS_BREAKDOWN = 2, KS_NAN = 3, KS_MAXIT = 4 };

struct StencilDesc {
    int dim, b;
    int nx, ny, nz;
    int64_t N;
    int64_t off[7];          // column offset of each slot
    int slots;
};

// Level schedule of the natural-order ILU(0) wavefront: cells sorted by ix+iy+iz.
struct LevelSchedule {
    int numLevels = 0;
    std::vector<int32_t> ptr;   // host copy, numLevels+1
};

template <class T>
struct IluFactors {
    T* L;       // [dim lower slots][N][bb]: L_ik = A_ik * D_j^{-1}
    T* Dinv;    // [N][bb]: inverted pivots
};

// Reduction scratch: per-block partial sums and a completion counter per reduction.
struct ReduceScratch {
    double* partials;       // [kMaxReduceBlocks * 3]
    unsigned* counter;      // [8]
};
constexpr int kReduceThreads = 256;
constexpr int kReducePerThread = 4;
constexpr int kMaxReduceBlocks = 1024;

}  // namespace dxg
