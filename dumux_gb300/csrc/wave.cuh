// wave.cuh -- cluster wavefront ILU(0) kernels (see wave.cu).
#pragma once

#include <vector>

#include "common.cuh"
#include "linalg.cuh"

namespace dxg {

template <class T>
struct WaveArgs {
    int dim, nx, ny, nz;
    int64_t N;
    int ctas, linesPerCta, haloLines;
    const T* A;               // slot matrix (lower slots for the factor, upper for the backward sweep)
    T* L;                     // lower factor
    T* Dinv;                  // inverted pivots
    const T* rhs;             // forward sweep input
    T* v;                     // forward output / backward in-out
    int* err;                 // DXG_ERR_TIMEOUT on an expired wait
    int* singular;            // set on a singular pivot
    const KrylovState* ks;    // sweeps are skipped once the solve has stopped
    unsigned long long waitNs;   // limit of every wait (0: the default 0.5 s)
};

// Sweeps of lanewave.cu (3D, 2x2 blocks): two lanes per x-line, one plane of up to 64 lines
// per CTA, clusters along z.
template <class T>
struct LaneWaveArgs {
    int nx, ny, nz;
    int64_t N;
    int nyb;                  // CTAs per plane (64 lines each)
    int ctas;                 // working CTAs (nz * nyb); the grid is padded to whole clusters
    int clusterSize;
    const T* Lf;              // lower factor (forward sweep)
    const T* A;               // matrix, upper slots (backward sweep)
    const T* Dinv;            // inverted pivots
    const T* rhs;             // forward input
    T* v;                     // forward output, backward in/out
    int* err;                 // DXG_ERR_TIMEOUT on an expired wait
    const KrylovState* ks;    // sweeps are skipped once the solve has stopped
    T* handoff;               // [ctas][nx][64][2] hand-offs between clusters, all bits set between launches
    unsigned long long waitNs;
};
struct LanePlan {
    bool ok = false;
    int nyb = 0, ctas = 0, clusterSize = 0, grid = 0, pfFwd = 0, pfBwd = 0;
    // the shared-memory-ring form (laneRingKernel): fits beside the register form (same
    // launch shape), its prefetch depths, and which form the sweeps run (0 registers, 1 ring)
    bool ringOk = false;
    int pfRingFwd = 0, pfRingBwd = 0;
    int ring = 0;
};
// Plan of the lane sweeps for a dim-D grid of b x b blocks (ok only for 3D, b == 2, grids whose
// sweeps fit: every cluster resident at once, the plane history in shared memory).
template <class T>
LanePlan makeLanePlan(int dim, int nx, int ny, int nz, int b);
template <class T>
void launchLaneWaveApply(const LanePlan& p, const LaneWaveArgs<T>& fwd, const LaneWaveArgs<T>& bwd, cudaStream_t st);
// One-CTA line sweeps of 2D cc-TPFA systems (linesweep.cu): one thread per grid line, both block
// rows, for grids of up to 512 lines; uses nx, ny, N, Lf, A, Dinv, rhs, v and ks of the args.
bool tpfaLine2dFits(int dim, int nx, int ny, int b);
template <class T>
void launchTpfaLine2d(const LaneWaveArgs<T>& fwd, const LaneWaveArgs<T>& bwd, int b, cudaStream_t st);

struct WavePlan {
    int ctas = 0, linesPerCta = 0, haloLines = 0, threads = 0, lpt = 0;
    size_t smemSolve = 0, smemFactor = 0;
    bool ok = false;
};

// Slab split of one problem under at most maxCtas CTAs.
struct WaveGeom {
    int ctas = 0, linesPerCta = 0, haloLines = 0;
};

// Launch shape shared by all problems of a batched sweep: clusters of `ctas` CTAs
// (one cluster per problem), `threads` per CTA, prefetch depth `pf`.
struct WaveBatchPlan {
    int ctas = 0, threads = 0, pf = 0;
    size_t smemFwd = 0, smemBwd = 0, smemFactor = 0;
};

WavePlan makeWavePlan(int dim, int nx, int ny, int nz, int b, bool fp64);
// Every plan that fits, one per cluster size (16, 8, 4, 2, 1 CTAs); the first is
// makeWavePlan's.  The factors and sweeps do not depend on the plan (same arithmetic
// per cell), so a context may switch between them at any time.
std::vector<WavePlan> wavePlanCandidates(int dim, int nx, int ny, int nz, int b, bool fp64);
WaveGeom waveGeom(int dim, int nx, int ny, int nz, int maxCtas);
int completeWaveBatchPlan(WaveBatchPlan& p, const std::vector<WaveGeom>& geoms, int dim, int b, bool fp64);
template <class T>
void launchWaveFactorBatch(const WaveBatchPlan& p, const WaveArgs<T>* batch, int count, int dim, int b,
                           cudaStream_t st);
template <class T>
void launchWaveApplyBatch(const WaveBatchPlan& p, const WaveArgs<T>* fwd, const WaveArgs<T>* bwd, int count, int dim,
                          int b, cudaStream_t st);
// Runs the bounded-wait self-test kernel (kind 0: mbarrier, 1: global flag) on the
// current device; *kernelStatus receives the kernel's verdict (DXG_ERR_TIMEOUT expected).
int runBoundedWaitSelfTest(int kind, long long limitNs, int* kernelStatus, double* waitedMs);
template <class T>
void launchWaveFactor(const WavePlan& plan, const WaveArgs<T>& a, int b, cudaStream_t st);
template <class T>
void launchWaveApply(const WavePlan& plan, const WaveArgs<T>& fwd, const WaveArgs<T>& bwd, int b, cudaStream_t st);

}  // namespace dxg
