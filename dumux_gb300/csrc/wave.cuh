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
};

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
