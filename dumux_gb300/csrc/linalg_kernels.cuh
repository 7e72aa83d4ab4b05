// linalg_kernels.cuh -- argument blocks and launchers of the linear-algebra kernels.
#pragma once

#include "linalg.cuh"

namespace dxg {

template <class MT, class VT>
struct SpmvArgs {
    const MT* A;
    const uint8_t* nbmask;
    const VT* x;
    VT* y;
    const VT* w;              // second operand of the fused dot(s)
    int64_t N;
    int64_t off[7];
    KrylovState* ks;
    ReduceScratch scratch;
};

template <class MT, class VT>
struct IluArgs {
    const MT* A;              // assembled matrix (upper slots are the U factor)
    MT* L;
    MT* Dinv;
    const uint8_t* nbmask;
    const int32_t* perm;      // cells sorted by level
    int64_t N;
    int64_t off[7];
    int* singular;            // set when a pivot block is singular
    const KrylovState* ks;    // apply kernels skip when the solve has stopped
};

template <class VT>
struct BicgArgs {
    VT *x, *r, *rt, *p, *v, *t, *y;
    int64_t M;                // N*b scalars
    KrylovState* ks;
    ReduceScratch scratch;
};

int reduceBlocks(int64_t M);

template <class MT, class VT>
void launchSpmv(const SpmvArgs<MT, VT>& a, int b, int dim, int mode, cudaStream_t st);
template <class MT>
int64_t launchIluFactor(const IluArgs<MT, MT>& a, const LevelSchedule& ls, int b, int dim, cudaStream_t st);
template <class MT, class VT>
int64_t launchIluApply(const IluArgs<MT, VT>& a, const LevelSchedule& ls, int b, int dim, const VT* d, VT* v,
                       cudaStream_t st);
template <class VT>
void launchBicgInit(const BicgArgs<VT>& a, const double* rhs, cudaStream_t st);
template <class VT>
void launchBicgRho(const BicgArgs<VT>& a, cudaStream_t st);
template <class VT>
void launchBicgUpdateP(const BicgArgs<VT>& a, cudaStream_t st);
template <class VT>
void launchBicgAxpyNorm(const BicgArgs<VT>& a, int stage, cudaStream_t st);
template <class VT>
void launchCopyToDouble(const VT* x, double* y, int64_t M, cudaStream_t st);
void launchNewtonUpdate(const double* uLast, const double* delta, double* u, double lambda, int64_t M,
                        const ReduceScratch& sc, double* shiftOut, cudaStream_t st);
void launchNorm2(const double* x, int64_t M, const ReduceScratch& sc, double* out, cudaStream_t st);

}  // namespace dxg
