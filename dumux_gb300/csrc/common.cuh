// common.cuh -- shared device/host helpers of the GB300 cc-TPFA library.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>

#include "../../include/dumux_gb300.h"

namespace dxg {

// Thrown inside the library only; converted to a status code at the C ABI.
struct Error : std::runtime_error {
    int status;
    Error(int st, const std::string& msg) : std::runtime_error(msg), status(st) {}
};

#define DXG_CUDA(call)                                                                       \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess)                                                               \
            throw ::dxg::Error(e_ == cudaErrorMemoryAllocation ? DXG_ERR_OOM : DXG_ERR_CUDA, \
                               std::string(#call) + ": " + cudaGetErrorString(e_));          \
    } while (0)

// One device allocation that the buffers of a problem upload are carved from: while a
// thread has a block installed (DevBlockScope), DevBuf::alloc takes 256-byte aligned pieces
// of it instead of calling cudaMalloc once per buffer.  The owner keeps the block alive
// for as long as the buffers carved from it.
struct DevBlock {
    unsigned char* base = nullptr;
    size_t cap = 0, used = 0;
};
inline DevBlock*& currentDevBlock()
{
    thread_local DevBlock* b = nullptr;
    return b;
}
struct DevBlockScope {
    DevBlock* prev;
    explicit DevBlockScope(DevBlock* b) : prev(currentDevBlock()) { currentDevBlock() = b; }
    ~DevBlockScope() { currentDevBlock() = prev; }
};

// Owning device buffer (or a piece of the installed DevBlock, which it does not free).
template <class T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    bool owned = true;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void release()
    {
        if (p && owned) cudaFree(p);
        p = nullptr;
        n = 0;
        owned = true;
    }
    void alloc(size_t count)
    {
        if (count == n && p) return;
        release();
        if (count == 0) return;
        const size_t bytes = (count * sizeof(T) + 255) & ~(size_t)255;
        DevBlock* blk = currentDevBlock();
        if (blk && blk->used + bytes <= blk->cap) {
            p = reinterpret_cast<T*>(blk->base + blk->used);
            blk->used += bytes;
            owned = false;
            n = count;
            return;
        }
        DXG_CUDA(cudaMalloc(&p, count * sizeof(T)));
        n = count;
    }
    T* get() const { return p; }
    size_t bytes() const { return n * sizeof(T); }
};

constexpr int kMaxMaterials = 16;

// Derived constants of one regularised Brooks-Corey parameter set
// (BrooksCoreyRegularization::initPcParameters_, brookscorey.hh:477-486).
// Two-point cubic spline of the Van Genuchten regularisation (Spline<Scalar, 2>,
// dumux/common/spline.hh:310-345): end points, values and the moments of the clamped
// spline (dumux/common/splinecommon_.hh:419-440).
struct Spline2 {
    double x0, x1, y0, y1, M0, M1;
};

struct MaterialLaw {
    int kind;                      // 0 regularised Brooks-Corey, 1 regularised Van Genuchten
    double pe, lambda, swr, snr, pcLowSwe;
    double denom;                  // 1.0 - swr - snr
    double expPc;                  // -1.0/lambda
    double expKrw;                 // 2.0/lambda + 3.0
    double expKrn;                 // 2.0/lambda + 1.0
    double pcLowSwePcValue, pcDerivativeLowSw, pcDerivativeHighSwEnd, entryPressure;
    // derivative constants (brookscorey.hh:166-174, 241-249, 295-305; efftoabsdefaultpolicy.hh:135)
    double dsweDsw;                // 1.0/(1.0 - swr - snr)
    double dpcCoef, dpcExp;        // -pe/lambda, -1.0/lambda - 1.0
    double dkrwCoef, dkrwExp;      // 2.0/lambda + 3.0, 2.0/lambda + 2.0
    double lambdaInv, dkrnExp;     // 1.0/lambda, 2*lambdaInv
    // Van Genuchten (vangenuchten.hh:30-300): alpha, n, m = 1 - 1/n, l and the exponents
    // the reference forms at run time; regularisation thresholds and splines
    double vgAlpha, vgN, vgM, vgL;
    double vgNegInvM, vgInvN, vgInvM;       // -1.0/m, 1.0/n, 1.0/m
    double pcHighSwe, krnLowSwe, krwHighSwe;
    Spline2 pcSpline, krwSpline, krnSpline;
};

// Problem constants visible to the kernels.
struct ProblemConsts {
    int dim, b;
    int nx, ny, nz;
    int64_t N;
    int64_t sideOffset[7];
    int gravity;                   // Problem.EnableGravity
    int gravAxisMask;              // bit a set: faces normal to axis a carry gravity terms
    double density[2], viscosity[2];
    double mobility1p;             // 1.0/viscosity (1p)
    double upwindWeight;
    int upwindFull;                // upwind weight != 1
    int method;                    // numeric difference method (3: analytic derivatives)
    double baseEps;
    double magnitude[2];
    int numMaterials;
    int hasSource;
    MaterialLaw law[kMaxMaterials];
};

__host__ __device__ inline int slotOfFace(int dim, int f)
{
    const int a = f >> 1;
    return (f & 1) ? dim + 1 + a : dim - 1 - a;
}

}  // namespace dxg
