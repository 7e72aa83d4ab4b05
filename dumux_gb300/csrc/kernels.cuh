// kernels.cuh -- kernel argument blocks and launcher declarations.
#pragma once

#include "common.cuh"

namespace dxg {

// Perturbed states per primary variable of a numeric difference method: 1 forward /
// backward, 2 central, 4 five-point stencil (1, -1, 0, 5); none for the residual-only pass
// (2) and the analytic Jacobian (3).
__host__ __device__ constexpr int statesPerPv(int method)
{
    return method == 0 ? 2 : method == 5 ? 4 : (method == 2 || method == 3) ? 0 : 1;
}

// Everything the assembly kernels read or write (device pointers).
struct AssemblyArgs {
    const ProblemConsts* pc;
    int64_t N, nb;
    // per cell
    const double* vol;
    const double* phi;
    const double* extr;
    const int32_t* mat;
    const double* srcterm;      // [b][N]: (0 + source)*(V*extrusion)
    const double* tijPlus;      // [dim][N]: transmissibility of the + face of each axis
    const double* G1;           // [2 sides][b][N]: gravity terms of the vertical faces
    const double* G2;
    // boundary faces
    const int8_t* btype;
    const double* bTij;         // [nb]
    const double* bG1;          // [b][nb]
    const double* bP;           // [b][nb] Dirichlet ghost phase pressures
    const double* bU;           // [b][nb] Dirichlet ghost rho*lambda
    const double* bNeu;         // [b][nb] Neumann flux * area * extrusion
    // volume variables
    double* vvP;                // [states][b][N]
    double* vvU;
    double* vvS;
    double* eps;                // [b][N]
    double* dvv;                // analytic path: [3][N] dkrw/dSn, dkrn/dSn, dpc/dSn
    double* stPrev;             // [b][N]
    // outputs
    double* A;                  // [slots][N][b*b]
    double* r;                  // [N][b]
    double dt;
    // state read by the volume-variable kernels
    const double* u;            // current solution [N][b]
    const double* uprev;        // previous time level [N][b]
    // partial reassembly: per-cell color, 1 red (reassemble the cell's Jacobian column),
    // 0 green (keep it); nullptr: everything red
    const uint8_t* color;
};

void launchVolvars(const AssemblyArgs& a, int b, int method, const double* u, cudaStream_t st);
void launchPrevStorage(const AssemblyArgs& a, int b, const double* uprev, cudaStream_t st);
void launchRow(const AssemblyArgs& a, int b, int dim, int method, bool jac, bool grav, bool transient, bool fullup,
               cudaStream_t st);
// Batched forms: one launch over `count` problems of the same kind (b, dim, method,
// gravity, transient, upwind); problem p reads batch[p] (device array), blockIdx.y = p.
// maxN is the largest cell count of the batch (sizes the grid).
void launchVolvarsBatch(const AssemblyArgs* batch, int count, int64_t maxN, int b, int method, cudaStream_t st);
void launchPrevStorageBatch(const AssemblyArgs* batch, int count, int64_t maxN, int b, cudaStream_t st);
void launchRowBatch(const AssemblyArgs* batch, int count, int64_t maxN, int b, int dim, int method, bool jac, bool grav,
                    bool transient, bool fullup, cudaStream_t st);

// Element-wise correctly rounded pow (crpow.cuh) of host arrays on the current device
// (diagnostic: checks the device's pow against the host's).
int runDevicePow(const double* x, const double* y, double* out, int64_t n);
// Dense FP64 FMA rate of the current device (all SMs, independent chains), TFLOP/s.
int runFp64Rate(double* tflops);

}  // namespace dxg
