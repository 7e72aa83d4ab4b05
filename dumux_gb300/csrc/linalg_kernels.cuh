// linalg_kernels.cuh -- argument blocks and launchers of the linear-algebra kernels.
#pragma once

#include <vector>

#include "linalg.cuh"

namespace dxg {

// y = A x with matrix values MT, input XT and output / dot operands VT.  With MT = XT =
// float (the mixed form's FP32 Jacobian times the FP32 preconditioner output) the block
// products and row sums are FP32 and the result is widened to VT.
template <class MT, class VT, class XT = VT>
struct SpmvArgs {
    const MT* A;
    const uint8_t* nbmask;
    const XT* x;
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

// Red-black ordered block ILU(0): cells coloured by the parity of x+y+z (red even).
// With no red-red or black-black couplings on the TPFA stencil, ILU(0) in this order
// keeps D_r = A_rr and D_b = A_bb - sum_r A_br D_r^-1 A_rb, and a sweep pair is two
// fully parallel passes: black v_b = D_b^-1 (d_b - sum_r A_br D_r^-1 d_r), then red
// v_r = D_r^-1 (d_r - sum_b A_rb v_b).
template <class T>
struct RbArgs {
    const T* A;
    T* Dinv;
    const uint8_t* nbmask;
    int64_t N;
    int64_t off[7];
    int nx, ny, nz;
    int* singular;
    const KrylovState* ks;    // apply passes skip when the solve has stopped
    const T* d;               // apply: input
    T* v;                     // apply: output
};
// cells of one colour slot range: rows * ceil(nx / 2) (the red-black kernels' index space)
inline int64_t rbSlots(int nx, int ny, int nz) { return (int64_t)ny * nz * ((nx + 1) / 2); }

template <class VT>
struct BicgArgs {
    VT *x, *r, *rt, *p, *v, *t, *y;
    int64_t M;                // N*b scalars
    KrylovState* ks;
    ReduceScratch scratch;
    const double* rhs;        // right-hand side read by the init kernel
    double reduction;         // init kernel: written to ks when maxHalf > 0
    int maxHalf;
    // FP32 copies of p (written by the p update) and r (written by the first-half
    // update): the inputs of an FP32 preconditioner inside an FP64 iteration
    float* pLow;
    float* rLow;
    // FP32 preconditioner output read by the x updates in place of y (x += s*yLow)
    const float* yLow;
};

struct ToDoubleArgs {
    const float* src;
    double* dst;
    int64_t n;
};

// u = uLast - lambda*delta and the maximum relative shift
struct NewtonUpdArgs {
    const double* uLast;
    const double* delta;
    double* u;
    double lambda;
    int64_t M;
    ReduceScratch scratch;
    double* shiftOut;
};
struct NormArgs {
    const double* x;
    int64_t M;
    ReduceScratch scratch;
    double* out;
};
// elementwise helpers of the mixed-precision solve
struct ToFloatArgs {
    const double* src;
    float* dst;
    int64_t n;
};
struct AccumArgs {
    double* y;                // y += x
    const float* x;
    int64_t n;
};
struct DefectArgs {
    const double* A;
    const uint8_t* nbmask;
    const double* x;          // accumulated update
    const double* rhs;
    double* y;                // rhs - A x
    int64_t N;
    int64_t off[7];
};

int reduceBlocks(int64_t M);

// Scalar rows over the 3^dim neighbourhood of a cell (MPFA-O): A[slot][row] with slot
// s = (ox+1) + 3(oy+1) + 9(oz+1), valid for row i when bit s of mask[i] is set; LU / Dinv the
// ILU(0) factors (multipliers in the lower slots, U in the upper ones, inverted pivots).
// The ILU(0) update of row i by its lower entry s touches entry t of row i with entry u of
// row i + off[s]: tri[k] = {s, t, u}, s then t ascending.
struct StencilArgs {
    int b = 1;                             // block size: 1 (1p) or 2 (2p, blocks [slot][row][4])
    int nx = 1, ny = 1, nz = 1;
    int64_t N = 0;
    int S = 0, center = 0;
    int64_t off[27] = {};
    const uint32_t* mask = nullptr;
    const double* A = nullptr;
    double* LU = nullptr;
    double* Dinv = nullptr;
    int* singular = nullptr;
    KrylovState* ks = nullptr;
    ReduceScratch scratch{};
    int nTri = 0;
    int8_t tri[104][3] = {};
    int* err = nullptr;                    // DXG_ERR_TIMEOUT of a sweep that gave up waiting
    unsigned long long waitNs = 0;         // wait limit of the cluster sweeps (0: 0.5 s)
};
void launchStencilSpmv(const StencilArgs& a, const double* x, double* y, const double* w, int mode, cudaStream_t st);
void launchStencilFactor(const StencilArgs& a, cudaStream_t st);
// the preconditioner apply: the level-by-level kernel (any stencil), the one-CTA line sweeps
// of 2D stencils with ny <= 1024 (stencilWave2dKernel)
void launchStencilApplyLevels(const StencilArgs& a, const double* d, double* v, cudaStream_t st);
void launchStencilWave2d(const StencilArgs& a, const double* d, double* v, cudaStream_t st);
bool stencilWave2dFits(const StencilArgs& a);
// 2D 9-point sweeps over a cluster (stencilwave.cu): lines spread over up to 16 CTAs of four
// warps, point-to-point hand-offs through shared-memory histories
bool stencilLane2dFits(const StencilArgs& a);
void launchStencilLane2d(const StencilArgs& a, const double* d, double* v, cudaStream_t st);
// 3D 27-point sweeps over a cluster (stencillane.cu): one z-plane per CTA (nz <= 16), one lane
// per grid line and block row
bool stencilLane3dFits(const StencilArgs& a);
void launchStencilLane3d(const StencilArgs& a, const double* d, double* v, cudaStream_t st);
// ILU(0) factorisation of a 3D (27-point) stencil matrix over a cluster of 16 CTAs, one warp per
// row of a level (stencillane.cu)
void launchStencilFactorCluster(const StencilArgs& a, cudaStream_t st);

template <class MT, class VT, class XT = VT>
void launchSpmv(const SpmvArgs<MT, VT, XT>& a, int b, int dim, int mode, cudaStream_t st);
template <class MT>
int64_t launchIluFactor(const IluArgs<MT, MT>& a, const LevelSchedule& ls, int b, int dim, cudaStream_t st);
template <class MT, class VT>
int64_t launchIluApply(const IluArgs<MT, VT>& a, const LevelSchedule& ls, int b, int dim, const VT* d, VT* v,
                       cudaStream_t st);
template <class VT>
void launchBicgInit(const BicgArgs<VT>& a, const double* rhs, cudaStream_t st);
template <class VT>
void launchBicgUpdateP(const BicgArgs<VT>& a, cudaStream_t st);
template <class VT>
void launchBicgAxpyNorm(const BicgArgs<VT>& a, int stage, cudaStream_t st);
template <class VT>
void launchCopyToDouble(const VT* x, double* y, int64_t M, cudaStream_t st);
void launchNewtonUpdate(const double* uLast, const double* delta, double* u, double lambda, int64_t M,
                        const ReduceScratch& sc, double* shiftOut, cudaStream_t st);
void launchNorm2(const double* x, int64_t M, const ReduceScratch& sc, double* out, cudaStream_t st);
void launchPartialColors(const double* uLast, const double* u, double* dist, uint8_t* color, int64_t N, int b,
                         double threshold, cudaStream_t st);
template <class T>
int64_t launchRbFactor(const RbArgs<T>& a, int b, int dim, cudaStream_t st);
template <class T>
int64_t launchRbApply(const RbArgs<T>& a, int b, int dim, const T* d, T* v, cudaStream_t st);
void launchToFloat(const ToFloatArgs& a, cudaStream_t st);
void launchToDouble(const ToDoubleArgs& a, cudaStream_t st);
void launchAccum(const AccumArgs& a, cudaStream_t st);
void launchDefect(const DefectArgs& a, int b, int dim, cudaStream_t st);

// Batched forms: one launch over several problems, problem p reading batch[p] (device
// array).  The vector kernels and the SpMV run through a block map: block k of the
// grid works on problem map[k].x as that problem's block map[k].y, each problem with
// exactly the blocks of its single launch (vector kernels: reduceBlocks(M); SpMV:
// cellBlocks(N)), so batched and single results are identical and no block idles.
struct BlockMap {
    const uint2* map = nullptr;   // device array of `blocks` entries
    unsigned blocks = 0;
};
int cellBlocks(int64_t N);
// Host side of a block map: the entries for problems of the given lengths, blocks
// per problem from reduceBlocks (cells == false) or cellBlocks (cells == true).
void buildBlockMap(const std::vector<int64_t>& lengths, bool cells, std::vector<uint2>& out);

template <class MT, class VT, class XT = VT>
void launchSpmvBatch(const SpmvArgs<MT, VT, XT>* batch, const BlockMap& cellMap, int b, int dim, int mode,
                     cudaStream_t st);
template <class VT>
void launchBicgInitBatch(const BicgArgs<VT>* batch, const BlockMap& map, cudaStream_t st);
template <class VT>
void launchBicgUpdatePBatch(const BicgArgs<VT>* batch, const BlockMap& map, cudaStream_t st);
template <class VT>
void launchBicgAxpyNormBatch(const BicgArgs<VT>* batch, const BlockMap& map, int stage, cudaStream_t st);
void launchNewtonUpdateBatch(const NewtonUpdArgs* batch, const BlockMap& map, cudaStream_t st);
// red-black ILU(0) over several problems: block map over rbSlots of each problem (cells == true)
template <class T>
void launchRbFactorBatch(const RbArgs<T>* batch, const BlockMap& map, int b, int dim, cudaStream_t st);
template <class T>
void launchRbApplyBatch(const RbArgs<T>* batch, const BlockMap& map, int b, int dim, cudaStream_t st);
void launchNorm2Batch(const NormArgs* batch, const BlockMap& map, cudaStream_t st);
void launchToDoubleBatch(const ToDoubleArgs* batch, const BlockMap& map, cudaStream_t st);
// grid-stride elementwise kernels, blockIdx.y = problem (maxN: the longest)
void launchToFloatBatch(const ToFloatArgs* batch, int count, int64_t maxN, cudaStream_t st);
void launchAccumBatch(const AccumArgs* batch, int count, int64_t maxN, cudaStream_t st);
void launchDefectBatch(const DefectArgs* batch, int count, int64_t maxN, int b, int dim, cudaStream_t st);
}  // namespace dxg
