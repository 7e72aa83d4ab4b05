// context.h -- the opaque dxg_ctx behind the C ABI.
#pragma once

#include <string>
#include <vector>

#include "amg.cuh"
#include "common.cuh"
#include "kernels.cuh"
#include "linalg_kernels.cuh"
#include "mpfa.cuh"
#include "wave.cuh"

struct dxg_ctx {
    // the device memory the first upload's buffers are carved from (declared first, so
    // it is released after every buffer)
    dxg::DevBuf<unsigned char> uploadBlock;
    dxg::DevBlock uploadCarve;
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    int64_t launches = 0;
    int precision = DXG_PRECISION_FP64;
    bool uploaded = false;

    // problem
    dxg::ProblemConsts pcHost{};
    dxg::DevBuf<dxg::ProblemConsts> pcDev;
    int dim = 0, b = 0, slots = 0, bb = 0, method = 1;
    int64_t N = 0, nb = 0, M = 0, nnzb = 0;
    bool gravity = false, fullUpwind = false;
    int64_t off[7] = {0, 0, 0, 0, 0, 0, 0};
    dxg::LevelSchedule levels;
    std::vector<uint8_t> nbmaskHost;

    dxg::DevBuf<double> vol, phi, extr, srcterm, tijPlus, G1, G2;
    dxg::DevBuf<int32_t> mat, perm;
    dxg::DevBuf<int8_t> btype;
    dxg::DevBuf<double> bTij, bG1, bP, bU, bNeu;
    dxg::DevBuf<uint8_t> nbmask;

    // MPFA-O (1p): per-(cell, scvf) flux rows, the 3^dim stencil of the Jacobian and its
    // ILU(0) (L holds the LU factor [S][N], Dinv the inverted pivots)
    bool mpfa = false;
    dxg::MpfaLayout mpLayout{};
    int64_t mpOff[27] = {};
    dxg::DevBuf<double> mpCoef, mpCst;
    dxg::DevBuf<int8_t> mpKind;
    dxg::DevBuf<uint32_t> mpMask;
    std::vector<uint32_t> mpMaskHost;
    double mpMob = 0.0, mpUp = 0.0;
    int mpNTri = 0;
    int8_t mpTri[104][3] = {};

    // state
    dxg::DevBuf<double> u, uprev, uLast, stPrev;
    dxg::DevBuf<double> vvP, vvU, vvS, eps;
    dxg::DevBuf<double> dvv;          // analytic derivatives: [dkrw/dSn, dkrn/dSn, dpc/dSn][N]
    dxg::DevBuf<double> A, r;
    double dt = 0.0;
    bool havePrev = false, stPrevValid = false, haveJac = false, haveRes = false, haveFactor = false;

    // linear solver (FP64)
    dxg::DevBuf<double> L, Dinv;
    dxg::DevBuf<double> kx, kr, krt, kp, kv, kt, ky;
    // mixed precision: FP32 Jacobian copy, ILU(0) factors and preconditioner operands
    dxg::DevBuf<float> Af, Lf, Dinvf, fr, fp, fy;
    dxg::DevBuf<double> delta;

    dxg::DevBuf<dxg::KrylovState> ks;
    dxg::DevBuf<double> partials;
    dxg::DevBuf<unsigned> counters;
    dxg::DevBuf<double> scal;         // [0] shift, [1] norm
    dxg::DevBuf<int> singular;        // [0] singular pivot, [1] wavefront wait timeout
    dxg::KrylovState* ksHost = nullptr;   // pinned
    double* scalHost = nullptr;           // pinned

    int lastNewtonSteps = 0;

    // captured chunk of BiCGSTAB iterations per preconditioner precision ([0] FP64, [1] FP32)
    struct ChunkGraph {
        cudaGraphExec_t exec = nullptr;
        int key[4] = {-1, -1, -1, -1};
        int64_t launches = 0;
    };
    ChunkGraph chunkGraph[2];
    void dropGraphs()
    {
        for (auto& g : chunkGraph) {
            if (g.exec) cudaGraphExecDestroy(g.exec);
            g.exec = nullptr;
        }
    }

    // partial reassembly (active during a Newton solve that asks for it)
    bool partialActive = false;
    dxg::DevBuf<double> partialDist;
    dxg::DevBuf<uint8_t> partialColor;

    // preconditioner of the BiCGSTAB solve: ILU(0) (default) or aggregation AMG
    int linearSolver = DXG_LINEAR_SOLVER_ILU_BICGSTAB;
    dxg::DevBuf<unsigned char> amgMem;   // fine-level scratch, then every coarse level (one allocation)

    // ILU(0) kernels: cluster wavefront (default) or level-scheduled launches
    int iluKernel = DXG_ILU_AUTO;
    dxg::WavePlan wavePlan;
    bool waveTuned = false;           // launch shape chosen by timing (first factorisation)
    double waveTuneMs[5] = {0, 0, 0, 0, 0};   // ms per apply of each candidate tried
    int waveTuneCtas[5] = {0, 0, 0, 0, 0};
    int waveTuneCount = 0;
    // lane sweeps (lanewave.cu): chosen by the timing at the first factorisation when faster
    // (DXG_ILU_AUTO) or forced (DXG_ILU_LANES); their inter-cluster hand-off buffer
    dxg::LanePlan lanePlan;
    bool laneWave = false;
    double laneTuneMs = 0.0;       // the lane sweeps' time per apply at the tuning (the form run)
    double laneFormMs[2] = {0.0, 0.0};   // per form: 0 registers, 1 shared-memory ring
    int laneRingMode = 0;          // 0 timed, 1 register form, 2 shared-memory-ring form
    bool line2dOk = false;         // the one-CTA line sweeps of 2D TPFA systems fit
    bool line2d = false;           // ... and the timing at the first factorisation chose them
    double line2dMs = 0.0;
    dxg::DevBuf<unsigned char> laneHandoff;
    size_t laneHandoffBytes = 0;
    // limit of every bounded wait of the sweeps (0: the kernels' default, 0.5 s)
    unsigned long long waitNs = 0;

    // optional event timing per kernel class (pairs resolved lazily)
    struct TimedLaunch {
        cudaEvent_t start, stop;
        int kclass;
        double bytes;
    };
    bool timing = false;
    std::vector<TimedLaunch> pending;
    std::vector<cudaEvent_t> eventPool;
    int64_t kcLaunches[DXG_KC_COUNT] = {};
    double kcMs[DXG_KC_COUNT] = {};
    double kcBytes[DXG_KC_COUNT] = {};
    double bytesSweep = 0, bytesAssembly = 0, bytesSpmv = 0;   // algorithmic bytes per launch (FP64 sizes)
    double bytesFactor = 0;   // factorisation: matrix read, factor and pivots written once

    dxg::AssemblyArgs asmArgs() const;
    dxg::ReduceScratch scratch() const { return {partials.get(), counters.get()}; }
};

namespace dxg {
// The aggregation AMG levels of a context in value type T (level 0: the Jacobian A with
// the inverted pivots Dinv, the preconditioner input `in` and output `out`); the coarse
// levels live in the context's AMG allocation, made on first use.
template <class T>
std::vector<AmgLevel<T>> amgLevelsOf(dxg_ctx* c, const T* A, T* Dinv, const T* in, T* out);
}  // namespace dxg
