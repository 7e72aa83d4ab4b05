// mpfa.cuh -- MPFA-O for the 1p model: layout of the per-cell flux rows, host tabulation
// of the interaction volumes, device assembly (mpfa.cu).
#pragma once
#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/dumux_gb300.h"

namespace dxg {

// Per dim: stencil slots S = 3^dim (slot s = (ox+1) + 3(oy+1) + 9(oz+1)), scvfs per cell F
// (faces -x,+x,-y,+y,-z,+z, each with its 2^(dim-1) corners in reference-element order), IV
// cells per scvf K = 2^dim (cell k = vertex - 1 + bits of k), the stencil slot of IV cell k
// of scvf f, and per scvf the mask of the slots its IV covers.
struct MpfaLayout {
    int dim = 2, S = 9, center = 4, F = 8, K = 4;
    int8_t slotOf[24][8] = {};
    uint32_t scvfSlots[24] = {};
};
MpfaLayout mpfaLayout(int dim);
// The ILU(0) update triples (s, t, u) of the 3^dim stencil (see StencilArgs).
void mpfaTriples(int dim, int& n, int8_t (*tri)[3]);

// Flux rows of every (cell, scvf): coef[(f*K + k)*N + i] the transmissibility of IV cell k
// signed for cell i, cst[(f*b + e)*N + i] the IV's Dirichlet and gravity part of phase e (or,
// kind 1, the Neumann flux of equation e times area and extrusion), kind[f*N + i] 0 (IV flux)
// / 1 (Neumann).
// dirP: 2p, the Dirichlet ghosts' phase pressures [phase][boundary face] (unused for 1p).
void mpfaTabulate(const dxg_problem_desc* d, const MpfaLayout& L, const int64_t* sideOffset, const double* dirP,
                  std::vector<double>& coef, std::vector<double>& cst, std::vector<int8_t>& kind);

struct MpfaArgs {
    int64_t N = 0;
    int S = 9, F = 8, K = 4;
    int64_t off[27] = {};
    int8_t slotOf[24][8] = {};
    uint32_t scvfSlots[24] = {};
    const double* coef = nullptr;
    const double* cst = nullptr;
    const int8_t* kind = nullptr;
    const uint32_t* mask = nullptr;
    const double* srcterm = nullptr;   // source * volume * extrusion
    const double* u = nullptr;
    double mob = 0.0;                  // density * (1 / viscosity): the flux's upwind term
    double up = 0.0;                   // density / viscosity: the analytic derivatives' factor
    double baseEps = 1e-10, magnitude = -1.0;
    bool transient = false;
    double* A = nullptr;               // [S][N][b*b]
    double* r = nullptr;               // [N][b]
    // 2p: the volume variables of every cell at its own and perturbed states (the TPFA
    // volume-variable kernel's [state][phase][N] arrays), numeric epsilons, previous storage,
    // cell volumes, the Dirichlet ghosts' upwind terms [phase][boundary face], upwind weight
    int b = 1;
    int nx = 1, ny = 1, nz = 1;
    int64_t nb = 0;
    int64_t sideOffset[7] = {};
    const double* vvP = nullptr;
    const double* vvU = nullptr;
    const double* vvS = nullptr;
    const double* eps = nullptr;
    const double* stPrev = nullptr;
    const double* vol = nullptr;
    const double* bU = nullptr;
    double w = 1.0, dt = 0.0;
};
// Residual (and with jac the Jacobian rows: numeric differences, method 1 / -1 / 0 / 5, or
// the analytic derivatives, method 3).
void launchMpfaAssemble(const MpfaArgs& a, int method, bool jac, cudaStream_t st);

}  // namespace dxg
