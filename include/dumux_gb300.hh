// dumux_gb300.hh -- C++ adapter over the C ABI of dumux_gb300.h (header only, C++17).
//
// What a DuMux application keeps: its Problem and SpatialParams classes, called through
// the reference's *AtPos interface, and the call pattern of the Assembler / LinearSolver /
// NewtonSolver concepts.  What changes: the classes below replace FVAssembler,
// ILUBiCGSTABIstlSolver and NewtonSolver; they tabulate the problem once
// (dxg_problem_upload) and run assembly, the linear solve and the Newton loop on the GPU.
//
//   reference                                              here
//   Dumux::FVAssembler          (assembly/fvassembler.hh)   GpuFVAssembler
//   Dumux::ILUBiCGSTABIstlSolver (linear/istlsolvers.hh)    GpuILUBiCGSTABSolver
//   Dumux::NewtonSolver         (nonlinear/newtonsolver.hh) GpuNewtonSolver
//
// Problem interface used (dumux/common/fvproblem.hh:99-524; the reference's 2p test
// problem, test/porousmediumflow/2p/incompressible/problem.hh:59-139, has this shape):
//   BoundaryTypes boundaryTypesAtPos(const GlobalPosition&)   -- all Dirichlet or all Neumann
//   PrimaryVariables dirichletAtPos(const GlobalPosition&)
//   NumEqVector neumannAtPos(const GlobalPosition&)           -- mass flux, positive = outflow
//   NumEqVector sourceAtPos(const GlobalPosition&)
//   PrimaryVariables initialAtPos(const GlobalPosition&)
// SpatialParams interface used (dumux/porousmediumflow/fvspatialparams*.hh):
//   double permeabilityAtPos(const GlobalPosition&)           -- isotropic
//   double porosityAtPos(const GlobalPosition&)
//   double extrusionFactorAtPos(const GlobalPosition&)
//   BrooksCoreyParams fluidMatrixInteractionAtPos(const GlobalPosition&)   (2p only)
// Values are indexed with operator[] (FieldVector-like); GlobalPosition here is a
// std::array<double, 3> (DUNE's FieldVector is not required).  Solution vectors are flat
// std::vector<double> in the BlockVector<FieldVector<double, numEq>> order (cell major).
#ifndef DUMUX_GB300_HH
#define DUMUX_GB300_HH

#include <array>
#include <cmath>
#include <stdexcept>
#include <string>
#include <vector>

#include "dumux_gb300.h"

namespace dumux_gb300 {

using GlobalPosition = std::array<double, 3>;

// Dumux::NumericalProblem: the recoverable failure of a linear or Newton solve.
struct NumericalProblem : std::runtime_error {
    int status;
    NumericalProblem(int s, const std::string& m) : std::runtime_error(m), status(s) {}
};
struct Error : std::runtime_error {
    int status;
    Error(int s, const std::string& m) : std::runtime_error(m), status(s) {}
};

inline bool recoverable(int st)
{
    return st == DXG_ERR_LINEAR_BREAKDOWN || st == DXG_ERR_LINEAR_NOT_CONVERGED || st == DXG_ERR_NAN ||
           st == DXG_ERR_NEWTON_NOT_CONVERGED;
}

// Dumux::BoundaryTypes restricted to what the device path supports: every equation of a
// boundary face Dirichlet, or every equation Neumann (mixed faces are rejected, as the
// reference's cc-TPFA local residual does, cclocalresidual.hh:49-105).
struct BoundaryTypes {
    bool dirichlet = false;
    void setAllDirichlet() { dirichlet = true; }
    void setAllNeumann() { dirichlet = false; }
    bool hasDirichlet() const { return dirichlet; }
    bool hasNeumann() const { return !dirichlet; }
};

// Parameters of Dumux's regularised Brooks-Corey law (BrooksCoreyDefault):
// pcEntry, lambda, Swr, Snr and the pc regularisation threshold pcLowSwe.
struct BrooksCoreyParams {
    double pcEntry = 0.0, lambda = 2.0, swr = 0.0, snr = 0.0, pcLowSwe = 0.01;
};

// A structured tensor-product grid (YaspGrid with tensor-product coordinates).
struct StructuredGrid {
    int dim = 3;
    std::array<std::vector<double>, 3> coords;   // vertex coordinates per axis

    static StructuredGrid equidistant(const std::array<double, 3>& lower, const std::array<double, 3>& upper,
                                      const std::array<int, 3>& cells, int dim)
    {
        StructuredGrid g;
        g.dim = dim;
        for (int a = 0; a < dim; ++a) {
            g.coords[a].resize(cells[a] + 1);
            const double h = (upper[a] - lower[a]) / cells[a];
            for (int i = 0; i <= cells[a]; ++i) g.coords[a][i] = lower[a] + i * h;
        }
        return g;
    }
    int cells(int a) const { return a < dim ? (int)coords[a].size() - 1 : 1; }
    long long numCells() const { return (long long)cells(0) * cells(1) * cells(2); }
    double center(int a, int i) const { return 0.5 * (coords[a][i] + coords[a][i + 1]); }
};

// Fluid constants of the immiscible phases (constant liquids, fluidsystems/2pimmiscible.hh).
struct FluidProperties {
    std::array<double, 2> density{1000.0, 1000.0};
    std::array<double, 2> viscosity{1e-3, 1e-3};
};

// Numeric differentiation and upwinding parameters (Assembly.NumericDifference*,
// Flux.UpwindWeight) and gravity (Problem.EnableGravity).
struct AssemblyParams {
    double baseEpsilon = 1e-10;
    std::array<double, 2> priVarMagnitude{-1.0, -1.0};
    int numericDifferenceMethod = 1;
    double upwindWeight = 1.0;
    bool enableGravity = true;
};

// The tables of dxg_problem_desc filled from a problem / spatial-params pair.
struct Tabulation {
    StructuredGrid grid;
    int numEq = 1;
    std::vector<double> permeability, porosity, extrusion, source, materialParams, bcValues, initial;
    std::vector<int32_t> material;
    std::vector<int8_t> bcType;
    FluidProperties fluids;
    AssemblyParams assembly;
    dxg_problem_desc desc{};

    // Points dxg_problem_desc at the tables (valid while this object lives unchanged).
    const dxg_problem_desc& descriptor()
    {
        desc = dxg_problem_desc{};
        desc.dim = grid.dim;
        for (int a = 0; a < 3; ++a) {
            desc.cells[a] = grid.cells(a);
            desc.coords[a] = a < grid.dim ? grid.coords[a].data() : nullptr;
        }
        desc.num_eq = numEq;
        desc.enable_gravity = assembly.enableGravity ? 1 : 0;
        desc.gravity[0] = desc.gravity[1] = desc.gravity[2] = 0.0;
        desc.gravity[grid.dim - 1] = -9.81;
        for (int p = 0; p < 2; ++p) {
            desc.density[p] = fluids.density[p];
            desc.viscosity[p] = fluids.viscosity[p];
            desc.privar_magnitude[p] = assembly.priVarMagnitude[p];
        }
        desc.permeability = permeability.data();
        desc.porosity = porosity.data();
        desc.extrusion = extrusion.data();
        desc.material = material.data();
        desc.source = source.data();
        desc.num_materials = (int32_t)(materialParams.size() / 5);
        desc.material_params = materialParams.data();
        desc.bc_type = bcType.data();
        desc.bc_values = bcValues.data();
        desc.base_epsilon = assembly.baseEpsilon;
        desc.numeric_difference_method = assembly.numericDifferenceMethod;
        desc.upwind_weight = assembly.upwindWeight;
        return desc;
    }
};

namespace detail {
// SpatialParams without extrusionFactorAtPos use 1 (the reference's default).
template <class S>
auto extrusionOf(const S& s, const GlobalPosition& x, int) -> decltype(s.extrusionFactorAtPos(x))
{
    return s.extrusionFactorAtPos(x);
}
template <class S>
double extrusionOf(const S&, const GlobalPosition&, long)
{
    return 1.0;
}
template <class S>
auto materialOf(const S& s, const GlobalPosition& x, int) -> decltype(s.fluidMatrixInteractionAtPos(x))
{
    return s.fluidMatrixInteractionAtPos(x);
}
template <class S>
BrooksCoreyParams materialOf(const S&, const GlobalPosition&, long)
{
    return BrooksCoreyParams{};
}
}  // namespace detail

// Evaluates the problem's and spatial parameters' *AtPos callbacks at the cell centres
// and boundary-face centres (fvgridgeometry / fvproblem semantics), in the orderings
// documented in dumux_gb300.h.
template <int NumEq, class Problem, class SpatialParams>
Tabulation tabulate(const StructuredGrid& grid, const Problem& problem, const SpatialParams& params,
                    const FluidProperties& fluids, const AssemblyParams& assembly)
{
    static_assert(NumEq == 1 || NumEq == 2, "1p or 2p immiscible");
    Tabulation t;
    t.grid = grid;
    t.numEq = NumEq;
    t.fluids = fluids;
    t.assembly = assembly;
    const int dim = grid.dim;
    const int n0 = grid.cells(0), n1 = grid.cells(1), n2 = grid.cells(2);
    const long long N = grid.numCells();
    t.permeability.resize(N);
    t.porosity.resize(N);
    t.extrusion.resize(N);
    t.material.resize(N);
    t.source.resize(N * NumEq);
    t.initial.resize(N * NumEq);
    std::vector<BrooksCoreyParams> laws;
    for (int k = 0; k < n2; ++k)
        for (int j = 0; j < n1; ++j)
            for (int i = 0; i < n0; ++i) {
                const long long c = i + (long long)n0 * (j + (long long)n1 * k);
                GlobalPosition x{grid.center(0, i), dim > 1 ? grid.center(1, j) : 0.0,
                                 dim > 2 ? grid.center(2, k) : 0.0};
                t.permeability[c] = params.permeabilityAtPos(x);
                t.porosity[c] = params.porosityAtPos(x);
                t.extrusion[c] = detail::extrusionOf(params, x, 0);
                const auto q = problem.sourceAtPos(x);
                const auto u0 = problem.initialAtPos(x);
                for (int e = 0; e < NumEq; ++e) {
                    t.source[c * NumEq + e] = q[e];
                    t.initial[c * NumEq + e] = u0[e];
                }
                int m = 0;
                if (NumEq == 2) {
                    const BrooksCoreyParams law = detail::materialOf(params, x, 0);
                    for (m = 0; m < (int)laws.size(); ++m) {
                        const auto& l = laws[m];
                        if (l.pcEntry == law.pcEntry && l.lambda == law.lambda && l.swr == law.swr &&
                            l.snr == law.snr && l.pcLowSwe == law.pcLowSwe)
                            break;
                    }
                    if (m == (int)laws.size()) laws.push_back(law);
                }
                t.material[c] = m;
            }
    if (laws.empty()) laws.push_back(BrooksCoreyParams{});
    for (const auto& l : laws)
        t.materialParams.insert(t.materialParams.end(), {l.pcEntry, l.lambda, l.swr, l.snr, l.pcLowSwe});
    // boundary faces: sides -x,+x,-y,+y,-z,+z, each lexicographic over the other axes
    for (int f = 0; f < 2 * dim; ++f) {
        const int a = f / 2, side = f % 2;
        int o[2] = {-1, -1}, no = 0;
        for (int q = 0; q < dim; ++q)
            if (q != a) o[no++] = q;
        const int m0 = no > 0 ? grid.cells(o[0]) : 1, m1 = no > 1 ? grid.cells(o[1]) : 1;
        for (int jj = 0; jj < m1; ++jj)
            for (int ii = 0; ii < m0; ++ii) {
                GlobalPosition x{0.0, 0.0, 0.0};
                x[a] = side == 0 ? grid.coords[a].front() : grid.coords[a].back();
                if (no > 0) x[o[0]] = grid.center(o[0], ii);
                if (no > 1) x[o[1]] = grid.center(o[1], jj);
                const auto bt = problem.boundaryTypesAtPos(x);
                const bool dir = bt.hasDirichlet();
                t.bcType.push_back(dir ? 1 : 2);
                if (dir) {
                    const auto v = problem.dirichletAtPos(x);
                    for (int e = 0; e < NumEq; ++e) t.bcValues.push_back(v[e]);
                } else {
                    const auto v = problem.neumannAtPos(x);
                    for (int e = 0; e < NumEq; ++e) t.bcValues.push_back(v[e]);
                }
            }
    }
    return t;
}

// Owning handle of one device context.
class Context {
public:
    explicit Context(int device = 0, int precision = DXG_PRECISION_FP64)
    {
        const int st = dxg_ctx_create(&ctx_, device);
        if (st != DXG_OK) throw Error(st, dxg_last_error(nullptr));
        check(dxg_set_precision(ctx_, precision));
    }
    ~Context()
    {
        if (ctx_) dxg_ctx_destroy(ctx_);
    }
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;
    dxg_ctx* get() const { return ctx_; }
    void check(int st) const
    {
        if (st == DXG_OK) return;
        if (recoverable(st)) throw NumericalProblem(st, dxg_last_error(ctx_));
        throw Error(st, dxg_last_error(ctx_));
    }

private:
    dxg_ctx* ctx_ = nullptr;
};

class GpuFVAssembler;

// The assembler's Jacobian, resident on the device: the JacobianMatrix the reference's
// FVAssembler::jacobian() returns (a Dune::BCRSMatrix<FieldMatrix<double, b, b>>,
// fvassembler.hh:339-341).  Host copies in the same BCRS layout on demand.
class GpuJacobian {
public:
    explicit GpuJacobian(const GpuFVAssembler* a = nullptr) : a_(a) {}
    const GpuFVAssembler& assembler() const { return *a_; }
    int64_t N() const;             // block rows
    int64_t M() const { return N(); }
    int64_t nonzeroes() const;     // blocks
    // row pointers, block columns (sorted per row), row-major block values
    void copyToHost(std::vector<int64_t>& rowPtr, std::vector<int32_t>& col, std::vector<double>& values) const;

private:
    const GpuFVAssembler* a_;
};

// The assembler's residual, resident on the device: the ResidualType the reference's
// FVAssembler::residual() returns (fvassembler.hh:343-345).  norm() and the linear
// solver's right-hand side read it in place; host values on demand.
class GpuResidual {
public:
    explicit GpuResidual(const GpuFVAssembler* a = nullptr) : a_(a) {}
    const GpuFVAssembler& assembler() const { return *a_; }
    int64_t size() const;
    std::vector<double> toHost() const;

private:
    const GpuFVAssembler* a_;
};

// The state behind FVAssembler::gridVariables() (fvgridvariables.hh:54-129): the current
// solution lives on the device and its volume variables are evaluated from it at each
// assembly, so update / resetTimeStep / advanceTimeStep are solution transfers.
class GpuGridVariables {
public:
    explicit GpuGridVariables(GpuFVAssembler* a = nullptr) : a_(a) {}
    void update(const std::vector<double>& curSol);
    void resetTimeStep(const std::vector<double>& curSol);
    void advanceTimeStep();

private:
    GpuFVAssembler* a_;
};

// Dumux::FVAssembler over the device: the same method names, signatures and meanings
// (fvassembler.hh:101-390).  jacobian() and residual() return device-resident handles.
class GpuFVAssembler {
public:
    using Scalar = double;
    using SolutionVector = std::vector<double>;
    using ResidualType = GpuResidual;
    using JacobianMatrix = GpuJacobian;
    using GridVariables = GpuGridVariables;

    // Stationary (no previous solution) or transient (prevSol set, time step dt).
    GpuFVAssembler(Tabulation tab, int device = 0, int precision = DXG_PRECISION_FP64)
        : tab_(std::move(tab)), ctx_(device, precision), jac_(this), res_(this), gv_(this)
    {
        ctx_.check(dxg_problem_upload(ctx_.get(), &tab_.descriptor()));
        int32_t b = 0;
        ctx_.check(dxg_sizes(ctx_.get(), &numCells_, &b, &numBlocks_));
        numEq_ = b;
    }
    GpuFVAssembler(const GpuFVAssembler&) = delete;
    GpuFVAssembler& operator=(const GpuFVAssembler&) = delete;

    // FVAssembler::setLinearSystem (fvassembler.hh:294-302): the pattern and the device
    // storage of the system exist from the upload on, so this only marks the system set up
    void setLinearSystem() { linearSystemSet_ = true; }
    void setPreviousSolution(const SolutionVector& u)
    {
        ctx_.check(dxg_set_prev_solution(ctx_.get(), u.data()));
        prevSol_ = u;
        stationary_ = false;
    }
    const SolutionVector& prevSol() const { return prevSol_; }
    void setTimeStepSize(double dt)
    {
        ctx_.check(dxg_set_time_step(ctx_.get(), dt));
        dt_ = dt;
    }
    double timeStepSize() const { return dt_; }
    bool isStationaryProblem() const { return stationary_; }
    // FVAssembler::assembleJacobianAndResidual(curSol, partialReassembler): partial
    // reassembly is a Newton option on the device (dxg_newton_params); a reassembler
    // passed here is ignored
    template <class PartialReassembler = void>
    void assembleJacobianAndResidual(const SolutionVector& u, const PartialReassembler* = nullptr)
    {
        ctx_.check(dxg_set_solution(ctx_.get(), u.data()));
        ctx_.check(dxg_assemble_jacobian_and_residual(ctx_.get()));
    }
    void assembleResidual(const SolutionVector& u)
    {
        ctx_.check(dxg_set_solution(ctx_.get(), u.data()));
        ctx_.check(dxg_assemble_residual(ctx_.get()));
    }
    JacobianMatrix& jacobian() { return jac_; }
    ResidualType& residual() { return res_; }
    GridVariables& gridVariables() { return gv_; }
    // FVAssembler::updateGridVariables / resetTimeStep (fvassembler.hh:379-390)
    void updateGridVariables(const SolutionVector& u) { gv_.update(u); }
    void resetTimeStep(const SolutionVector& u) { gv_.resetTimeStep(u); }

    std::vector<double> residualHost() const
    {
        std::vector<double> r(numDofs());
        ctx_.check(dxg_get_residual(ctx_.get(), r.data()));
        return r;
    }
    // BCRS of FieldMatrix<double, numEq, numEq> blocks: row pointers, block columns, values
    void jacobianHost(std::vector<int64_t>& rowPtr, std::vector<int32_t>& col, std::vector<double>& values) const
    {
        rowPtr.resize(numCells_ + 1);
        col.resize(numBlocks_);
        values.resize(numBlocks_ * numEq_ * numEq_);
        ctx_.check(dxg_get_jacobian(ctx_.get(), rowPtr.data(), col.data(), values.data()));
    }
    double residualNorm() const
    {
        double n = 0.0;
        ctx_.check(dxg_residual_norm(ctx_.get(), &n));
        return n;
    }
    SolutionVector initialSolution() const { return tab_.initial; }
    int64_t numCells() const { return numCells_; }
    int64_t numBlocks() const { return numBlocks_; }
    int numEq() const { return numEq_; }
    int64_t numDofs() const { return numCells_ * numEq_; }
    dxg_ctx* context() const { return ctx_.get(); }
    const Context& handle() const { return ctx_; }

private:
    friend class GpuGridVariables;
    Tabulation tab_;
    Context ctx_;
    GpuJacobian jac_;
    GpuResidual res_;
    GpuGridVariables gv_;
    SolutionVector prevSol_;
    int64_t numCells_ = 0, numBlocks_ = 0;
    int numEq_ = 1;
    double dt_ = 0.0;
    bool stationary_ = true;
    bool linearSystemSet_ = false;
};

inline int64_t GpuJacobian::N() const { return a_->numCells(); }
inline int64_t GpuJacobian::nonzeroes() const { return a_->numBlocks(); }
inline void GpuJacobian::copyToHost(std::vector<int64_t>& rowPtr, std::vector<int32_t>& col,
                                    std::vector<double>& values) const
{
    a_->jacobianHost(rowPtr, col, values);
}
inline int64_t GpuResidual::size() const { return a_->numDofs(); }
inline std::vector<double> GpuResidual::toHost() const { return a_->residualHost(); }
inline void GpuGridVariables::update(const std::vector<double>& u)
{
    a_->ctx_.check(dxg_set_solution(a_->ctx_.get(), u.data()));
}
inline void GpuGridVariables::resetTimeStep(const std::vector<double>& u)
{
    a_->ctx_.check(dxg_set_solution(a_->ctx_.get(), u.data()));
}
inline void GpuGridVariables::advanceTimeStep()
{
    a_->ctx_.check(dxg_advance_time_step(a_->ctx_.get()));
    a_->prevSol_.resize(a_->numDofs());
    a_->ctx_.check(dxg_get_solution(a_->ctx_.get(), a_->prevSol_.data()));
}

// IstlSolverResult (istlsolvers.hh:153-163): converges-flag, bool-convertible.
struct GpuSolverResult : dxg_linear_result {
    explicit operator bool() const { return converged != 0; }
};

// Dumux::ILUBiCGSTABIstlSolver over the device (istlsolvers.hh:635-642): ILU(0)-
// preconditioned BiCGSTAB.  solve(A, x, b) and norm(x) take the assembler's device
// handles as the reference's take its BCRS matrix and block vectors
// (istlsolvers.hh:273, 306).
class GpuILUBiCGSTABSolver {
public:
    void setResidualReduction(double r) { reduction_ = r; }
    void setMaxIter(int n) { maxIter_ = n; }
    // DXG_ILU_AUTO (natural order, the reference's SeqILU; default) or DXG_ILU_REDBLACK
    // (red-black ordered ILU(0): not the reference's preconditioner, faster per time step);
    // takes effect at the assembler's next factorisation
    void setIluKernel(GpuFVAssembler& A, int kind) { A.handle().check(dxg_set_ilu_kernel(A.context(), kind)); }
    void setLaneRing(GpuFVAssembler& A, int form) { A.handle().check(dxg_set_lane_ring(A.context(), form)); }
    // x = A^-1 b from x = 0: A and b are the assembler's device system (the b handle must
    // be that assembler's residual); x receives the update on the host
    GpuSolverResult solve(const GpuJacobian& A, std::vector<double>& x, const GpuResidual& b)
    {
        const GpuFVAssembler& asmb = A.assembler();
        if (&b.assembler() != &asmb) throw Error(DXG_ERR_ARG, "solve: matrix and right-hand side of different assemblers");
        asmb.handle().check(dxg_set_linear_solver(asmb.context(), kind_));
        GpuSolverResult res{};
        const int st = dxg_linear_solve(asmb.context(), reduction_, maxIter_, &res);
        if (st != DXG_OK && !recoverable(st)) asmb.handle().check(st);
        if (st != DXG_OK) res.converged = 0;
        last_ = res;
        x.resize(asmb.numDofs());
        asmb.handle().check(dxg_get_update(asmb.context(), x.data()));
        return res;
    }
    // Euclidean norm (IstlIterativeLinearSolver::norm, istlsolvers.hh:306-337)
    double norm(const GpuResidual& r) const { return r.assembler().residualNorm(); }
    double norm(const std::vector<double>& x) const
    {
        double s = 0.0;
        for (double v : x) s += v * v;
        return std::sqrt(s);
    }
    const dxg_linear_result& result() const { return last_; }

protected:
    int kind_ = DXG_LINEAR_SOLVER_ILU_BICGSTAB;

private:
    double reduction_ = 1e-13;
    int maxIter_ = 250;
    dxg_linear_result last_{};
};

// Dumux::AMGBiCGSTABIstlSolver over the device (istlsolvers.hh:729-736): BiCGSTAB
// preconditioned by one V-cycle of the library's aggregation AMG (structured 2x2(x2)
// aggregates, Galerkin coarse operators, damped block-Jacobi smoothing).
class GpuAMGBiCGSTABSolver : public GpuILUBiCGSTABSolver {
public:
    GpuAMGBiCGSTABSolver() { kind_ = DXG_LINEAR_SOLVER_AMG_BICGSTAB; }
};

// Dumux::NewtonSolver over the device (newtonsolver.hh:179-852): the loop, the update,
// the shift criterion, the dt retries and the time-step suggestion run in the library.
// TimeLoop is anything with timeStepSize() and setTimeStepSize(dt), as Dumux::TimeLoop.
class GpuNewtonSolver {
public:
    explicit GpuNewtonSolver(GpuFVAssembler& assembler) : assembler_(assembler)
    {
        dxg_newton_default_params(&params_);
    }
    dxg_newton_params& params() { return params_; }
    GpuFVAssembler& assembler() { return assembler_; }

    // NewtonSolver::solve(vars, timeLoop) (newtonsolver.hh:309-355): one implicit Euler
    // step of timeLoop.timeStepSize() from the assembler's previous solution, retried with
    // dt * RetryTimeStepReductionFactor up to MaxTimeStepDivisions times; the time loop's
    // step size is left at the one that succeeded.  Throws NumericalProblem when all fail.
    template <class TimeLoop>
    void solve(std::vector<double>& x, TimeLoop& timeLoop)
    {
        if (assembler_.isStationaryProblem())
            throw Error(DXG_ERR_STATE, "time step control with a stationary problem");
        run(x, timeLoop.timeStepSize(), params_);
        timeLoop.setTimeStepSize(report_.dt_used);
    }
    // NewtonSolver::solve(vars) (newtonsolver.hh:362-368): the stationary solve, or one
    // step of the assembler's time-step size when it is transient; no retries
    void solve(std::vector<double>& x) { run(x, currentDt(), noRetry()); }
    // NewtonSolver::apply(vars) (newtonsolver.hh:380-383): as solve(vars) but reports
    // failure instead of throwing
    bool apply(std::vector<double>& x)
    {
        try {
            run(x, currentDt(), noRetry());
            return true;
        } catch (const NumericalProblem&) {
            return false;
        }
    }
    // TimeLoop::advanceTimeStep: the converged solution becomes the previous time level
    void advanceTimeStep() { assembler_.gridVariables().advanceTimeStep(); }
    double suggestTimeStepSize(double oldDt) const
    {
        return dxg_suggest_time_step(assembler_.context(), oldDt, &params_);
    }
    const dxg_newton_report& report() const { return report_; }

private:
    double currentDt() const { return assembler_.isStationaryProblem() ? 0.0 : assembler_.timeStepSize(); }
    dxg_newton_params noRetry() const
    {
        dxg_newton_params p = params_;
        p.max_time_step_divisions = 0;
        return p;
    }
    void run(std::vector<double>& x, double dt, const dxg_newton_params& p)
    {
        dxg_ctx* c = assembler_.context();
        assembler_.handle().check(dxg_set_solution(c, x.data()));
        const int st = dxg_newton_solve(c, dt, &p, &report_);
        if (st != DXG_OK) {
            // the library restored the previous solution; hand it back as the reference does
            dxg_get_solution(c, x.data());
            assembler_.handle().check(st);
        }
        assembler_.handle().check(dxg_get_solution(c, x.data()));
    }

    GpuFVAssembler& assembler_;
    dxg_newton_params params_{};
    dxg_newton_report report_{};
};

}  // namespace dumux_gb300

#endif  // DUMUX_GB300_HH
