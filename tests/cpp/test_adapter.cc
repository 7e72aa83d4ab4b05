// Drop-in check of the C++ adapter (include/dumux_gb300.hh): a DuMux-style 2p problem and
// spatial-params class, written against the reference's *AtPos interface (the shape of
// test/porousmediumflow/2p/incompressible/problem.hh and spatialparams.hh), driven through
// GpuFVAssembler / GpuILUBiCGSTABSolver / GpuNewtonSolver with the reference's method
// signatures, and by a Newton loop written only against the reference's Assembler /
// LinearSolver concepts (the calls dumux/nonlinear/newtonsolver.hh makes; the concept's
// mock is test/nonlinear/newton/test_newton.cc:30-78).
//
//   test_adapter NX NY NZ STEPS OUT.bin
// writes the solution after STEPS implicit Euler steps of 250 s as raw doubles; exits 3
// with "no-device" when no GPU is present.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "dumux_gb300.hh"

using namespace dumux_gb300;

struct Vec2 {
    double v[2];
    double operator[](int i) const { return v[i]; }
};

// Water-DNAPL problem: hydrostatic Dirichlet left/right (alpha-scaled depth), DNAPL inflow
// on the top strip 0.5 < (xmax - x)/width < 2/3, no flow elsewhere (problem.hh:74-168).
class DnaplProblem {
public:
    DnaplProblem(double xmax, double zmax, int vertical) : xmax_(xmax), zmax_(zmax), v_(vertical) {}
    BoundaryTypes boundaryTypesAtPos(const GlobalPosition& x) const
    {
        BoundaryTypes bt;
        if (x[0] < eps_ || x[0] > xmax_ - eps_) bt.setAllDirichlet();
        else bt.setAllNeumann();
        return bt;
    }
    Vec2 dirichletAtPos(const GlobalPosition& x) const
    {
        const double height = zmax_;
        const double depth = zmax_ - x[v_];
        const double alpha = 1 + 1.5 / height;
        const double width = xmax_;
        const double factor = (width * alpha + (1.0 - alpha) * x[0]) / width;
        return Vec2{{1e5 - factor * 1000.0 * (-9.81) * depth, 0.0}};
    }
    Vec2 neumannAtPos(const GlobalPosition& x) const
    {
        const double lambda = (xmax_ - x[0]) / xmax_;
        if (x[v_] > zmax_ - eps_ && 0.5 < lambda && lambda < 2.0 / 3.0) return Vec2{{0.0, -0.04}};
        return Vec2{{0.0, 0.0}};
    }
    Vec2 sourceAtPos(const GlobalPosition&) const { return Vec2{{0.0, 0.0}}; }
    Vec2 initialAtPos(const GlobalPosition& x) const
    {
        return Vec2{{1e5 - 1000.0 * (-9.81) * (zmax_ - x[v_]), 0.0}};
    }

private:
    double xmax_, zmax_;
    int v_;
    double eps_ = 1e-6;
};

// Smoothly varying permeability, porosity 0.4, BrooksCoreyDefault (pe 500, lambda 2).
class DnaplSpatialParams {
public:
    double permeabilityAtPos(const GlobalPosition& x) const
    {
        return 1e-11 * (1.0 + 0.3 * x[0] + 0.2 * x[1] * x[1] + 0.1 * x[2]);
    }
    double porosityAtPos(const GlobalPosition&) const { return 0.4; }
    BrooksCoreyParams fluidMatrixInteractionAtPos(const GlobalPosition&) const
    {
        return BrooksCoreyParams{500.0, 2.0, 0.05, 0.0, 0.01};
    }
};

// Dumux::TimeLoop's step-size interface.
struct FixedTimeLoop {
    double dt;
    double timeStepSize() const { return dt; }
    void setTimeStepSize(double d) { dt = d; }
};

// The reference's Newton iteration over any Assembler / LinearSolver pair, using only the
// calls NewtonSolver makes: setLinearSystem (newtonsolver.hh:228), setResidualReduction
// (:232), assembleJacobianAndResidual (:469-475), norm(residual()) (:494-495),
// solve(jacobian(), deltaU, residual()) (:1205), the update u = uLastIter - deltaU (:556-558),
// updateGridVariables (:861-867), the maximum relative shift (:110-128, 1138-1144) and the
// MinSteps / MaxSteps / shift-criterion decisions (:428-446, 657-701).
template <class Assembler, class LinearSolver>
int referenceShapedNewton(Assembler& assembler, LinearSolver& linearSolver, typename Assembler::SolutionVector& u,
                          double maxRelativeShift = 1e-8, int minSteps = 2, int maxSteps = 18)
{
    assembler.setLinearSystem();
    linearSolver.setResidualReduction(1e-6);
    typename Assembler::SolutionVector uLastIter = u, deltaU(u.size(), 0.0);
    double shift = 1e300;
    int numSteps = 0;
    double initialResidual = 0.0;
    auto converged = [&] { return shift <= maxRelativeShift; };
    while (numSteps < minSteps || (!converged() && numSteps < maxSteps)) {
        uLastIter = u;
        assembler.assembleJacobianAndResidual(u);
        if (numSteps == 0) initialResidual = linearSolver.norm(assembler.residual());
        std::fill(deltaU.begin(), deltaU.end(), 0.0);
        if (!linearSolver.solve(assembler.jacobian(), deltaU, assembler.residual()))
            throw NumericalProblem(DXG_ERR_LINEAR_NOT_CONVERGED, "linear solve did not converge");
        for (size_t k = 0; k < u.size(); ++k) u[k] = uLastIter[k] - deltaU[k];
        assembler.updateGridVariables(u);
        shift = 0.0;
        for (size_t k = 0; k < u.size(); ++k) {
            const double rel = std::fabs(uLastIter[k] - u[k]) / std::max(1.0, std::fabs(uLastIter[k] + u[k]) / 2.0);
            shift = std::max(shift, rel);
        }
        ++numSteps;
    }
    if (!(initialResidual > 0.0)) throw NumericalProblem(DXG_ERR_NAN, "no initial residual");
    return converged() ? numSteps : -numSteps;
}

int main(int argc, char** argv)
{
    if (argc < 6) {
        std::fprintf(stderr, "usage: %s NX NY NZ STEPS OUT.bin\n", argv[0]);
        return 2;
    }
    const int nx = std::atoi(argv[1]), ny = std::atoi(argv[2]), nz = std::atoi(argv[3]), steps = std::atoi(argv[4]);
    const StructuredGrid grid = StructuredGrid::equidistant({0.0, 0.0, 0.0}, {6.0, 4.0, 1.0}, {nx, ny, nz}, 3);
    FluidProperties fluids;
    fluids.density = {1000.0, 1460.0};
    fluids.viscosity = {1e-3, 5.7e-4};
    const DnaplProblem problem(6.0, 1.0, 2);
    const DnaplSpatialParams params;
    try {
        GpuFVAssembler assembler(tabulate<2>(grid, problem, params, fluids, AssemblyParams{}));
        std::vector<double> u = assembler.initialSolution();
        assembler.setPreviousSolution(u);
        assembler.setTimeStepSize(250.0);

        // assembler + linear solver as a LinearPDESolver would use them
        assembler.setLinearSystem();
        assembler.assembleJacobianAndResidual(u);
        std::vector<int64_t> rowPtr;
        std::vector<int32_t> col;
        std::vector<double> vals;
        assembler.jacobian().copyToHost(rowPtr, col, vals);
        if (rowPtr.back() != assembler.jacobian().nonzeroes() || assembler.jacobian().N() != assembler.numCells())
            return 1;
        GpuILUBiCGSTABSolver linear;
        linear.setResidualReduction(1e-10);
        std::vector<double> du;
        if (!linear.solve(assembler.jacobian(), du, assembler.residual())) {
            std::fprintf(stderr, "linear solve did not converge\n");
            return 1;
        }
        // norm(residual()) reads the device residual; the host copy gives the same norm
        const double rDev = linear.norm(assembler.residual()), rHost = linear.norm(assembler.residual().toHost());
        if (std::fabs(rDev - rHost) > 1e-12 * rHost) {
            std::fprintf(stderr, "norms differ: %g %g\n", rDev, rHost);
            return 1;
        }
        // the AMGBiCGSTAB solver type on the same system: the same update to the tolerance
        GpuAMGBiCGSTABSolver amg;
        amg.setResidualReduction(1e-10);
        std::vector<double> duAmg;
        if (!amg.solve(assembler.jacobian(), duAmg, assembler.residual())) {
            std::fprintf(stderr, "AMG linear solve did not converge\n");
            return 1;
        }
        double dmax = 0, umax = 0;
        for (size_t k = 0; k < du.size(); ++k) {
            dmax = std::max(dmax, std::fabs(du[k] - duAmg[k]));
            umax = std::max(umax, std::fabs(du[k]));
        }
        if (dmax > 1e-6 * umax) {
            std::fprintf(stderr, "AMG and ILU updates differ: %g of %g\n", dmax, umax);
            return 1;
        }
        // the Newton loop below uses the default ILU(0)-BiCGSTAB again
        if (dxg_set_linear_solver(assembler.context(), DXG_LINEAR_SOLVER_ILU_BICGSTAB) != DXG_OK) return 1;

        // (1) the library's Newton loop through NewtonSolver::solve(vars, timeLoop)
        GpuNewtonSolver newton(assembler);
        FixedTimeLoop timeLoop{250.0};
        std::vector<int> itsLib;
        for (int s = 0; s < steps; ++s) {
            newton.solve(u, timeLoop);
            itsLib.push_back(newton.report().iterations);
            newton.advanceTimeStep();
        }
        // (2) the reference's Newton iteration over the same classes, on a second assembler
        GpuFVAssembler asm2(tabulate<2>(grid, problem, params, fluids, AssemblyParams{}));
        std::vector<double> u2 = asm2.initialSolution();
        asm2.setPreviousSolution(u2);
        asm2.setTimeStepSize(250.0);
        GpuILUBiCGSTABSolver linear2;
        linear2.setMaxIter(newton.params().linear_max_iter);
        for (int s = 0; s < steps; ++s) {
            const int its = referenceShapedNewton(asm2, linear2, u2);
            if (its != itsLib[s]) {
                std::fprintf(stderr, "step %d: reference-shaped loop %d iterations, library %d\n", s, its, itsLib[s]);
                return 1;
            }
            asm2.gridVariables().advanceTimeStep();
            if (asm2.prevSol() != u2) return 1;
        }
        double diff = 0, scale = 0;
        for (size_t k = 0; k < u.size(); ++k) {
            diff = std::max(diff, std::fabs(u[k] - u2[k]));
            scale = std::max(scale, std::fabs(u[k]));
        }
        if (diff > 1e-12 * scale) {
            std::fprintf(stderr, "reference-shaped loop differs from the library loop: %g of %g\n", diff, scale);
            return 1;
        }
        std::FILE* f = std::fopen(argv[5], "wb");
        if (!f) return 1;
        std::fwrite(u.data(), sizeof(double), u.size(), f);
        std::fclose(f);
        std::printf("ok cells=%lld newton_last=%d linear_first=%d loops_max_diff=%g\n",
                    (long long)assembler.numCells(), newton.report().iterations, linear.result().iterations,
                    diff / scale);
        return 0;
    } catch (const Error& e) {
        if (e.status == DXG_ERR_NO_DEVICE) {
            std::printf("no-device\n");
            return 3;
        }
        std::fprintf(stderr, "error %d: %s\n", e.status, e.what());
        return 1;
    } catch (const NumericalProblem& e) {
        std::fprintf(stderr, "numerical problem %d: %s\n", e.status, e.what());
        return 1;
    }
}
