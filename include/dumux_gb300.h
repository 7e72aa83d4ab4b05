/*
 * dumux_gb300.h -- C ABI of the GB300-native cell-centred TPFA porous-flow hot path.
 *
 * One opaque context (dxg_ctx) owns one problem resident in device memory: the
 * tabulated problem / spatial parameters, the solution vectors, the block Jacobian,
 * the ILU(0) factors and the Krylov work vectors.  Every entry point returns an int
 * status (DXG_OK == 0); no C++ exception crosses this boundary.  Host buffers are
 * owned by the caller; device buffers are owned by the context.  A context is not
 * re-entrant; distinct contexts may be used from distinct threads.
 *
 * Each entry point names the reference interface it replaces (paths are relative to
 * the DuMux source tree).
 */
#ifndef DUMUX_GB300_H
#define DUMUX_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------ */
enum {
    DXG_OK = 0,
    DXG_ERR_ARG = 1,             /* invalid argument / unsupported configuration      */
    DXG_ERR_CUDA = 2,            /* CUDA runtime error (message via dxg_last_error)   */
    DXG_ERR_OOM = 3,             /* device allocation failed                          */
    DXG_ERR_STATE = 4,           /* call order violated (e.g. solve before assemble)  */
    DXG_ERR_LINEAR_BREAKDOWN = 5,/* BiCGSTAB breakdown (|rho| or |h| below 1e-80)     */
    DXG_ERR_LINEAR_NOT_CONVERGED = 6, /* BiCGSTAB hit maxit                           */
    DXG_ERR_NAN = 7,             /* non-finite residual / defect                      */
    DXG_ERR_NEWTON_NOT_CONVERGED = 8, /* Newton failed after all dt divisions         */
    DXG_ERR_TIMEOUT = 9,         /* a bounded device-side wait gave up                */
    DXG_ERR_NO_DEVICE = 10,      /* no CUDA device / extension built without GPU      */
    DXG_ERR_SIZE = 11,           /* input larger than a fixed capacity                */
    DXG_ERR_BUDGET = 12          /* admission would exceed the device-memory budget   */
};

/* ---- problem description (tabulated Problem + SpatialParams) ------------------
 * A structured tensor-product grid (YaspGrid semantics): cells are numbered
 * lexicographically with x fastest; the local faces of a cell are ordered
 * -x, +x, -y, +y, -z, +z (dune-grid reference-element numbering, used through
 * dumux/discretization/cellcentered/tpfa/fvgridgeometry.hh:239-330).
 *
 * Boundary faces are listed side by side in the order -x, +x, -y, +y, -z, +z; on
 * each side they are numbered lexicographically over the two remaining axes (the
 * lower axis fastest).  For dim == 2 there are four sides.
 *
 * All pointers are host pointers read during dxg_problem_upload only.            */
typedef struct dxg_problem_desc {
    int32_t dim;                 /* 2 or 3                                          */
    int32_t cells[3];            /* cells per axis (cells[2] == 1 when dim == 2)    */
    const double* coords[3];     /* vertex coordinates per axis, cells[d]+1 values  */
    int32_t num_eq;              /* 1: 1p (p), 2: 2p immiscible p0s1 (p_w, S_n)     */
    int32_t enable_gravity;      /* Problem.EnableGravity (reference default true)  */
    double gravity[3];           /* used when enable_gravity != 0                   */
    double density[2];           /* constant liquid density per phase [kg/m^3]      */
    double viscosity[2];         /* constant liquid viscosity per phase [Pa s]      */
    /* per-cell spatial parameters, N = cells[0]*cells[1]*cells[2] entries          */
    const double* permeability;  /* isotropic intrinsic permeability [m^2]          */
    const double* porosity;      /* [-]                                             */
    const double* extrusion;     /* extrusion factor, NULL -> 1                     */
    const int32_t* material;     /* material-law index per cell, NULL -> 0          */
    const double* source;        /* N*num_eq source rates [kg/m^3/s], NULL -> 0     */
    /* regularised Brooks-Corey parameter sets, 5 doubles each:
     * pcEntry, lambda, Swr, Snr, pcLowSwe (BrooksCoreyDefault)                     */
    int32_t num_materials;
    const double* material_params;
    /* boundary faces (see ordering above)                                          */
    const int8_t* bc_type;       /* 1 = Dirichlet, 2 = Neumann                      */
    const double* bc_values;     /* num_eq values per boundary face: Dirichlet
                                    primary variables or Neumann mass flux
                                    [kg/m^2/s] (positive = outflow)                  */
    /* numeric differentiation (dumux/assembly/numericepsilon.hh)                   */
    double base_epsilon;         /* Assembly.NumericDifference.BaseEpsilon (1e-10)  */
    double privar_magnitude[2];  /* Assembly.NumericDifference.PriVarMagnitude (<=0: |x|+1) */
    int32_t numeric_difference_method; /* Assembly.NumericDifferenceMethod: 1 forward, 0 central, -1 backward,
                                          5 five-point stencil (common/numericdifferentiation.hh:79-88) */
    double upwind_weight;        /* Flux.UpwindWeight (1.0)                         */
    /* Jacobian differentiation (the assembler's DiffMethod): 0 numeric (default), 1
     * analytic -- CCLocalAssembler<DiffMethod::analytic>, dumux/assembly/cclocalassembler.hh:
     * 488-604, with the flux, Dirichlet and storage derivatives of the incompressible 1p / 2p
     * local residuals (porousmediumflow/{1p,2p}/incompressiblelocalresidual.hh)         */
    int32_t diff_method;
    /* Material law of the 2p parameter sets: 0 regularised Brooks-Corey (5 doubles per set,
     * see above), 1 regularised Van Genuchten (VanGenuchtenDefault, material/
     * fluidmatrixinteractions/2p/vangenuchten.hh; 9 doubles per set: alpha [1/Pa], n, l,
     * Swr, Snr, pcLowSwe, pcHighSwe, krnLowSwe, krwHighSwe -- the reference's defaults
     * for the last four are 0.01, 0.99, 0.1, 0.9)                                        */
    int32_t material_law;
    /* Discretisation of the fluxes: DXG_DISC_TPFA (0, default) two-point flux approximation
     * (discretization/cellcentered/tpfa), or DXG_DISC_MPFA_O (1) the multi-point flux
     * approximation O-method (discretization/cellcentered/mpfa/omethod, flux/ccmpfa/darcyslaw.hh)
     * with continuity points at the face centres (MPFA.Q = 0), for the 1p and 2p models in
     * FP64 single contexts: one interaction volume per grid vertex, its local flux-continuity
     * system solved once at upload (the transmissibilities depend on geometry and permeability
     * only), a 3^dim-point Jacobian stencil and ILU(0) over it.                            */
    int32_t discretization;
    /* Full intrinsic permeability tensor per cell, N*dim*dim values (row-major, symmetric
     * positive definite), or NULL: the isotropic `permeability` above.  MPFA-O only.      */
    const double* permeability_tensor;
} dxg_problem_desc;

enum { DXG_DISC_TPFA = 0, DXG_DISC_MPFA_O = 1 };

/* Number of boundary faces implied by the grid of desc. */
int64_t dxg_num_boundary_faces(const dxg_problem_desc* desc);

/* ---- context lifecycle --------------------------------------------------------- */
typedef struct dxg_ctx dxg_ctx;

/* Creates a context on CUDA device `device`.  Replaces the construction of
 * FVAssembler + ILUBiCGSTABIstlSolver + NewtonSolver
 * (dumux/assembly/fvassembler.hh:154-172, dumux/linear/istlsolvers.hh:635-642,
 *  dumux/nonlinear/newtonsolver.hh:210-237). */
int dxg_ctx_create(dxg_ctx** out, int device);
int dxg_ctx_destroy(dxg_ctx* ctx);
/* Human-readable description of the last error of this context (or of the last
 * failed dxg_ctx_create when ctx == NULL). */
const char* dxg_last_error(const dxg_ctx* ctx);

/* Precision of the linear solve: FP64 everywhere (the plain drop-in), or the mixed
 * form: the preconditioner in FP32 (an FP32 copy of the Jacobian, FP32 ILU(0) factors and
 * triangular sweeps, or the FP32 AMG hierarchy) inside an FP64 BiCGSTAB whose operator
 * products take the FP64 Jacobian times the FP32 preconditioner output, with FP64 Krylov
 * vectors, updates and dot products -- iterative refinement of the FP64 system by an FP32
 * preconditioner, inside the FP64 residual, numeric differentiation, Newton update and
 * norms.  Must be set before upload. */
enum { DXG_PRECISION_FP64 = 0, DXG_PRECISION_MIXED = 1 };
int dxg_set_precision(dxg_ctx* ctx, int precision);

/* Tabulates the problem into device memory and builds the sparsity pattern.
 * Replaces CCTpfaFVGridGeometry::update_ (dumux/discretization/cellcentered/tpfa/
 * fvgridgeometry.hh:216), CCSimpleConnectivityMap::update (dumux/discretization/
 * cellcentered/connectivitymap.hh:66-114), getJacobianPattern (dumux/assembly/
 * jacobianpattern.hh:25-53) and FVAssembler::setLinearSystem
 * (dumux/assembly/fvassembler.hh:294-302). */
int dxg_problem_upload(dxg_ctx* ctx, const dxg_problem_desc* desc);

/* Sizes: cells, equations per cell, nonzero blocks of the Jacobian. */
int dxg_sizes(const dxg_ctx* ctx, int64_t* num_cells, int32_t* num_eq, int64_t* num_blocks);

/* ---- state ----------------------------------------------------------------------- */
/* Current solution (N*num_eq doubles, cell-major: u[cell*num_eq + pv]).
 * dxg_set_solution replaces FVAssembler::updateGridVariables
 * (dumux/assembly/fvassembler.hh:379-382). */
int dxg_set_solution(dxg_ctx* ctx, const double* u);
int dxg_get_solution(dxg_ctx* ctx, double* u);
/* Previous time level.  Replaces FVAssembler::setPreviousSolution / resetTimeStep
 * (dumux/assembly/fvassembler.hh:360-390). */
int dxg_set_prev_solution(dxg_ctx* ctx, const double* u_prev);
/* Time step size for the storage term; dt <= 0 selects the stationary residual
 * (FVAssembler::isStationaryProblem, dumux/assembly/fvassembler.hh:340). */
int dxg_set_time_step(dxg_ctx* ctx, double dt);

/* ---- assembler (dumux/assembly/fvassembler.hh) ----------------------------------- */
/* Residual and numeric-differentiation Jacobian at the current solution.
 * Replaces FVAssembler::assembleJacobianAndResidual (fvassembler.hh:178-207) with
 * CCLocalAssembler<numeric, implicit> (dumux/assembly/cclocalassembler.hh:164-348). */
int dxg_assemble_jacobian_and_residual(dxg_ctx* ctx);
/* Residual only.  Replaces FVAssembler::assembleResidual (fvassembler.hh:240-267). */
int dxg_assemble_residual(dxg_ctx* ctx);
/* Copies of the device residual / Jacobian.  The Jacobian is exported in BCRS form:
 * row_ptr[N+1], col_idx[num_blocks], values[num_blocks*num_eq*num_eq] (row-major
 * blocks, columns sorted), the layout of Dune::BCRSMatrix<FieldMatrix<double,b,b>>
 * (dumux/discretization/fvproperties.hh:66-75). */
int dxg_get_residual(dxg_ctx* ctx, double* r);
int dxg_get_jacobian(dxg_ctx* ctx, int64_t* row_ptr, int32_t* col_idx, double* values);
/* Loads a host BCRS matrix with the context's sparsity pattern (same layout as
 * dxg_get_jacobian) and a right-hand side, for stand-alone linear solves. */
int dxg_set_linear_system(dxg_ctx* ctx, const int64_t* row_ptr, const int32_t* col_idx,
                          const double* values, const double* rhs);

/* ---- linear solver (dumux/linear/istlsolvers.hh) ----------------------------------- */
typedef struct dxg_linear_result {
    int32_t converged;           /* IstlSolverResult::converged                      */
    int32_t iterations;          /* BiCGSTAB iterations (half steps rounded up)      */
    double reduction;            /* final defect / initial defect                    */
    double initial_defect;
    double final_defect;
} dxg_linear_result;
/* Solves J x = r with ILU(0)-preconditioned BiCGSTAB from x = 0 on the device (the
 * assembled Jacobian and residual), stopping when defect < reduction * defect0 or
 * after max_iter iterations.  Replaces ILUBiCGSTABIstlSolver::solve
 * (dumux/linear/istlsolvers.hh:273, 457-491, 635-642).  The solution stays on the
 * device as the Newton update; dxg_get_update copies it out. */
int dxg_linear_solve(dxg_ctx* ctx, double reduction, int32_t max_iter, dxg_linear_result* res);
int dxg_get_update(dxg_ctx* ctx, double* delta);
/* Euclidean norm of the device residual.  Replaces IstlIterativeLinearSolver::norm
 * (dumux/linear/istlsolvers.hh:306-337). */
int dxg_residual_norm(dxg_ctx* ctx, double* norm);

/* ---- Newton (dumux/nonlinear/newtonsolver.hh) ---------------------------------------- */
typedef struct dxg_newton_params {
    double max_relative_shift;   /* Newton.MaxRelativeShift (1e-8)                   */
    int32_t min_steps;           /* Newton.MinSteps (2)                              */
    int32_t max_steps;           /* Newton.MaxSteps (18)                             */
    int32_t target_steps;        /* Newton.TargetSteps (10)                          */
    int32_t use_line_search;     /* Newton.UseLineSearch (false)                     */
    double line_search_min_relaxation; /* Newton.LineSearchMinRelaxationFactor (0.125) */
    int32_t enable_residual_criterion; /* Newton.EnableResidualCriterion (false)     */
    double residual_reduction;   /* Newton.ResidualReduction (1e-5)                  */
    int32_t max_time_step_divisions;   /* Newton.MaxTimeStepDivisions (10)           */
    double retry_time_step_reduction;  /* Newton.RetryTimeStepReductionFactor (0.5)  */
    double linear_reduction;     /* LinearSolver.ResidualReduction used in Newton (1e-6) */
    int32_t linear_max_iter;     /* LinearSolver.MaxIterations (250)                 */
    int32_t record_residual_norms; /* compute ||r|| after each update as a diagnostic */
    /* Partial reassembly (Newton.EnablePartialReassembly, newtonsolver.hh:565-603 with
     * PartialReassemblerEngine<CCTpfa>, assembly/partialreassembler.hh:300-391): only the
     * Jacobian columns of cells whose relative shift accumulated since their last
     * linearisation exceeds max(min, min(max, weight*shift)) are reassembled; the others
     * keep their values.  Numeric differentiation only; single contexts only.          */
    int32_t enable_partial_reassembly;     /* (false)                                    */
    double reassembly_min_threshold;       /* Newton.ReassemblyMinThreshold (<= 0: 1e-1*max_relative_shift) */
    double reassembly_max_threshold;       /* Newton.ReassemblyMaxThreshold (<= 0: 1e2*max_relative_shift)  */
    double reassembly_shift_weight;        /* Newton.ReassemblyShiftWeight (1e-3)        */
} dxg_newton_params;

/* Fills p with the reference defaults (newtonsolver.hh:1213-1247). */
void dxg_newton_default_params(dxg_newton_params* p);

#define DXG_MAX_NEWTON_RECORD 64
typedef struct dxg_newton_report {
    int32_t converged;
    int32_t iterations;          /* Newton iterations of the last (successful) attempt */
    int32_t time_step_divisions; /* retries with reduced dt                            */
    double dt_used;              /* dt of the last attempt                             */
    int32_t linear_iterations;   /* summed over the successful attempt                 */
    int32_t wasted_iterations;   /* iterations of failed attempts                      */
    double initial_residual;     /* ||r(u^0)||                                         */
    double shift[DXG_MAX_NEWTON_RECORD];          /* max relative shift per iteration  */
    double residual_norm[DXG_MAX_NEWTON_RECORD];  /* ||r(u^{k+1})|| (when recorded)    */
    int32_t linear_iters[DXG_MAX_NEWTON_RECORD];  /* BiCGSTAB iterations per Newton step */
    double time_assemble, time_solve, time_update; /* seconds, host clock            */
} dxg_newton_report;

/* Solves one implicit-Euler time step u^{n+1} from the current solution (used as
 * initial guess) and the previous solution, with dt halving on failure.  On success
 * the solution is u^{n+1} and dt_used is reported; on failure the solution is reset
 * to the previous solution and DXG_ERR_NEWTON_NOT_CONVERGED is returned.
 * Replaces NewtonSolver::solve(x, timeLoop) (newtonsolver.hh:309-355).
 * dt <= 0: stationary problem, NewtonSolver::solve(x) (newtonsolver.hh:362-368). */
int dxg_newton_solve(dxg_ctx* ctx, double dt, const dxg_newton_params* params,
                     dxg_newton_report* report);
/* Time-step size proposal from the last Newton iteration count.
 * Replaces NewtonSolver::suggestTimeStepSize (newtonsolver.hh:784-798). */
double dxg_suggest_time_step(const dxg_ctx* ctx, double old_dt, const dxg_newton_params* params);
/* Accepts the current solution as the new previous solution (advanceTimeStep,
 * dumux/discretization/fvgridvariables.hh:54-129). */
int dxg_advance_time_step(dxg_ctx* ctx);

/* ---- tuning --------------------------------------------------------------------------- */
/* Kernels of the ILU(0) factorisation and sweeps.  DXG_ILU_AUTO / DXG_ILU_WAVEFRONT: one
 * thread-block-cluster wavefront launch per sweep; DXG_ILU_LEVELS: one launch per
 * wavefront level.  Both compute SeqILU's natural-order ILU(0) (the drop-in setting).
 * DXG_ILU_REDBLACK: ILU(0) of the red-black reordered matrix (cells coloured by the parity
 * of x+y+z) -- a different preconditioner, not the reference's: BiCGSTAB needs more
 * iterations (about 1.6-2.2x on the 2p problems), but a sweep pair is two fully
 * parallel passes instead of nx+ny+nz-2 dependent levels; the Newton solution is the
 * same to the linear and Newton tolerances.  No counterpart in the reference (dune-istl's
 * SeqILU is sequential, natural order). */
enum { DXG_ILU_AUTO = 0, DXG_ILU_WAVEFRONT = 1, DXG_ILU_LEVELS = 2, DXG_ILU_REDBLACK = 3, DXG_ILU_LANES = 4 };
/* DXG_ILU_LANES: the natural-order sweeps of 3D 2x2-block systems with two lanes per grid line
 * and one z-plane per CTA over several thread-block clusters (more SMs on the level chain);
 * the same factors and arithmetic per cell as DXG_ILU_WAVEFRONT, so the same results.
 * DXG_ILU_AUTO takes it when the timing at the first factorisation finds it faster. */
int dxg_set_ilu_kernel(dxg_ctx* ctx, int kind);
/* Form of the lane sweeps: 0 (default) times both at the first factorisation and keeps the
 * faster, 1 the register form (each step's records in a register ring, no vote per step), 2 the
 * shared-memory-ring form (records copied ahead with cp.async, faster where most plane
 * hand-offs cross thread-block clusters); both give the same bits.  DXG_ERR_ARG for 2 when it
 * does not fit the grid.  No counterpart in the reference. */
int dxg_set_lane_ring(dxg_ctx* ctx, int form);
/* Limit of every bounded wait inside the ILU(0) sweeps, in seconds (default 0.5; at most
 * 60).  A wait that runs out ends the sweep with DXG_ERR_TIMEOUT, which the Newton driver
 * treats like a failed linear solve (a time-step retry).  Raise it where the GPU is
 * time-sliced with other processes, whose turns can stall a sweep for longer.  No
 * counterpart in the reference (its sweeps run on one CPU thread). */
int dxg_set_wait_limit(dxg_ctx* ctx, double seconds);
/* The linear solver of dxg_linear_solve / dxg_newton_solve, as the reference's solver
 * types: DXG_LINEAR_SOLVER_ILU_BICGSTAB (ILUBiCGSTABIstlSolver, istlsolvers.hh:635-642;
 * default) or DXG_LINEAR_SOLVER_AMG_BICGSTAB (AMGBiCGSTABIstlSolver, istlsolvers.hh:729-736):
 * BiCGSTAB preconditioned by one V-cycle of aggregation AMG -- 2x2(x2) box aggregates of
 * the structured grid down to one cell, Galerkin coarse operators, damped block-Jacobi
 * smoothing (the parallel counterpart of dune-istl's SSOR smoother).  In the context's
 * precision (FP32 in mixed precision).  Fewer iterations than ILU(0) and no level chain;
 * not dune-istl's AMG iterate for iterate (its aggregation and smoother differ). */
enum { DXG_LINEAR_SOLVER_ILU_BICGSTAB = 0, DXG_LINEAR_SOLVER_AMG_BICGSTAB = 1 };
int dxg_set_linear_solver(dxg_ctx* ctx, int kind);
/* The ILU(0) kernels in use, as text: the wavefront launch shape (cluster size, threads,
 * prefetch depth) and, once the first factorisation has chosen it by timing, the time per
 * apply of every shape tried. */
int dxg_describe(const dxg_ctx* ctx, char* buf, int64_t len);

/* ---- diagnostics --------------------------------------------------------------------- */
/* The CUDA stream (cudaStream_t) all work of this context runs on, for event timing
 * by the caller.  No counterpart in the reference. */
void* dxg_stream_handle(const dxg_ctx* ctx);
/* Per-kernel-class event timing on the context stream (off by default).  Classes:
 * DXG_KC_ILU_SWEEP (ILU(0) forward+backward sweeps), DXG_KC_ASSEMBLY (volume
 * variables + residual/Jacobian rows), DXG_KC_SPMV, DXG_KC_ILU_FACTOR (the preconditioner's
 * setup: ILU(0) factorisation, red-black pivots or the AMG hierarchy).  Reports launches, summed device
 * milliseconds and the algorithmic bytes those launches move (each matrix block,
 * vector entry and coefficient read or written once).  No counterpart in the
 * reference. */
enum { DXG_KC_ILU_SWEEP = 0, DXG_KC_ASSEMBLY = 1, DXG_KC_SPMV = 2, DXG_KC_ILU_FACTOR = 3, DXG_KC_COUNT = 4 };
int dxg_set_kernel_timing(dxg_ctx* ctx, int enable);
int dxg_get_kernel_timing(dxg_ctx* ctx, int kernel_class, int64_t* launches, double* total_ms, double* bytes);
/* ---- allocation-free norm --------------------------------------------------------------- */
/* ||x||_2 of n doubles at device address x, written to the device address `result`,
 * queued on `stream` (a cudaStream_t; NULL selects the default stream).  For callers
 * that must not allocate device memory while they run (their device memory belongs to
 * their own allocator or budget, or a cudaMalloc would synchronise the device and stall
 * other streams): this call allocates nothing.  Its reduction scratch is a fixed 33 KB
 * array in the library's device memory, held by every GPU that loads the library until
 * the process exits; vectors longer than 8,388,608 entries are refused with
 * DXG_ERR_SIZE.  The first call on a device looks up that array's device address (once
 * per device, with the device current); make that first call before any stream capture.
 * The address is kept for the life of the process: after a cudaDeviceReset of a device the
 * entry point must not be called on that device again.
 * All calls on a device share the array, so calls whose kernels may overlap on the GPU
 * (unordered streams) race and must be ordered by the caller.  No counterpart in the
 * reference (dune-istl's norms run on the host). */
int dxg_norm2_noalloc(const double* x, int64_t n, double* result, void* stream);

/* Failure-detection self-test: runs, on `device`, the bounded wait the ILU(0) sweeps use
 * on a condition nothing satisfies -- kind 0: an mbarrier phase that never completes,
 * kind 1: a global flag nobody sets -- with a limit of limit_ns (at most 1 s).  The
 * kernel gives up, writes *kernel_status = DXG_ERR_TIMEOUT (the expected verdict) and
 * returns; *waited_ms receives how long it waited.  The call returns DXG_OK when the
 * test ran and the device stayed usable.  No counterpart in the reference. */
int dxg_selftest_bounded_wait(int device, int32_t kind, int64_t limit_ns, int32_t* kernel_status,
                              double* waited_ms);

/* Element-wise pow(x[i], y[i]) of n host values, evaluated on `device` with the library's
 * device pow -- the pow of the material laws (Brooks-Corey, Van Genuchten), which is
 * correctly rounded in binary64 on host and device alike -- and copied back to out.  For
 * checking the device arithmetic against a host's.  No counterpart in the reference (its
 * laws call the C library's std::pow). */
int dxg_device_pow(int device, const double* x, const double* y, double* out, int64_t n);

/* Dense FP64 FMA rate of `device` in TFLOP/s (all SMs, independent FMA chains, timed with
 * CUDA events): the FP64 roof of the FP64 kernels' roofline.  No counterpart in the
 * reference. */
int dxg_fp64_fma_rate(int device, double* tflops);

/* Kernel launches issued by this context since creation (all of them ours). */
int64_t dxg_kernel_launch_count(const dxg_ctx* ctx);
/* Synchronises the context stream and reports any pending CUDA error. */
int dxg_sync(dxg_ctx* ctx);

/* ---- batched and served forms -----------------------------------------------------------
 * A dxg_batch advances many independent problems together.  Each admitted problem
 * keeps its whole state (tables, solution, Jacobian, factors, Krylov vectors) in
 * device memory until it is removed.  One call of dxg_batch_iterate is one tick:
 * problems that start a Newton iteration are assembled and their ILU(0) factors
 * computed, every active problem then runs 8 BiCGSTAB iterations, and problems whose
 * linear solve ended take the Newton update and convergence test.  Problems of the
 * same kind (num_eq, dim, difference method, gravity, transient) share each kernel
 * launch, one launch per kernel for all of them, with one thread-block cluster per
 * problem in the ILU(0) sweeps; a slow problem does not hold up the others.  Between
 * iterations each problem follows its own time loop: a converged time step advances
 * it (TimeLoop::advanceTimeStep + NewtonSolver::suggestTimeStepSize, capped at the
 * problem's dt), a failed one restarts from the previous time level with dt times
 * retry_time_step_reduction (NewtonSolver::solve, dumux/nonlinear/newtonsolver.hh:
 * 309-382).  Problems may be added between iterations (continuous batching); the
 * arithmetic of a problem does not depend on what else is in the batch.
 * The reference runs such ensembles as separate processes; these entry points have
 * no counterpart there.                                                                   */
typedef struct dxg_batch dxg_batch;

typedef struct dxg_batch_problem_info {
    int32_t state;               /* 0 active, 1 finished, 2 failed                     */
    int32_t status;              /* DXG_OK or the status that ended a failed problem   */
    int32_t time_steps;          /* accepted time steps                                */
    int32_t time_step_divisions; /* dt reductions after failed Newton solves           */
    int64_t newton_iterations;   /* all Newton iterations, including wasted ones       */
    int64_t linear_iterations;   /* BiCGSTAB iterations                                */
    int64_t cells;
    double time;                 /* simulated time reached                             */
    double seconds_admitted;     /* engine clock (s since dxg_batch_create) at admission */
    double seconds_finished;     /* engine clock when it finished or failed, else -1   */
} dxg_batch_problem_info;

enum { DXG_BATCH_OPT_GRAPHS = 0, DXG_BATCH_OPT_AUTOTUNE = 1, DXG_BATCH_OPT_ILU_REDBLACK = 2, DXG_BATCH_OPT_AMG = 3 };

int dxg_batch_create(dxg_batch** out, int device, int precision);
int dxg_batch_destroy(dxg_batch* batch);
const char* dxg_batch_last_error(const dxg_batch* batch);
/* DXG_BATCH_OPT_GRAPHS: replay the BiCGSTAB iterations of a solve from one captured
 * CUDA graph (default 1).  DXG_BATCH_OPT_AUTOTUNE: choose the cluster size, threads
 * and prefetch depth of the batched ILU(0) sweeps by timing candidates on the first
 * solve of each batch shape, kept for every batch of the process on that device
 * (default 1; 0 uses a fixed rule).  DXG_BATCH_OPT_ILU_REDBLACK:
 * red-black ordered ILU(0) (as DXG_ILU_REDBLACK for a context) for every problem of the
 * batch (default 0, natural order); set before the first dxg_batch_add, else
 * DXG_ERR_STATE.  DXG_BATCH_OPT_AMG: AMG-BiCGSTAB (as DXG_LINEAR_SOLVER_AMG_BICGSTAB for a
 * context) for every problem of the batch, each V-cycle pass batched over the problems
 * that have that level (default 0); set before the first dxg_batch_add. */
int dxg_batch_set_option(dxg_batch* batch, int option, int value);
/* Device memory that admitting this problem takes (tables and all solver state). */
int64_t dxg_problem_device_bytes(const dxg_problem_desc* desc, int precision);
/* Admission limit on the device memory of all admitted problems (0: unlimited).
 * dxg_batch_add refuses with DXG_ERR_BUDGET a problem that would exceed it. */
int dxg_batch_set_memory_budget(dxg_batch* batch, int64_t bytes);
int64_t dxg_batch_device_bytes(const dxg_batch* batch);
/* Admit a problem: initial solution u0 (N*num_eq values, also the first previous
 * time level), initial time step dt, maximum time step max_dt (TimeLoop.MaxTimeStepSize;
 * <= 0: unlimited) and end time t_end (t_end <= 0: one stationary Newton solve), Newton
 * and linear-solver parameters (NULL: defaults; line search and the residual criterion
 * as in a context, partial reassembly refused with DXG_ERR_ARG).  *id receives its handle. */
int dxg_batch_add(dxg_batch* batch, const dxg_problem_desc* desc, const double* u0, double dt, double max_dt,
                  double t_end, const dxg_newton_params* params, int64_t* id);
/* One tick (see above); *active receives the number of problems still active. */
int dxg_batch_iterate(dxg_batch* batch, int32_t* active);
/* Iterates until no problem is active. */
int dxg_batch_run(dxg_batch* batch);
int dxg_batch_info(const dxg_batch* batch, int64_t id, dxg_batch_problem_info* info);
int dxg_batch_get_solution(dxg_batch* batch, int64_t id, double* u);
/* Frees the device memory of a problem (any state). */
int dxg_batch_remove(dxg_batch* batch, int64_t id);
/* Kernel launches issued by the batch (graph replays count each kernel node). */
int64_t dxg_batch_launch_count(const dxg_batch* batch);
/* Text description of the current groups and their ILU(0) sweep launch shapes. */
int dxg_batch_describe(const dxg_batch* batch, char* buf, int64_t len);
/* Per-kernel-class event timing of the batched launches (as dxg_set_kernel_timing;
 * bytes summed over the problems of each launch).  While it is on, BiCGSTAB
 * iterations are launched directly instead of from a captured graph. */
int dxg_batch_set_kernel_timing(dxg_batch* batch, int enable);
int dxg_batch_get_kernel_timing(dxg_batch* batch, int kernel_class, int64_t* launches, double* total_ms,
                                double* bytes);
void* dxg_batch_stream(const dxg_batch* batch);

#ifdef __cplusplus
}
#endif
#endif /* DUMUX_GB300_H */
