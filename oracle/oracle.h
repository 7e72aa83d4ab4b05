/*
 * oracle.h -- CPU oracle for the cc-TPFA hot path.  TEST INFRASTRUCTURE ONLY.
 *
 * A plain FP64 C++ restatement of the reference algorithm, used by the test suite,
 * the smoke check and the CPU-baseline leg of bench.py as the checker.  It is never
 * linked into, called from, or used as a fallback by the product library.
 *
 * Parity anchors (see tests/): the reference golden files
 * test/references/test_1p_cc-reference.vtu and
 * test/references/test_pcsw_brookscorey-reference.dat, the numeric-differentiation
 * known-answer table of test/common/numericdifferentiation/test_numericdifferentiation.cc
 * and the Newton mock problem of test/nonlinear/newton/test_newton.cc.
 * The dune-istl parts (ILU(0), BiCGSTAB) are restated from the published algorithms
 * (Saad, "Iterative methods for sparse linear systems", ILU(0); van der Vorst 1992,
 * BiCGSTAB) with the stopping rules of dune-istl's IterativeSolver; no golden data
 * exists for their iterates, so those are parity-unpinned beyond the converged
 * solutions.
 */
#ifndef DXG_ORACLE_H
#define DXG_ORACLE_H

#include "../include/dumux_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* number of threads used by the element loop (OpenMP); <= 0 -> all */
void orc_set_threads(int n);
int orc_get_threads(void);

/* pow of the material laws: 0 the C library's pow (as the reference, default), 1 the
 * correctly rounded pow of dumux_gb300/csrc/crpow.cuh. */
void orc_set_pow_mode(int mode);
int orc_get_pow_mode(void);
/* out[i] = pow(x[i], y[i]) in the given mode. */
void orc_pow_batch(int32_t mode, int64_t n, const double* x, const double* y, double* out);

/* Threads of the linear solve: 1 (default) sequential, as dune-istl's SeqILU and
 * BiCGSTABSolver; 0 all, n > 1 that many -- SpMV rows, vector updates and the ILU(0) rows of
 * each wavefront level in parallel, dot products sequential; identical results. */
void orc_set_linear_threads(int n);
/* Summation order of the linear solver's dot products: 0 sequential (default, as dune-istl),
 * 1 blocked by 256 -- for measuring the sensitivity of BiCGSTAB to the order alone. */
void orc_set_dot_order(int order);

/* Jacobian pattern: diagonal + (J, I) for each neighbour J of I, sorted columns. */
int orc_num_blocks(const dxg_problem_desc* d, int64_t* nnzb);
int orc_pattern(const dxg_problem_desc* d, int64_t* row_ptr, int32_t* col_idx);

/* Residual (and Jacobian if values != NULL) at u, previous solution u_prev, dt
 * (dt <= 0: stationary).  values follow orc_pattern's layout. */
int orc_assemble(const dxg_problem_desc* d, const double* u, const double* u_prev, double dt,
                 double* values, double* r);

/* ILU(0)-preconditioned BiCGSTAB from x = 0 (dune-istl SeqILU(n=0, w=1) +
 * BiCGSTABSolver semantics).  rhs is not modified. */
int orc_linear_solve(int64_t n, int32_t b, const int64_t* row_ptr, const int32_t* col_idx,
                     const double* values, const double* rhs, double* x,
                     double reduction, int32_t max_iter, dxg_linear_result* res);

/* One implicit-Euler step (or the stationary solve for dt <= 0) with the reference
 * Newton driver; u is the initial guess on entry and the solution on exit. */
int orc_newton_solve(const dxg_problem_desc* d, double* u, const double* u_prev, double dt,
                     const dxg_newton_params* p, dxg_newton_report* rep);
double orc_suggest_time_step(int32_t newton_iterations, double old_dt, const dxg_newton_params* p);

/* Regularised Brooks-Corey law (BrooksCoreyDefault); params = pcEntry, lambda, Swr,
 * Snr, pcLowSwe.  what: 0 pc, 1 krw, 2 krn. */
int orc_brooks_corey(const double* params, int32_t what, int64_t n, const double* sw, double* out);
/* Regularised Van Genuchten (VanGenuchtenDefault); params: alpha, n, l, Swr, Snr, pcLowSwe,
 * pcHighSwe, krnLowSwe, krwHighSwe; what: 0 pc, 1 krw, 2 krn, 3 dpc/dsw, 4 dkrw/dsw, 5 dkrn/dsw. */
int orc_van_genuchten(const double* params, int32_t what, int64_t n, const double* sw, double* out);

/* Numeric differentiation of the reference polynomial test function
 * f(x) = x^4/24 + x^3/6 + x^2/2 + x at x0 with the given method and eps. */
double orc_numdiff_poly(int32_t method, double eps, double x0);

/* Newton on the scalar mock problem x^2 - 5 = 0 (mock assembler / linear solver). */
int orc_newton_scalar(double x0, const dxg_newton_params* p, double* x_out, int32_t* iterations);

#ifdef __cplusplus
}
#endif
#endif
