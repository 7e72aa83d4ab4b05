"""Device ILU(0)-BiCGSTAB and Newton against the CPU oracle and the golden data."""
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN
from dumux_gb300 import Context, newton_params, problems

pytestmark = pytest.mark.gpu


def _golden_p():
    return np.array([float(v) for v in open(os.path.join(GOLDEN, "onep_lens_p.txt")).read().split("\n")[1:] if v.strip()])


def test_onep_lens_linear_step_matches_reference_vtu():
    desc, u0 = problems.onep_lens_problem(numeric_epsilon=True)
    ctx = Context(desc)
    ctx.set_solution(u0)
    ctx.assemble_jacobian_and_residual()
    res = ctx.linear_solve(1e-13, 250)
    assert res["converged"]
    p = u0 - ctx.update()
    assert np.max(np.abs(p - _golden_p())) <= 0.5 + 1e-9
    # against the oracle's own solve of its own system
    row_ptr, col, vals, r = oracle.assemble(desc, u0)
    _, dx, ores = oracle.linear_solve(row_ptr, col, vals, r, 1, reduction=1e-13)
    assert np.max(np.abs(p - (u0 - dx))) <= 1e-9 * np.max(np.abs(u0 - dx))
    assert abs(res["iterations"] - ores.iterations) <= 1


@pytest.mark.parametrize("dims", [(9, 7), (6, 5, 4)])
def test_linear_solve_matches_oracle(dims):
    d, u0 = problems.dnapl_2p(cells=dims, extent=(6.0, 4.0, 1.0)[:len(dims)], seed=2)
    u = u0.reshape(-1, 2).copy()
    u[:, 1] = np.random.default_rng(1).uniform(0, 0.5, len(u))
    u = u.reshape(-1)
    ctx = Context(d)
    ctx.set_solution(u)
    ctx.set_prev_solution(u0)
    ctx.set_time_step(250.0)
    ctx.assemble_jacobian_and_residual()
    res = ctx.linear_solve(1e-13, 500)
    assert res["converged"] and res["reduction"] < 1e-13
    x = ctx.update()
    row_ptr, col, vals = ctx.jacobian()
    r = ctx.residual()
    st, xo, ores = oracle.linear_solve(row_ptr, col, vals, r, 2, reduction=1e-13, max_iter=500)
    assert st == 0
    assert np.max(np.abs(x - xo)) <= 1e-8 * np.max(np.abs(xo))
    assert abs(res["iterations"] - ores.iterations) <= max(2, 0.1 * ores.iterations)


def _run_time_loop_gpu(desc, u0, dt, steps, params, precision="fp64"):
    ctx = Context(desc, precision=precision)
    ctx.set_solution(u0)
    ctx.set_prev_solution(u0)
    reps = []
    for _ in range(steps):
        rep = ctx.newton_solve(dt, params)
        reps.append(rep)
        ctx.advance_time_step()
    return ctx.solution(), reps


def _norm_deviation(reps_a, reps_b):
    """Largest per-iteration residual-norm difference, relative to each step's initial residual."""
    dev = 0.0
    for a, b in zip(reps_a, reps_b):
        n = a["iterations"]
        d = np.abs(np.array(a["residual_norm"][:n]) - np.array(b["residual_norm"][:n])) / b["initial_residual"]
        dev = max(dev, float(d.max()))
    return dev


@pytest.mark.parametrize("pow_mode", [oracle.POW_CORRECTLY_ROUNDED, oracle.POW_LIBM], ids=["crpow", "libm"])
def test_newton_2p_matches_oracle_fp64(pow_mode):
    desc, u0 = problems.dnapl_2p(cells=(8, 6, 5), seed=4, inflow=0.04)
    p = newton_params(linear_reduction=1e-13, linear_max_iter=500, record_residual_norms=1)
    u_gpu, reps = _run_time_loop_gpu(desc, u0, 250.0, 3, p)
    with oracle.pow_mode(pow_mode):
        u_orc, oreps = oracle.time_loop(desc, u0, 250.0, 3, params=p, max_dt=250.0)
        # the same oracle with its dot products summed in another order: BiCGSTAB's solution
        # moves by its forward error (~condition number x rounding), and with it the
        # intermediate Newton residuals, by ~1e-7 of r0 on this problem
        oracle.set_dot_order(1)
        try:
            _, oreps2 = oracle.time_loop(desc, u0, 250.0, 3, params=p, max_dt=250.0)
        finally:
            oracle.set_dot_order(0)
    floor = _norm_deviation(oreps2, oreps)
    for rg, ro in zip(reps, oreps):
        assert rg["iterations"] == ro["iterations"]
        assert rg["dt_used"] == ro["dt_used"]
        assert rg["initial_residual"] == pytest.approx(ro["initial_residual"], rel=1e-12)
    # with the correctly rounded pow the assembly is bit-identical, and the device's
    # per-iteration residual norms follow the oracle's to within the oracle's own
    # sensitivity to the summation order; with the C library's pow (not correctly rounded in
    # ~0.1% of arguments) an ulp of a capillary pressure adds a ~1e-8 relative Jacobian
    # difference
    dev = _norm_deviation(reps, oreps)
    assert dev <= max(1e-9, (4.0 if pow_mode == oracle.POW_CORRECTLY_ROUNDED else 20.0) * floor), (dev, floor)
    scale = np.max(np.abs(u_orc.reshape(-1, 2)), axis=0)
    err = np.max(np.abs((u_gpu - u_orc).reshape(-1, 2)), axis=0) / scale
    assert np.all(err <= 1e-9), err
    assert np.max(u_gpu.reshape(-1, 2)[:, 1]) > 1e-3      # DNAPL entered


def test_newton_2p_mixed_precision_within_1e6():
    desc, u0 = problems.dnapl_2p(cells=(8, 6, 5), seed=4, inflow=0.04)
    p = newton_params(linear_reduction=1e-13, linear_max_iter=500)
    u_orc, _ = oracle.time_loop(desc, u0, 250.0, 3, params=p, max_dt=250.0)
    pm = newton_params(linear_reduction=1e-6, linear_max_iter=500)
    u_mix, reps = _run_time_loop_gpu(desc, u0, 250.0, 3, pm, precision="mixed")
    assert all(r["converged"] for r in reps)
    uo, um = u_orc.reshape(-1, 2), u_mix.reshape(-1, 2)
    assert np.max(np.abs(um[:, 0] - uo[:, 0])) / np.max(np.abs(uo[:, 0])) <= 1e-6
    assert np.max(np.abs(um[:, 1] - uo[:, 1])) / max(np.max(np.abs(uo[:, 1])), 1e-12) <= 1e-6


@pytest.mark.parametrize("dims,precision", [((13, 11), "fp64"), ((100, 100), "fp64"), ((37, 300), "fp64"),
                                            ((33, 70), "mixed"), ((7, 6, 9), "fp64"), ((64, 64, 32), "fp64"),
                                            ((7, 6, 9), "mixed"), ((40, 1, 3), "fp64"), ((1, 5, 4), "fp64"),
                                            ((9, 70, 5), "fp64"), ((6, 5, 37), "fp64"), ((6, 5, 37), "mixed"),
                                            ((5, 100, 19), "fp64")])
def test_wavefront_ilu_equals_level_scheduled(dims, precision):
    # the cluster wavefront kernels, the lane sweeps and the per-level kernels compute the same
    # factor and sweeps (identical operand order; the per-level kernels may differ by FMA
    # contraction).  (9, 70, 5): two CTAs per plane in the lane sweeps; (6, 5, 37) and
    # (5, 100, 19): planes in several clusters, hand-offs through global memory.
    d, u0 = problems.dnapl_2p(cells=dims, extent=(6.0, 4.0, 1.0)[:len(dims)], seed=6)
    u = u0.reshape(-1, 2).copy()
    # saturations up to 0.6 (0.3 on the long thin grids, whose systems are near BiCGSTAB
    # breakdown at 1e-12 with 0.6 -- the oracle needs 633 iterations on (9, 70, 5))
    smax = 0.3 if max(dims) >= 37 or (len(dims) == 3 and dims[1] >= 70) else 0.6
    u[:, 1] = np.random.default_rng(2).uniform(0, smax, len(u))
    out = {}
    # 2D "lanes": the one-CTA line sweeps (one thread per grid line)
    kinds = (("levels", "wavefront", "lanes", "lanes-registers", "lanes-ring") if len(dims) == 3
             else ("levels", "wavefront", "lanes"))
    for kind in kinds:
        ctx = Context(d, precision=precision)
        ctx.set_ilu_kernel(kind.split("-")[0])
        if kind != "lanes" and kind.startswith("lanes"):
            ctx.set_lane_ring(kind.split("-")[1])
        ctx.set_solution(u.reshape(-1))
        ctx.set_prev_solution(u0)
        ctx.set_time_step(250.0)
        ctx.assemble_jacobian_and_residual()
        res = ctx.linear_solve(1e-12 if precision == "fp64" else 1e-5, 1000)
        out[kind] = (res, ctx.update())
    (rl, xl), (rw, xw) = out["levels"], out["wavefront"]
    assert rl["converged"] and rw["converged"]
    assert abs(rl["iterations"] - rw["iterations"]) <= 2
    tol = 1e-7 if precision == "fp64" else 1e-3
    assert np.max(np.abs(xl - xw)) <= tol * np.max(np.abs(xl))
    for kind in ("lanes", "lanes-registers", "lanes-ring"):
        if kind in out:
            # both forms of the lane sweeps: the same arithmetic per cell as the cluster
            # wavefront, the same bits
            rn, xn = out[kind]
            assert rn["iterations"] == rw["iterations"]
            assert np.array_equal(xn, xw)


@pytest.mark.parametrize("criterion", ["line_search", "residual"])
def test_newton_line_search_and_residual_criterion_match_oracle(criterion):
    """NewtonSolver with UseLineSearch (newtonsolver.hh:1154-1178) or the residual
    criterion (EnableResidualCriterion, :657-701) on: the per-iteration residual norms
    drive the control flow, so iteration counts and fields must follow the oracle's."""
    desc, u0 = problems.twop_lens_problem(cells=(24, 16), analytic=True)
    kw = dict(use_line_search=1) if criterion == "line_search" else dict(enable_residual_criterion=1)
    p = newton_params(linear_reduction=1e-13, linear_max_iter=500, record_residual_norms=1, **kw)
    u_gpu, reps = _run_time_loop_gpu(desc, u0, 500.0, 3, p)
    u_orc, oreps = oracle.time_loop(desc, u0, 500.0, 3, params=p, max_dt=500.0)
    for rg, ro in zip(reps, oreps):
        assert rg["iterations"] == ro["iterations"]
        rn_g, rn_o = np.array(rg["residual_norm"]), np.array(ro["residual_norm"])
        assert np.all(np.abs(rn_g - rn_o) <= 1e-9 * rg["initial_residual"])
    assert np.max(np.abs(u_gpu - u_orc)) <= 1e-9 * np.max(np.abs(u_orc))


@pytest.mark.parametrize("mpfa", [False, True])
def test_kernel_timing_classes_cover_the_factorisation(mpfa):
    """Per-class event timing: sweeps, assembly, SpMV and the preconditioner setup (one ILU(0)
    factorisation per Newton iteration) all report launches, time and algorithmic bytes."""
    d, u0 = (problems.dnapl_2p_mpfa(cells=(8, 6, 5), seed=2) if mpfa else
             problems.dnapl_2p(cells=(8, 6, 5), seed=2))
    ctx = Context(d)
    ctx.set_solution(u0)
    ctx.set_prev_solution(u0)
    ctx.set_kernel_timing(True)
    rep = ctx.newton_solve(250.0, newton_params())
    assert rep["converged"]
    for kind in ("ilu_sweep", "assembly", "spmv", "ilu_factor"):
        n, ms, by = ctx.kernel_timing(kind)
        assert n > 0 and ms > 0 and by > 0, kind
    assert ctx.kernel_timing("ilu_factor")[0] == rep["iterations"]
