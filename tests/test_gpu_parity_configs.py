"""The FP64 device path against the oracle at the benchmark configurations' full sizes.

* 1p stationary Darcy, 100x100 cells, one Newton step (LinearPDESolver semantics,
  dumux/linear/pdesolver.hh:62-298) with ILU(0)-BiCGSTAB to a relative residual of 1e-12;
* 2p water-DNAPL, 64x64x32 cells, ten implicit-Euler steps (NewtonSolver::solve with the
  time loop, dumux/nonlinear/newtonsolver.hh:309-382, 917-1072; TimeLoop.MaxTimeStepSize
  250 s, the step size the Newton solver's suggestTimeStepSize gives below that, :784-798),
  linear reduction 1e-13.

The oracle runs with the correctly rounded pow (the device's), so assembly is compared bit
for bit and the remaining differences come from the summation order of the dot products and
the FMA use inside BiCGSTAB.  Those move BiCGSTAB's solution by its forward error (condition
number x rounding), and with it the intermediate Newton residuals: the oracle itself moves
by as much under a change of its summation order, which the tests measure and use as the
bound.  Newton iteration counts, time-step sizes and the converged fields agree to 1e-9.
The oracle's linear solve runs on all host threads (level-scheduled ILU(0), identical
results to the sequential solve).
"""
import numpy as np
import pytest

import oracle
from dumux_gb300 import Context, newton_params, problems

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _oracle_setup():
    prev = oracle.get_pow_mode()
    oracle.set_pow_mode(oracle.POW_CORRECTLY_ROUNDED)
    oracle.set_linear_threads(0)
    yield
    oracle.set_linear_threads(1)
    oracle.set_pow_mode(prev)


def test_config1_darcy_100x100_one_step():
    desc, u0 = problems.darcy_1p(cells=(100, 100), seed=1)
    ctx = Context(desc)
    ctx.set_solution(u0)
    ctx.assemble_jacobian_and_residual()
    r_gpu = ctx.residual()
    row_ptr, col, vals = ctx.jacobian()
    orow, ocol, ovals, r_orc = oracle.assemble(desc, u0)
    assert np.array_equal(row_ptr, orow) and np.array_equal(col, ocol)
    assert np.array_equal(vals, ovals) and np.array_equal(r_gpu, r_orc)
    res = ctx.linear_solve(1e-12, 250)
    assert res["converged"] and res["reduction"] < 1e-12
    p_gpu = u0 - ctx.update()
    st, dx, ores = oracle.linear_solve(orow, ocol, ovals, r_orc, 1, reduction=1e-12, max_iter=250)
    assert st == 0 and ores.converged
    p_orc = u0 - dx
    assert np.max(np.abs(p_gpu - p_orc)) <= 1e-9 * np.max(np.abs(p_orc))
    # BiCGSTAB's iterates depend on the summation order of its dot products (sequential on
    # the host, tree-shaped on the device) and on the rounding of the factor; on this field
    # (sigma = 1) that moves the iteration count at 1e-12 by several percent, not the
    # solution.  The bound is the oracle's own spread under another summation order.
    oracle.set_dot_order(1)
    try:
        _, _, ores2 = oracle.linear_solve(orow, ocol, ovals, r_orc, 1, reduction=1e-12, max_iter=250)
    finally:
        oracle.set_dot_order(0)
    floor = abs(ores2.iterations - ores.iterations)
    assert abs(res["iterations"] - ores.iterations) <= max(2, 0.03 * ores.iterations, 1.5 * floor)


def test_config2_dnapl_64x64x32_ten_steps():
    desc, u0 = problems.dnapl_2p(cells=(64, 64, 32), seed=2)
    p = newton_params(linear_reduction=1e-13, linear_max_iter=500, record_residual_norms=1)
    steps = 10
    ctx = Context(desc)
    ctx.set_solution(u0)
    ctx.set_prev_solution(u0)
    reps = []
    dt = 250.0
    for _ in range(steps):
        rep = ctx.newton_solve(dt, p)
        assert rep["converged"]
        reps.append(rep)
        ctx.advance_time_step()
        # TimeLoop with MaxTimeStepSize 250 s: the Newton solver's suggestion, capped
        dt = min(ctx.suggest_time_step(rep["dt_used"], p), 250.0)
    u_gpu = ctx.solution()
    u_orc, oreps = oracle.time_loop(desc, u0, 250.0, steps, params=p, max_dt=250.0)
    # the oracle's own sensitivity to the summation order of its dot products, over the
    # first steps: the floor any two FP64 implementations of BiCGSTAB meet
    oracle.set_dot_order(1)
    try:
        _, oreps2 = oracle.time_loop(desc, u0, 250.0, 2, params=p, max_dt=250.0)
    finally:
        oracle.set_dot_order(0)
    worst, floor, worst_first = 0.0, 0.0, 0.0
    for k, (rg, ro) in enumerate(zip(reps, oreps)):
        assert rg["iterations"] == ro["iterations"], (k, rg["iterations"], ro["iterations"])
        assert rg["dt_used"] == ro["dt_used"]
        # the step's initial residual: bit-identical assembly of the first step's state; the
        # norms differ by their summation order (tree on the device, sequential on the host)
        r0 = ro["initial_residual"]
        assert abs(rg["initial_residual"] - r0) <= (1e-13 if k == 0 else 1e-9) * r0
        n = rg["iterations"]
        dev = np.abs(np.array(rg["residual_norm"][:n]) - np.array(ro["residual_norm"][:n])) / r0
        worst = max(worst, float(dev.max()))
        if k < len(oreps2):
            worst_first = max(worst_first, float(dev.max()))
            n2 = oreps2[k]["iterations"]
            assert n2 == ro["iterations"]
            d2 = np.abs(np.array(oreps2[k]["residual_norm"][:n2]) - np.array(ro["residual_norm"][:n2])) / r0
            floor = max(floor, float(d2.max()))
    uo, ug = u_orc.reshape(-1, 2), u_gpu.reshape(-1, 2)
    err_p = np.max(np.abs(ug[:, 0] - uo[:, 0])) / np.max(np.abs(uo[:, 0]))
    err_s = np.max(np.abs(ug[:, 1] - uo[:, 1])) / np.max(np.abs(uo[:, 1]))
    print(f"config 2 parity: residual-norm deviation of r0 {worst:.2e} (first steps {worst_first:.2e}, oracle "
          f"against itself with another summation order {floor:.2e}); fields p_w {err_p:.2e}, S_n {err_s:.2e}")
    assert worst_first <= max(1e-9, 4.0 * floor)
    # later steps start from states that already differ by the earlier steps' rounding
    assert worst <= max(1e-9, 10.0 * floor)
    assert err_p <= 1e-9 and err_s <= 1e-9
    assert np.max(uo[:, 1]) > 1e-2            # DNAPL has entered
