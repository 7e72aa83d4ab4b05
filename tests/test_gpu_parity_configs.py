"""The FP64 device path against the oracle at the benchmark configurations' full sizes.

* 1p stationary Darcy, 100x100 cells, one Newton step (LinearPDESolver semantics,
  dumux/linear/pdesolver.hh:62-298) with ILU(0)-BiCGSTAB to a relative residual of 1e-12;
* 2p water-DNAPL, 64x64x32 cells, ten implicit-Euler steps of 250 s (NewtonSolver::solve
  with the time loop, dumux/nonlinear/newtonsolver.hh:309-382, 917-1072), linear
  reduction 1e-13.

The oracle runs with the correctly rounded pow (the device's), so assembly is compared bit
for bit and the remaining differences are the summation order of the dot products inside
BiCGSTAB.  Its linear solve runs on all host threads (level-scheduled ILU(0), identical
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
    assert abs(res["iterations"] - ores.iterations) <= 1


def test_config2_dnapl_64x64x32_ten_steps():
    desc, u0 = problems.dnapl_2p(cells=(64, 64, 32), seed=2)
    p = newton_params(linear_reduction=1e-13, linear_max_iter=500, record_residual_norms=1)
    steps = 10
    ctx = Context(desc)
    ctx.set_solution(u0)
    ctx.set_prev_solution(u0)
    reps = []
    for _ in range(steps):
        rep = ctx.newton_solve(250.0, p)
        assert rep["converged"]
        reps.append(rep)
        ctx.advance_time_step()
    u_gpu = ctx.solution()
    u_orc, oreps = oracle.time_loop(desc, u0, 250.0, steps, params=p, max_dt=250.0)
    worst = 0.0
    for k, (rg, ro) in enumerate(zip(reps, oreps)):
        assert rg["iterations"] == ro["iterations"], (k, rg["iterations"], ro["iterations"])
        assert rg["dt_used"] == ro["dt_used"]
        # the residual of the step's initial state is assembled from identical states
        # (bit-identical assembly) until the first update
        r0 = ro["initial_residual"]
        if k == 0:
            assert rg["initial_residual"] == r0
        assert abs(rg["initial_residual"] - r0) <= 1e-9 * r0
        n = rg["iterations"]
        rn_g, rn_o = np.array(rg["residual_norm"][:n]), np.array(ro["residual_norm"][:n])
        # per-iteration residual norms, relative to the step's initial residual
        dev = np.abs(rn_g - rn_o) / r0
        worst = max(worst, float(dev.max()))
        assert np.all(dev <= 1e-9), (k, dev)
    uo, ug = u_orc.reshape(-1, 2), u_gpu.reshape(-1, 2)
    err_p = np.max(np.abs(ug[:, 0] - uo[:, 0])) / np.max(np.abs(uo[:, 0]))
    err_s = np.max(np.abs(ug[:, 1] - uo[:, 1])) / np.max(np.abs(uo[:, 1]))
    print(f"config 2 parity: worst residual-norm deviation {worst:.2e} of r0, p_w {err_p:.2e}, S_n {err_s:.2e}")
    assert err_p <= 1e-9 and err_s <= 1e-9
    assert np.max(uo[:, 1]) > 1e-2            # DNAPL has entered
