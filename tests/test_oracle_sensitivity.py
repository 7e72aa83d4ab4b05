"""How far FP64 ILU(0)-BiCGSTAB results move under a change of summation order alone.

Two runs of the same oracle, identical except for the order in which the dot products of
BiCGSTAB are summed (sequential as dune-istl's scalar product, or blocked by 256), solve the
same Newton steps.  Their per-iteration residual norms differ by ~1e-7 of the initial
residual: BiCGSTAB's solution moves by its forward error (condition number x rounding) even
at a linear reduction of 1e-13 or tighter.  Any two FP64 implementations of the algorithm
(host and device included) meet this floor; the Newton iteration counts and the converged
fields agree far below it.
"""
import numpy as np

import oracle
from dumux_gb300 import newton_params, problems


def test_summation_order_moves_intermediate_newton_residuals_not_the_solution():
    desc, u0 = problems.dnapl_2p(cells=(8, 6, 5), seed=4, inflow=0.04)
    runs = []
    for order in (0, 1):
        oracle.set_dot_order(order)
        try:
            p = newton_params(linear_reduction=1e-13, linear_max_iter=500, record_residual_norms=1)
            with oracle.pow_mode(oracle.POW_CORRECTLY_ROUNDED):
                runs.append(oracle.time_loop(desc, u0, 250.0, 3, params=p, max_dt=250.0))
        finally:
            oracle.set_dot_order(0)
    (ua, ra), (ub, rb) = runs
    dev = 0.0
    for a, b in zip(ra, rb):
        assert a["iterations"] == b["iterations"] and a["dt_used"] == b["dt_used"]
        n = a["iterations"]
        d = np.abs(np.array(a["residual_norm"][:n]) - np.array(b["residual_norm"][:n])) / a["initial_residual"]
        dev = max(dev, float(d.max()))
    assert 1e-9 < dev < 1e-5, dev
    assert np.max(np.abs(ua - ub)) <= 1e-12 * np.max(np.abs(ua))
