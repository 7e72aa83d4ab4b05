"""The oracle's analytic Jacobian (DiffMethod::analytic restated from
porousmediumflow/{1p,2p}/incompressiblelocalresidual.hh) against its own numeric one:
both differentiate the same residual, so they agree to the numeric difference's accuracy,
and the residuals are identical."""
import numpy as np
import pytest

import oracle
from dumux_gb300 import problems


def _state(desc, u0, seed):
    rng = np.random.default_rng(seed)
    u = u0.reshape(-1, 2).copy()
    u[:, 0] += rng.uniform(-2e3, 2e3, len(u))
    u[:, 1] = rng.uniform(0.05, 0.6, len(u))      # away from the regularisation kinks
    return u.reshape(-1)


@pytest.mark.parametrize("dims", [(7, 5), (5, 4, 3)])
def test_analytic_matches_central_differences_2p(dims):
    d, u0 = problems.dnapl_2p(cells=dims, extent=(6.0, 4.0, 1.0)[:len(dims)], seed=5)
    u = _state(d, u0, 1)
    up = _state(d, u0, 2)
    d.numeric_difference_method = 0            # central differences: O(eps^2)
    _, _, Jn, rn = oracle.assemble(d, u, up, 250.0)
    d.analytic = True
    _, _, Ja, ra = oracle.assemble(d, u, up, 250.0)
    assert np.array_equal(ra, rn)
    Jn = Jn.reshape(-1, 2, 2)
    Ja = Ja.reshape(-1, 2, 2)
    # compare each column of the blocks against that column's scale (pressure vs saturation)
    for pv in range(2):
        scale = np.max(np.abs(Jn[:, :, pv]))
        assert np.max(np.abs(Ja[:, :, pv] - Jn[:, :, pv])) <= 1e-5 * scale


def test_analytic_matches_numeric_1p():
    d, u0 = problems.darcy_1p(cells=(9, 7), seed=3)
    u = u0 + np.random.default_rng(0).uniform(-5e3, 5e3, u0.size)
    _, _, Jn, rn = oracle.assemble(d, u)
    d.analytic = True
    _, _, Ja, ra = oracle.assemble(d, u)
    assert np.array_equal(ra, rn)
    assert np.max(np.abs(Ja - Jn)) <= 1e-5 * np.max(np.abs(Jn))


def test_analytic_newton_converges_to_the_numeric_solution():
    d, u0 = problems.dnapl_2p(cells=(8, 6, 4), seed=7)
    from dumux_gb300.abi import newton_params
    p = newton_params(linear_reduction=1e-10)
    st_n, u_n, rep_n = oracle.newton_solve(d, u0, u0, 250.0, p)
    d.analytic = True
    st_a, u_a, rep_a = oracle.newton_solve(d, u0, u0, 250.0, p)
    assert st_n == 0 and st_a == 0
    assert np.max(np.abs(u_a - u_n)) <= 1e-6 * np.max(np.abs(u_n))
