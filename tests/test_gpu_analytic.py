"""Analytic Jacobian (DiffMethod::analytic) on the device against the oracle."""
import numpy as np
import pytest

import oracle
from dumux_gb300 import Batch, Context, newton_params, problems

pytestmark = pytest.mark.gpu


def _state(desc, u0, seed):
    rng = np.random.default_rng(seed)
    u = u0.reshape(-1, 2).copy()
    u[:, 0] += rng.uniform(-2e3, 2e3, len(u))
    u[:, 1] = rng.uniform(0.0, 0.9, len(u))
    u[::7, 1] = 0.0                 # regularised branches
    u[3::11, 1] = 0.96
    return u.reshape(-1)


def _cases():
    out = []
    d, u0 = problems.onep_lens_problem()
    d.analytic = True
    out.append(("1p-lens-2d", d, u0 + 1e5 + np.random.default_rng(0).uniform(-5e4, 5e4, u0.size), None, 0.0))
    d, u0 = problems.darcy_1p(cells=(7, 6, 5), seed=3, enable_gravity=True)
    d.analytic = True
    out.append(("1p-3d-transient", d, u0 + 5.0, u0 + 10.0, 50.0))
    for dims, name in [((12, 8), "2p-2d"), ((6, 5, 4), "2p-3d")]:
        d, u0 = problems.dnapl_2p(cells=dims, extent=(6.0, 4.0, 1.0)[:len(dims)], seed=5)
        d.analytic = True
        out.append((name, d, _state(d, u0, 7), _state(d, u0, 8), 250.0))
    return out


CASES = _cases()


@pytest.mark.parametrize("name,desc,u,up,dt", CASES, ids=[c[0] for c in CASES])
def test_analytic_jacobian_matches_oracle(name, desc, u, up, dt):
    ctx = Context(desc)
    ctx.set_solution(u)
    if up is not None:
        ctx.set_prev_solution(up)
    ctx.set_time_step(dt)
    ctx.assemble_jacobian_and_residual()
    row_ptr, col, J = ctx.jacobian()
    orow, ocol, Jo, ro = oracle.assemble(desc, u, up, dt)
    assert np.array_equal(row_ptr, orow) and np.array_equal(col, ocol)
    r = ctx.residual()
    assert np.max(np.abs(r - ro)) <= 1e-13 * np.max(np.abs(ro))
    b = desc.num_eq
    J = J.reshape(-1, b, b)
    Jo = Jo.reshape(-1, b, b)
    for pv in range(b):
        # no numeric difference to amplify the last-ulp differences of pow: ~1e-15
        scale = np.max(np.abs(Jo[:, :, pv]))
        assert np.max(np.abs(J[:, :, pv] - Jo[:, :, pv])) <= 1e-13 * scale
    if b == 1:
        assert np.array_equal(J, Jo)


def test_analytic_newton_matches_oracle():
    d, u0 = problems.dnapl_2p(cells=(8, 6, 5), seed=4)
    d.analytic = True
    p = newton_params(linear_reduction=1e-13)
    ctx = Context(d)
    ctx.set_solution(u0)
    ctx.set_prev_solution(u0)
    rep = ctx.newton_solve(250.0, p)
    st, uo, orep = oracle.newton_solve(d, u0, u0, 250.0, p)
    assert st == 0
    assert rep["iterations"] == orep["iterations"]
    assert np.max(np.abs(ctx.solution() - uo)) <= 1e-9 * np.max(np.abs(uo))


def test_analytic_problems_in_a_batch_equal_alone():
    p = newton_params(linear_max_iter=500)
    items = []
    for cells, seed in [((8, 6, 5), 31), ((7, 9, 4), 32)]:
        d, u0 = problems.dnapl_2p(cells=cells, seed=seed, corr_len=3.0)
        d.analytic = True
        items.append((d, u0))
    batch = Batch(precision="mixed")
    ids = [batch.add(d, u0, dt=250.0, t_end=500.0, params=p) for d, u0 in items]
    batch.run()
    for pid, (d, u0) in zip(ids, items):
        ctx = Context(d, precision="mixed")
        ctx.set_solution(u0)
        ctx.set_prev_solution(u0)
        for _ in range(2):
            ctx.newton_solve(250.0, p)
            ctx.advance_time_step()
        assert batch.info(pid)["state"] == "finished"
        assert np.array_equal(batch.solution(pid), ctx.solution())
