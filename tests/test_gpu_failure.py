"""Failure detection without a GPU fault: bounded device waits that expire on purpose,
and failures made on the host that a batch isolates to the failing problem."""
import numpy as np
import pytest

from dumux_gb300 import Batch, Context, newton_params, problems, selftest_bounded_wait

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", ["mbarrier", "flag"])
def test_bounded_wait_expires_and_reports_timeout(kind):
    status, waited = selftest_bounded_wait(kind, limit_ms=2.0)
    assert status == "DXG_ERR_TIMEOUT"
    assert 2.0 <= waited < 1000.0
    # the device stays usable: a solve on a fresh context runs normally afterwards
    desc, u0 = problems.dnapl_2p(cells=(6, 5, 4), seed=3)
    ctx = Context(desc)
    ctx.set_solution(u0)
    ctx.set_prev_solution(u0)
    rep = ctx.newton_solve(250.0, newton_params())
    assert rep["converged"]


def test_failing_problem_is_isolated_in_a_batch():
    """One member fails on the host's decision (one Newton step allowed, no dt retry):
    it ends failed with DXG_ERR_NEWTON_NOT_CONVERGED, the others finish as they would alone."""
    good = newton_params(linear_max_iter=500)
    bad = newton_params(linear_max_iter=500, min_steps=1, max_steps=1, max_time_step_divisions=0)
    d1, u1 = problems.dnapl_2p(cells=(8, 6, 5), seed=61, corr_len=3.0)
    d2, u2 = problems.dnapl_2p(cells=(7, 9, 6), seed=62, corr_len=3.0)
    batch = Batch(precision="mixed")
    p_ok = batch.add(d1, u1, dt=250.0, t_end=500.0, params=good)
    p_bad = batch.add(d2, u2, dt=250.0, t_end=500.0, params=bad)
    batch.run()
    assert batch.info(p_bad)["state"] == "failed"
    assert batch.info(p_bad)["status"] == 8          # DXG_ERR_NEWTON_NOT_CONVERGED
    assert batch.info(p_ok)["state"] == "finished"
    ctx = Context(d1, precision="mixed")
    ctx.set_solution(u1)
    ctx.set_prev_solution(u1)
    for _ in range(2):
        ctx.newton_solve(250.0, good)
        ctx.advance_time_step()
    assert np.array_equal(batch.solution(p_ok), ctx.solution())


@pytest.mark.parametrize("form", ["registers", "ring"])
def test_lane_sweep_wait_limit_expires_and_the_context_recovers(form):
    """A wait limit far below the hand-off latency of the lane sweeps (plane 31 of a 32-plane
    grid receives its first value after 31 plane steps): the sweeps give up and the solve
    reports DXG_ERR_TIMEOUT; with the limit restored, the same context solves to the same
    bits as before (the hand-off buffer is reset after a timeout)."""
    desc, u0 = problems.dnapl_2p(cells=(16, 16, 32), seed=8)
    u = u0.reshape(-1, 2).copy()
    u[:, 1] = np.random.default_rng(5).uniform(0.0, 0.4, len(u))
    ctx = Context(desc)
    ctx.set_ilu_kernel("lanes")
    ctx.set_lane_ring(form)
    ctx.set_solution(u.reshape(-1))
    ctx.set_prev_solution(u0)
    ctx.set_time_step(250.0)
    ctx.assemble_jacobian_and_residual()
    first = ctx.linear_solve(1e-10, 500)          # factorises with the default limit
    assert first["converged"]
    x0 = ctx.update()
    ctx.set_wait_limit(1e-6)
    with pytest.raises(Exception, match="timed out"):
        ctx.linear_solve(1e-10, 500)
    ctx.set_wait_limit(0.5)
    again = ctx.linear_solve(1e-10, 500)
    assert again["converged"] and again["iterations"] == first["iterations"]
    assert np.array_equal(ctx.update(), x0)


def test_lane_ring_form_refused_where_it_does_not_fit():
    """A grid whose lane sweeps fit only in the register form (200-cell lines: the
    shared-memory ring would not fit beside the plane history): dxg_set_lane_ring refuses the
    ring form with DXG_ERR_ARG and the context keeps working with the register form."""
    desc, u0 = problems.dnapl_2p(cells=(200, 8, 4), seed=3)
    u = u0.reshape(-1, 2).copy()
    u[:, 1] = np.random.default_rng(1).uniform(0.0, 0.3, len(u))
    ctx = Context(desc)
    ctx.set_ilu_kernel("lanes")
    with pytest.raises(Exception):
        ctx.set_lane_ring("ring")
    ctx.set_lane_ring("registers")
    ctx.set_solution(u.reshape(-1))
    ctx.set_prev_solution(u0)
    ctx.set_time_step(250.0)
    ctx.assemble_jacobian_and_residual()
    res = ctx.linear_solve(1e-10, 1000)
    assert res["converged"] and "register ring" in ctx.describe()
