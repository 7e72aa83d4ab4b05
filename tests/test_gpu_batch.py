"""Batched and served forms: every problem's result in a batch equals its result alone.

The batch engine launches each kernel once for all problems of a kind; a problem's
arithmetic (its reduction block counts, its operand order) does not depend on the rest
of the batch, so batched and single-context results are compared bit for bit.
"""
import numpy as np
import pytest

from dumux_gb300 import Batch, Context, NumericalProblem, newton_params, problem_device_bytes, problems

pytestmark = pytest.mark.gpu


def run_alone(desc, u0, dt, t_end, params, precision):
    """The same problem through one context: the reference's time loop
    (NewtonSolver::solve with dt retries, suggestTimeStepSize capped by dt and by the
    remaining time) driven from the host."""
    ctx = Context(desc, precision=precision)
    ctx.set_solution(u0)
    ctx.set_prev_solution(u0)
    iters = 0
    if t_end <= 0.0:
        rep = ctx.newton_solve(0.0, params)
        return ctx.solution(), rep["iterations"], "finished"
    t, dtc = 0.0, min(dt, t_end)
    while True:
        try:
            rep = ctx.newton_solve(dtc, params)
        except NumericalProblem:
            return ctx.solution(), None, "failed"
        iters += rep["iterations"] + rep["wasted_iterations"]
        t += rep["dt_used"]
        ctx.advance_time_step()
        remaining = t_end - t
        if remaining <= 1e-9 * max(1.0, t_end):
            return ctx.solution(), iters, "finished"
        dtc = min(ctx.suggest_time_step(rep["dt_used"], params), dt, remaining)


def _two_phase(cells, seed, sigma=1.0, corr=4.0, inflow=0.04):
    extent = (6.0, 4.0, 1.0)[:len(cells)]
    return problems.dnapl_2p(cells=cells, extent=extent, seed=seed, sigma=sigma, corr_len=corr, inflow=inflow)


def _check_same(ub, ua, label):
    if not np.array_equal(ub, ua):
        rel = np.max(np.abs(ub - ua)) / max(1e-300, np.max(np.abs(ua)))
        pytest.fail(f"{label}: batched result differs from the single-problem result (max rel {rel:.3e})")


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_ensemble_equals_single_problems(precision):
    """Uneven 3D grids, own ln K fields and inflow rates, three time steps each."""
    params = newton_params(linear_max_iter=500)
    cases = [((8, 6, 5), 11, 0.5, 3.0, 0.01), ((12, 10, 6), 12, 2.0, 10.0, 0.08), ((6, 9, 7), 13, 1.2, 5.0, 0.04),
             ((16, 5, 4), 14, 1.0, 6.0, 0.03)]
    batch = Batch(precision=precision)
    ids = []
    for cells, seed, sigma, corr, inflow in cases:
        desc, u0 = _two_phase(cells, seed, sigma, corr, inflow)
        ids.append((batch.add(desc, u0, dt=250.0, t_end=750.0, params=params), desc, u0))
    batch.run()
    assert batch.kernel_launches() > 0
    for pid, desc, u0 in ids:
        info = batch.info(pid)
        ua, iters, state = run_alone(desc, u0, 250.0, 750.0, params, precision)
        assert info["state"] == state == "finished"
        assert info["time_steps"] >= 3 and abs(info["time"] - 750.0) < 1e-6
        assert info["newton_iterations"] == iters
        _check_same(batch.solution(pid), ua, f"problem {desc.cells}")


def test_continuous_batching_mixed_kinds_equal_alone():
    """Requests of different kinds (1p 2D stationary, 2p 2D and 3D transient) admitted
    while others are in flight: each result equals the one computed alone."""
    params = newton_params(linear_max_iter=500)
    first = [_two_phase((8, 6, 5), 21) + (250.0, 750.0),
             problems.darcy_1p(cells=(12, 10), seed=22, corr_len=3.0) + (0.0, 0.0)]
    later = [_two_phase((6, 7, 6), 23, inflow=0.06) + (250.0, 500.0),
             _two_phase((10, 8), 24) + (100.0, 300.0),
             problems.darcy_1p(cells=(9, 14), seed=25, corr_len=2.0) + (0.0, 0.0)]
    batch = Batch(precision="mixed")
    admitted = []
    for desc, u0, dt, t_end in first:
        admitted.append((batch.add(desc, u0, dt=dt, t_end=t_end, params=params), desc, u0, dt, t_end))
    batch.iterate()
    batch.iterate()
    for desc, u0, dt, t_end in later:
        admitted.append((batch.add(desc, u0, dt=dt, t_end=t_end, params=params), desc, u0, dt, t_end))
    while batch.iterate() > 0:
        pass
    for pid, desc, u0, dt, t_end in admitted:
        info = batch.info(pid)
        ua, iters, state = run_alone(desc, u0, dt, t_end, params, "mixed")
        assert info["state"] == state == "finished", (desc.cells, info)
        assert info["newton_iterations"] == iters
        assert info["seconds_finished"] >= info["seconds_admitted"]
        _check_same(batch.solution(pid), ua, f"problem {desc.cells} num_eq={desc.num_eq}")


def test_graphs_and_autotuning_do_not_change_results():
    params = newton_params(linear_max_iter=500)
    cases = [_two_phase((10, 7, 6), 31), _two_phase((7, 12, 5), 32, sigma=1.5)]
    results = []
    for graphs, autotune in [(True, True), (False, False)]:
        batch = Batch(precision="mixed", graphs=graphs, autotune=autotune)
        ids = [batch.add(d, u0, dt=250.0, t_end=500.0, params=params) for d, u0 in cases]
        batch.run()
        results.append([batch.solution(i) for i in ids])
    for a, b in zip(*results):
        assert np.array_equal(a, b)


def test_admission_by_device_memory_budget():
    params = newton_params(linear_max_iter=500)
    d1, u1 = _two_phase((8, 6, 5), 41)
    d2, u2 = _two_phase((12, 10, 8), 42)
    need1 = problem_device_bytes(d1, "mixed")
    need2 = problem_device_bytes(d2, "mixed")
    assert need2 > need1
    batch = Batch(precision="mixed", memory_budget=need2 + need1 // 2)   # either alone fits, not both
    p1 = batch.add(d1, u1, dt=250.0, t_end=250.0, params=params)
    assert p1 is not None and batch.device_bytes() == need1
    assert batch.add(d2, u2, dt=250.0, t_end=250.0, params=params) is None   # over the budget
    batch.run()
    assert batch.info(p1)["state"] == "finished"
    batch.remove(p1)
    assert batch.device_bytes() == 0
    p2 = batch.add(d2, u2, dt=250.0, t_end=250.0, params=params)
    assert p2 is not None
    batch.run()
    ua, _, _ = run_alone(d2, u2, 250.0, 250.0, params, "mixed")
    _check_same(batch.solution(p2), ua, "admitted after release")


def test_time_step_retries_follow_the_single_problem_path():
    """A large first step that Newton may reject: dt reductions and the recovered
    solution match the single-problem time loop."""
    params = newton_params(linear_max_iter=500, max_steps=6)
    desc, u0 = _two_phase((8, 8, 6), 51, inflow=0.08)
    batch = Batch(precision="fp64")
    pid = batch.add(desc, u0, dt=20000.0, t_end=20000.0, params=params)
    batch.run()
    info = batch.info(pid)
    ua, iters, state = run_alone(desc, u0, 20000.0, 20000.0, params, "fp64")
    assert info["state"] == state
    if state == "finished":
        assert info["newton_iterations"] == iters
        _check_same(batch.solution(pid), ua, "retried step")


def test_line_search_and_residual_criterion_in_a_batch_equal_alone():
    """Newton.UseLineSearch and Newton.EnableResidualCriterion members batched beside a
    plain member of the same kind: each follows its single-problem path bit for bit."""
    plain = newton_params(linear_max_iter=500)
    search = newton_params(linear_max_iter=500, use_line_search=1)
    resid = newton_params(linear_max_iter=500, enable_residual_criterion=1, residual_reduction=1e-6)
    cases = [((8, 6, 5), 21, plain), ((10, 7, 6), 22, search), ((9, 8, 5), 23, resid), ((7, 9, 6), 24, search)]
    batch = Batch(precision="fp64")
    ids = []
    for cells, seed, params in cases:
        desc, u0 = _two_phase(cells, seed, sigma=1.5, inflow=0.08)
        ids.append((batch.add(desc, u0, dt=500.0, t_end=1500.0, params=params), desc, u0, params))
    batch.run()
    for pid, desc, u0, params in ids:
        info = batch.info(pid)
        ua, iters, state = run_alone(desc, u0, 500.0, 1500.0, params, "fp64")
        assert info["state"] == state == "finished"
        assert info["newton_iterations"] == iters
        _check_same(batch.solution(pid), ua, f"problem {desc.cells}")


def test_partial_reassembly_is_refused_by_a_batch():
    desc, u0 = _two_phase((6, 5, 4), 25)
    batch = Batch(precision="fp64")
    with pytest.raises(Exception):
        batch.add(desc, u0, dt=250.0, t_end=250.0, params=newton_params(enable_partial_reassembly=1))
