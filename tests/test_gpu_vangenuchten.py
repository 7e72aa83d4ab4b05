"""Van Genuchten on the device: assembly against the oracle, and the reference's 2p lens
case end to end against the oracle and the reference's golden VTU."""
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN
from dumux_gb300 import Batch, Context, newton_params, problems

pytestmark = pytest.mark.gpu


def _state(desc, u0, seed):
    rng = np.random.default_rng(seed)
    u = u0.reshape(-1, 2).copy()
    u[:, 0] += rng.uniform(-2e3, 2e3, len(u))
    u[:, 1] = rng.uniform(0.0, 0.85, len(u))
    u[::7, 1] = 0.0                 # regularised branches: pc spline, krw spline
    u[3::11, 1] = 0.995             # pc low-swe extension
    u[5::13, 1] = 0.9               # krn spline
    return u.reshape(-1)


@pytest.mark.parametrize("analytic", [False, True])
def test_vangenuchten_assembly_matches_oracle(analytic):
    desc, u0 = problems.twop_lens_problem(cells=(12, 10), analytic=analytic)
    u = _state(desc, u0, 1)
    up = _state(desc, u0, 2)
    ctx = Context(desc)
    ctx.set_solution(u)
    ctx.set_prev_solution(up)
    ctx.set_time_step(250.0)
    ctx.assemble_jacobian_and_residual()
    _, _, J = ctx.jacobian()
    _, _, Jo, ro = oracle.assemble(desc, u, up, 250.0)
    r = ctx.residual()
    assert np.max(np.abs(r - ro)) <= 1e-12 * np.max(np.abs(ro))
    J = J.reshape(-1, 2, 2)
    Jo = Jo.reshape(-1, 2, 2)
    tol = 1e-12 if analytic else 1e-7      # numeric differences amplify pow's last-ulp differences
    for pv in range(2):
        scale = np.max(np.abs(Jo[:, :, pv]))
        assert np.max(np.abs(J[:, :, pv] - Jo[:, :, pv])) <= tol * scale


def _gpu_time_loop(desc, u0, precision="fp64"):
    ctx = Context(desc, precision=precision)
    ctx.set_solution(u0)
    ctx.set_prev_solution(u0)
    p = newton_params()
    t, dt, times, iters = 0.0, 250.0, [], []
    while True:
        rep = ctx.newton_solve(dt, p)
        t += rep["dt_used"]
        ctx.advance_time_step()
        times.append(t)
        iters.append(rep["iterations"])
        if 3000.0 - t <= 1e-9 * 3000.0:
            return ctx.solution(), times, iters
        dt = min(ctx.suggest_time_step(rep["dt_used"], p), 3000.0 - t)


@pytest.mark.parametrize("analytic,precision", [(True, "fp64"), (False, "fp64"), (True, "mixed")])
def test_lens_case_end_to_end(analytic, precision):
    desc, u0 = problems.twop_lens_problem(analytic=analytic)
    u, times, iters = _gpu_time_loop(desc, u0, precision)
    uo, reps = oracle.time_loop(desc, u0, 250.0, 100, newton_params(), t_end=3000.0)
    assert len(times) == 7 and abs(times[4] - 2054.01) < 5e-3
    if precision == "fp64":
        assert iters == [r["iterations"] for r in reps]
        assert np.max(np.abs(u - uo)) <= 1e-9 * np.max(np.abs(uo))
    else:
        assert np.max(np.abs(u - uo)) <= 1e-6 * np.max(np.abs(uo))
    g = np.loadtxt(os.path.join(GOLDEN, "twop_lens_tpfa.txt"))
    u = u.reshape(-1, 2)
    assert np.max(np.abs(u[:, 0] - g[:, 1]) / np.abs(g[:, 1])) <= 2e-5
    mask = np.abs(g[:, 0]) > 1e-2 * np.max(g[:, 0])
    assert np.max(np.abs(u[mask, 1] - g[mask, 0]) / g[mask, 0]) <= 1e-4


def test_lens_case_in_a_batch_equals_alone():
    desc, u0 = problems.twop_lens_problem(analytic=True)
    batch = Batch(precision="mixed")
    pid = batch.add(desc, u0, dt=250.0, t_end=3000.0, params=newton_params(), max_dt=0.0)
    batch.run()
    u, _, _ = _gpu_time_loop(desc, u0, "mixed")
    assert batch.info(pid)["time_steps"] == 7
    assert np.array_equal(batch.solution(pid), u)


def test_partial_reassembly_matches_oracle():
    """Newton.EnablePartialReassembly on the device follows the oracle (same colors, same
    iteration counts) and still reproduces the reference's golden VTU."""
    desc, u0 = problems.twop_lens_problem(analytic=False)
    p = newton_params(enable_partial_reassembly=1)
    ctx = Context(desc)
    ctx.set_solution(u0)
    ctx.set_prev_solution(u0)
    t, dt, iters = 0.0, 250.0, []
    while True:
        rep = ctx.newton_solve(dt, p)
        t += rep["dt_used"]
        ctx.advance_time_step()
        iters.append(rep["iterations"])
        if 3000.0 - t <= 3e-6:
            break
        dt = min(ctx.suggest_time_step(rep["dt_used"], p), 3000.0 - t)
    uo, reps = oracle.time_loop(desc, u0, 250.0, 100, p, t_end=3000.0)
    assert iters == [r["iterations"] for r in reps]
    u = ctx.solution()
    assert np.max(np.abs(u - uo)) <= 1e-9 * np.max(np.abs(uo))
