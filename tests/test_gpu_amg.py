"""AMG-preconditioned BiCGSTAB (DXG_LINEAR_SOLVER_AMG_BICGSTAB) against a numpy
restatement of the same V-cycle, and Newton with it against the oracle's fields.

The restatement is test infrastructure: 2x2(x2) box aggregates until a level has at most
64 cells, Galerkin coarse operators P^T A P with piecewise-constant P, damped block
Jacobi (omega 0.8; one sweep, two on levels of at most 4096 cells), the exact solve of
the last level, inside the device solver's BiCGSTAB iteration.
"""
import numpy as np
import pytest
import scipy.sparse as sp

import oracle
from dumux_gb300 import Context, newton_params, problems

pytestmark = pytest.mark.gpu

OMEGA, SMALL, SMALL_SWEEPS, COARSEST = 0.8, 4096, 2, 64


def _csr(desc, row_ptr, col, vals):
    b, n = desc.num_eq, desc.num_cells
    return sp.bsr_matrix((np.asarray(vals).reshape(-1, b, b), col, row_ptr), shape=(n * b, n * b)).tocsr()


def _prolongation(dims, b):
    n = int(np.prod(dims))
    idx = np.arange(n)
    coords, rem = [], idx.copy()
    for d in dims:
        coords.append(rem % d)
        rem //= d
    cd = [(d + 1) // 2 for d in dims]
    agg, mul = np.zeros_like(idx), 1
    for c, d in zip(coords, cd):
        agg += (c // 2) * mul
        mul *= d
    rows = (idx[:, None] * b + np.arange(b)).ravel()
    cols = (agg[:, None] * b + np.arange(b)).ravel()
    return sp.csr_matrix((np.ones(len(rows)), (rows, cols)), shape=(n * b, int(np.prod(cd)) * b)), cd


def _dinv(A, b):
    n = A.shape[0] // b
    D = np.zeros((n, b, b))
    for r in range(b):
        for c in range(b):
            D[:, r, c] = A[np.arange(n) * b + r, np.arange(n) * b + c].A1
    return np.linalg.inv(D)


class _Amg:
    def __init__(self, A, dims, b):
        self.b = b
        self.levels = []
        dims = list(dims) + [1] * (3 - len(dims))
        while True:
            n = int(np.prod(dims))
            sweeps = SMALL_SWEEPS if n <= SMALL else 1
            if n <= COARSEST:
                self.levels.append((A, np.linalg.inv(A.toarray()), None, sweeps))
                break
            P, cd = _prolongation(dims, b)
            self.levels.append((A, _dinv(A, b), P, sweeps))
            A, dims = (P.T @ A @ P).tocsr(), cd

    def _d(self, D, v):
        return np.einsum("nij,nj->ni", D, v.reshape(-1, self.b)).ravel()

    def _v(self, l, rhs):
        A, D, P, sweeps = self.levels[l]
        if P is None:
            return D @ rhs
        x = OMEGA * self._d(D, rhs)
        for _ in range(sweeps - 1):
            x = x + OMEGA * self._d(D, rhs - A @ x)
        xc = self._v(l + 1, P.T @ (rhs - A @ x))
        x = x + P @ xc
        for _ in range(sweeps):
            x = x + OMEGA * self._d(D, rhs - A @ x)
        return x

    def __call__(self, r):
        return self._v(0, r)


def _bicgstab(A, M, rhs, reduction, max_iter):
    x = np.zeros_like(rhs)
    r = rhs.copy()
    rt = r.copy()
    p = np.zeros_like(r)
    v = np.zeros_like(r)
    rho = alpha = omega = 1.0
    d0 = np.linalg.norm(r)
    for it in range(1, max_iter + 1):
        rho_new = rt @ r
        p = r.copy() if it == 1 else r + (rho_new / rho) * (alpha / omega) * (p - omega * v)
        y = M(p)
        v = A @ y
        alpha = rho_new / (rt @ v)
        x += alpha * y
        r -= alpha * v
        if np.linalg.norm(r) < reduction * d0:
            return it, x
        z = M(r)
        t = A @ z
        omega = (t @ r) / (t @ t)
        x += omega * z
        r -= omega * t
        if np.linalg.norm(r) < reduction * d0:
            return it, x
        rho = rho_new
    return -1, x


@pytest.mark.parametrize("dims", [(9, 7), (13, 10, 6), (20, 17, 9), (33, 21)])
def test_amg_solve_matches_restatement(dims):
    d, u0 = problems.dnapl_2p(cells=dims, extent=(6.0, 4.0, 1.0)[:len(dims)], seed=3)
    u = u0.reshape(-1, 2).copy()
    u[:, 1] = np.random.default_rng(5).uniform(0, 0.5, len(u))
    ctx = Context(d)
    ctx.set_linear_solver("amg")
    ctx.set_solution(u.reshape(-1))
    ctx.set_prev_solution(u0)
    ctx.set_time_step(250.0)
    ctx.assemble_jacobian_and_residual()
    res = ctx.linear_solve(1e-10, 500)
    assert res["converged"]
    assert "AMG" in ctx.describe()
    x = ctx.update()
    row_ptr, col, vals = ctx.jacobian()
    A = _csr(d, row_ptr, col, vals)
    r = ctx.residual()
    it, xr = _bicgstab(A, _Amg(A, d.cells[:d.dim], 2), r, 1e-10, 500)
    assert it > 0
    assert abs(res["iterations"] - it) <= 1
    assert np.max(np.abs(x - xr)) <= 1e-8 * np.max(np.abs(xr))
    assert np.linalg.norm(r - A @ x) <= 1e-9 * np.linalg.norm(r)


def test_amg_onep_lens_matches_ilu_solution():
    desc, u0 = problems.onep_lens_problem(numeric_epsilon=True)
    out = {}
    for kind in ("ilu", "amg"):
        ctx = Context(desc)
        ctx.set_linear_solver(kind)
        ctx.set_solution(u0)
        ctx.assemble_jacobian_and_residual()
        res = ctx.linear_solve(1e-13, 250)
        assert res["converged"]
        out[kind] = (res["iterations"], ctx.update())
    assert out["amg"][0] < out["ilu"][0]
    assert np.max(np.abs(out["amg"][1] - out["ilu"][1])) <= 1e-9 * np.max(np.abs(out["ilu"][1]))


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-7), ("mixed", 1e-6)])
def test_newton_with_amg_matches_oracle_fields(precision, tol):
    desc, u0 = problems.dnapl_2p(cells=(10, 8, 6), seed=4, inflow=0.04)
    p = newton_params(linear_reduction=1e-13, linear_max_iter=500)
    u_orc, _ = oracle.time_loop(desc, u0, 250.0, 3, params=p, max_dt=250.0)
    pr = newton_params(linear_reduction=1e-6 if precision == "mixed" else 1e-10, linear_max_iter=500)
    ctx = Context(desc, precision=precision)
    ctx.set_linear_solver("amg")
    ctx.set_solution(u0)
    ctx.set_prev_solution(u0)
    for _ in range(3):
        rep = ctx.newton_solve(250.0, pr)
        assert rep["converged"]
        ctx.advance_time_step()
    u = ctx.solution().reshape(-1, 2)
    uo = u_orc.reshape(-1, 2)
    err = np.max(np.abs(u - uo), axis=0) / np.max(np.abs(uo), axis=0)
    assert np.all(err <= tol), err


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_amg_batch_equals_single_problems(precision):
    """DXG_BATCH_OPT_AMG: uneven grids (different level counts) in one batch, each result
    bit-identical to the same problem alone in a context with AMG-BiCGSTAB."""
    from dumux_gb300 import Batch
    params = newton_params(linear_max_iter=500)
    cases = [((8, 6, 5), 11, 0.5), ((24, 20, 12), 12, 2.0), ((7, 9, 4), 13, 1.2), ((30, 22), 15, 1.0),
             ((40, 33, 17), 16, 1.5)]
    batch = Batch(precision=precision, solver="amg")
    ids = []
    for cells, seed, sigma in cases:
        desc, u0 = problems.dnapl_2p(cells=cells, extent=(6.0, 4.0, 1.0)[:len(cells)], seed=seed, sigma=sigma,
                                     corr_len=4.0)
        ids.append((batch.add(desc, u0, dt=250.0, t_end=500.0, params=params), desc, u0))
    batch.run()
    assert "AMG" in batch.describe()
    for pid, desc, u0 in ids:
        info = batch.info(pid)
        assert info["state"] == "finished"
        ctx = Context(desc, precision=precision)
        ctx.set_linear_solver("amg")
        ctx.set_solution(u0)
        ctx.set_prev_solution(u0)
        t, iters, dt = 0.0, 0, 250.0
        while t < 500.0 - 1e-6:
            rep = ctx.newton_solve(dt, params)
            iters += rep["iterations"] + rep["wasted_iterations"]
            t += rep["dt_used"]
            ctx.advance_time_step()
            dt = min(ctx.suggest_time_step(rep["dt_used"], params), 250.0, 500.0 - t)
        assert info["newton_iterations"] == iters
        assert np.array_equal(batch.solution(pid), ctx.solution()), desc.cells


def test_amg_continuous_batching_mixed_kinds_equal_alone():
    """AMG batches with requests of different kinds (1p 2D stationary, 2p 2D and 3D
    transient) admitted while others are in flight: each result equals the one computed
    alone with AMG-BiCGSTAB."""
    from dumux_gb300 import Batch
    params = newton_params(linear_max_iter=500)
    first = [problems.dnapl_2p(cells=(9, 7, 5), seed=21, corr_len=4.0) + (250.0, 500.0),
             problems.darcy_1p(cells=(30, 26), seed=22, corr_len=3.0) + (0.0, 0.0)]
    later = [problems.dnapl_2p(cells=(20, 14), extent=(6.0, 4.0), seed=24, corr_len=4.0) + (100.0, 300.0),
             problems.darcy_1p(cells=(9, 14), seed=25, corr_len=2.0) + (0.0, 0.0)]
    batch = Batch(precision="mixed", solver="amg")
    admitted = []
    for desc, u0, dt, t_end in first:
        admitted.append((batch.add(desc, u0, dt=dt, t_end=t_end, params=params), desc, u0, dt, t_end))
    batch.iterate()
    for desc, u0, dt, t_end in later:
        admitted.append((batch.add(desc, u0, dt=dt, t_end=t_end, params=params), desc, u0, dt, t_end))
    while batch.iterate() > 0:
        pass
    for pid, desc, u0, dt, t_end in admitted:
        info = batch.info(pid)
        assert info["state"] == "finished", (desc.cells, info)
        ctx = Context(desc, precision="mixed")
        ctx.set_linear_solver("amg")
        ctx.set_solution(u0)
        ctx.set_prev_solution(u0)
        if t_end <= 0.0:
            ctx.newton_solve(0.0, params)
        else:
            t, cur = 0.0, min(dt, t_end)
            while t_end - t > 1e-9 * t_end:
                rep = ctx.newton_solve(cur, params)
                t += rep["dt_used"]
                ctx.advance_time_step()
                cur = min(ctx.suggest_time_step(rep["dt_used"], params), dt, t_end - t)
        assert np.array_equal(batch.solution(pid), ctx.solution()), (desc.cells, desc.num_eq)
