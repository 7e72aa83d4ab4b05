"""Red-black ordered ILU(0) (DXG_ILU_REDBLACK) against a numpy restatement, and Newton
with it against the FP64 oracle's natural-order fields.

The red-black preconditioner is not the reference's (SeqILU factors the matrix in its
natural order); it is this library's option for throughput.  The restatement below is
test infrastructure: D_r = A_rr, D_b = A_bb - sum_r A_br D_r^-1 A_rb, and a sweep pair
v_b = D_b^-1 (d_b - sum_r A_br D_r^-1 d_r), v_r = D_r^-1 (d_r - sum_b A_rb v_b), inside
the same BiCGSTAB iteration (half-step convergence tests) as the device solver.
"""
import numpy as np
import pytest

import oracle
from dumux_gb300 import Context, newton_params, problems

pytestmark = pytest.mark.gpu


def _slots(desc, row_ptr, col, vals):
    n, b = desc.num_cells, desc.num_eq
    nx, ny = desc.cells[0], desc.cells[1]
    offs = [-nx * ny, -nx, -1, 0, 1, nx, nx * ny] if desc.dim == 3 else [-nx, -1, 0, 1, nx]
    A = np.zeros((len(offs), n, b, b))
    mask = np.zeros((len(offs), n), bool)
    rows = np.repeat(np.arange(n), np.diff(row_ptr))
    V = np.asarray(vals).reshape(-1, b, b)
    for s, o in enumerate(offs):
        sel = (col - rows) == o
        A[s, rows[sel]] = V[sel]
        mask[s, rows[sel]] = True
    return A, mask, offs


def _matvec(A, mask, offs, x):
    y = np.zeros_like(x)
    for s, o in enumerate(offs):
        idx = np.nonzero(mask[s])[0]
        y[idx] += np.einsum("nij,nj->ni", A[s, idx], x[idx + o])
    return y


def _redblack(desc, A, mask, offs):
    n = desc.num_cells
    nx, ny = desc.cells[0], desc.cells[1]
    i = np.arange(n)
    color = (i % nx + (i // nx) % ny + i // (nx * ny)) % 2
    red, blk = np.nonzero(color == 0)[0], np.nonzero(color == 1)[0]
    c = len(offs) // 2
    Dinv = np.zeros_like(A[c])
    Dinv[red] = np.linalg.inv(A[c, red])
    D = A[c].copy()
    for s in range(len(offs)):
        if s == c:
            continue
        m = mask[s, blk]
        ci = blk[m]
        j = ci + offs[s]
        D[ci] -= A[s, ci] @ Dinv[j] @ A[len(offs) - 1 - s, j]
    Dinv[blk] = np.linalg.inv(D[blk])

    def apply(d):
        v = np.zeros_like(d)
        zb = d[blk].copy()
        for s in range(len(offs)):
            if s == c:
                continue
            m = mask[s, blk]
            ci = blk[m]
            j = ci + offs[s]
            zb[m] -= np.einsum("nij,nj->ni", A[s, ci], np.einsum("nij,nj->ni", Dinv[j], d[j]))
        v[blk] = np.einsum("nij,nj->ni", Dinv[blk], zb)
        zr = d[red].copy()
        for s in range(len(offs)):
            if s == c:
                continue
            m = mask[s, red]
            ci = red[m]
            j = ci + offs[s]
            zr[m] -= np.einsum("nij,nj->ni", A[s, ci], v[j])
        v[red] = np.einsum("nij,nj->ni", Dinv[red], zr)
        return v
    return apply


def _bicgstab(A, mask, offs, M, rhs, reduction, max_iter):
    x = np.zeros_like(rhs)
    r = rhs.copy()
    rt = r.copy()
    p = np.zeros_like(r)
    v = np.zeros_like(r)
    rho = alpha = omega = 1.0
    d0 = np.linalg.norm(r)
    for it in range(1, max_iter + 1):
        rho_new = np.sum(rt * r)
        p = r.copy() if it == 1 else r + (rho_new / rho) * (alpha / omega) * (p - omega * v)
        y = M(p)
        v = _matvec(A, mask, offs, y)
        alpha = rho_new / np.sum(rt * v)
        x += alpha * y
        r -= alpha * v
        if np.linalg.norm(r) < reduction * d0:
            return it, x
        z = M(r)
        t = _matvec(A, mask, offs, z)
        omega = np.sum(t * r) / np.sum(t * t)
        x += omega * z
        r -= omega * t
        if np.linalg.norm(r) < reduction * d0:
            return it, x
        rho = rho_new
    return -1, x


@pytest.mark.parametrize("dims", [(9, 7), (7, 6, 5), (12, 9, 8)])
def test_redblack_solve_matches_restatement(dims):
    d, u0 = problems.dnapl_2p(cells=dims, extent=(6.0, 4.0, 1.0)[:len(dims)], seed=3)
    u = u0.reshape(-1, 2).copy()
    u[:, 1] = np.random.default_rng(5).uniform(0, 0.5, len(u))
    ctx = Context(d)
    ctx.set_ilu_kernel("redblack")
    ctx.set_solution(u.reshape(-1))
    ctx.set_prev_solution(u0)
    ctx.set_time_step(250.0)
    ctx.assemble_jacobian_and_residual()
    res = ctx.linear_solve(1e-10, 1000)
    assert res["converged"]
    x = ctx.update()
    assert "red-black" in ctx.describe()
    row_ptr, col, vals = ctx.jacobian()
    A, mask, offs = _slots(d, row_ptr, col, vals)
    it, xr = _bicgstab(A, mask, offs, _redblack(d, A, mask, offs), ctx.residual().reshape(-1, 2), 1e-10, 1000)
    assert it > 0
    assert abs(res["iterations"] - it) <= 1
    assert np.max(np.abs(x - xr.reshape(-1))) <= 1e-8 * np.max(np.abs(xr))
    # the true residual of the device solution
    r = ctx.residual().reshape(-1, 2)
    rres = r - _matvec(A, mask, offs, x.reshape(-1, 2))
    assert np.linalg.norm(rres) <= 1e-9 * np.linalg.norm(r)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-7), ("mixed", 1e-6)])
def test_newton_with_redblack_matches_oracle_fields(precision, tol):
    desc, u0 = problems.dnapl_2p(cells=(10, 8, 6), seed=4, inflow=0.04)
    p = newton_params(linear_reduction=1e-13, linear_max_iter=500)
    u_orc, oreps = oracle.time_loop(desc, u0, 250.0, 3, params=p, max_dt=250.0)
    pr = newton_params(linear_reduction=1e-6 if precision == "mixed" else 1e-10, linear_max_iter=1000)
    ctx = Context(desc, precision=precision)
    ctx.set_ilu_kernel("redblack")
    ctx.set_solution(u0)
    ctx.set_prev_solution(u0)
    for _ in range(3):
        rep = ctx.newton_solve(250.0, pr)
        assert rep["converged"]
        ctx.advance_time_step()
    u = ctx.solution().reshape(-1, 2)
    uo = u_orc.reshape(-1, 2)
    scale = np.max(np.abs(uo), axis=0)
    err = np.max(np.abs(u - uo), axis=0) / scale
    assert np.all(err <= tol), err
    assert np.max(uo[:, 1]) > 1e-3


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_redblack_batch_equals_single_problems(precision):
    """DXG_BATCH_OPT_ILU_REDBLACK: uneven grids in one batch, each result bit-identical to
    the same problem alone in a context with the red-black ordering."""
    from dumux_gb300 import Batch
    params = newton_params(linear_max_iter=1000)
    cases = [((8, 6, 5), 11, 0.5), ((12, 10, 6), 12, 2.0), ((7, 9, 4), 13, 1.2), ((14, 11), 15, 1.0)]
    batch = Batch(precision=precision, ilu="redblack")
    ids = []
    for cells, seed, sigma in cases:
        desc, u0 = problems.dnapl_2p(cells=cells, extent=(6.0, 4.0, 1.0)[:len(cells)], seed=seed, sigma=sigma,
                                     corr_len=4.0)
        ids.append((batch.add(desc, u0, dt=250.0, t_end=500.0, params=params), desc, u0))
    batch.run()
    assert "red-black" in batch.describe()
    for pid, desc, u0 in ids:
        info = batch.info(pid)
        assert info["state"] == "finished"
        ctx = Context(desc, precision=precision)
        ctx.set_ilu_kernel("redblack")
        ctx.set_solution(u0)
        ctx.set_prev_solution(u0)
        t, iters = 0.0, 0
        dt = 250.0
        while t < 500.0 - 1e-6:
            rep = ctx.newton_solve(dt, params)
            iters += rep["iterations"] + rep["wasted_iterations"]
            t += rep["dt_used"]
            ctx.advance_time_step()
            dt = min(ctx.suggest_time_step(rep["dt_used"], params), 250.0, 500.0 - t)
        assert info["newton_iterations"] == iters
        assert np.array_equal(batch.solution(pid), ctx.solution()), desc.cells
