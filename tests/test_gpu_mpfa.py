"""MPFA-O on the device against the oracle and the reference's MPFA tests.

The host tabulation (interaction-volume systems) and the oracle follow the same operation
order, and the device evaluates the scvf fluxes and the numeric-difference Jacobian in the
oracle's order without FMA contraction: residual and Jacobian are compared bit for bit.
"""
import numpy as np
import pytest

import oracle
from dumux_gb300 import Context, newton_params, problems
from test_oracle_mpfa import _load

pytestmark = pytest.mark.gpu


def _cases():
    rng = np.random.default_rng(7)
    out = []
    d, u = problems.onep_lens_problem(numeric_epsilon=True, discretization="mpfa")
    out.append(("lens-2d-gravity", d, 1e5 + rng.uniform(-1e3, 1e3, d.num_cells)))
    d, u, _ = problems.mpfa_convergence_problem(12)
    out.append(("tensor-2d-source", d, 10.0 + rng.uniform(-1, 1, d.num_cells)))
    d, u, _ = problems.mpfa_linear_field_problem(cells=(5, 4, 3), K=((2.0, 0.3, 0.1), (0.3, 1.0, 0.2),
                                                                     (0.1, 0.2, 1.5)), gravity=True, spacing_seed=5)
    d.bc_type[:12] = 2
    d.bc_values[:12] = rng.uniform(-1e-3, 1e-3, 12)
    d.source = rng.uniform(-1e-2, 1e-2, d.num_cells)
    d.extrusion = rng.uniform(0.5, 2.0, d.num_cells)
    out.append(("tensor-3d-gravity-neumann", d, 1e5 + rng.uniform(-1e3, 1e3, d.num_cells)))
    return out


@pytest.mark.parametrize("name,desc,u", _cases(), ids=lambda v: v if isinstance(v, str) else "")
@pytest.mark.parametrize("method", [1, 0, -1, 5, "analytic"])
def test_mpfa_residual_and_jacobian_equal_the_oracle(name, desc, u, method):
    desc.analytic = method == "analytic"
    desc.numeric_difference_method = 1 if method == "analytic" else method
    ctx = Context(desc)
    ctx.set_solution(u)
    ctx.assemble_jacobian_and_residual()
    row_ptr, col, vals = ctx.jacobian()
    orow, ocol, ovals, r_orc = oracle.assemble(desc, u)
    assert np.array_equal(row_ptr, orow) and np.array_equal(col, ocol)
    assert np.array_equal(ctx.residual(), r_orc)
    assert np.array_equal(vals, ovals)


@pytest.mark.parametrize("analytic", [False, True])
def test_mpfa_lens_on_the_device_matches_reference_vtu(analytic):
    # the reference's test_1p_incompressible_mpfa assembles the analytic Jacobian
    ref = _load("onep_lens_p.txt")
    desc, u0 = problems.onep_lens_problem(numeric_epsilon=True, discretization="mpfa")
    desc.analytic = analytic
    ctx = Context(desc)
    ctx.set_solution(u0)
    ctx.assemble_jacobian_and_residual()
    res = ctx.linear_solve(1e-13, 500)
    assert res["converged"]
    p = u0 - ctx.update()
    assert np.max(np.abs(p - ref)) <= 0.5 + 1e-9
    orow, ocol, ovals, r = oracle.assemble(desc, u0)
    st, dx, ores = oracle.linear_solve(orow, ocol, ovals, r, 1, reduction=1e-13, max_iter=500)
    assert np.max(np.abs(p - (u0 - dx))) <= 1e-9 * np.max(np.abs(p))


def test_mpfa_convergence_rate_on_the_device():
    p = newton_params(min_steps=1, max_steps=1, max_relative_shift=1e300, linear_reduction=1e-12,
                      max_time_step_divisions=0, linear_max_iter=2000)
    errs = []
    for cells in (10, 20, 40, 80):
        desc, u0, exact = problems.mpfa_convergence_problem(cells)
        ctx = Context(desc)
        ctx.set_solution(u0)
        ctx.set_prev_solution(u0)
        rep = ctx.newton_solve(0.0, p)
        u = ctx.solution()
        st, uo, _ = oracle.newton_solve(desc, u0, u0, 0.0, p)
        assert st == 0 and np.max(np.abs(u - uo)) <= 1e-9 * np.max(np.abs(uo))
        h = 1.0 / cells
        errs.append(np.sqrt(np.sum(h * h * (u - exact) ** 2)))
    rates = [np.log2(errs[i] / errs[i + 1]) for i in range(3)]
    assert np.mean(rates) >= 1.8, rates


def test_mpfa_newton_3d_linear_field_and_oracle_iterations():
    desc, u0, exact = problems.mpfa_linear_field_problem(cells=(9, 7, 6), K=((2.0, 0.3, 0.1), (0.3, 1.0, 0.2),
                                                                             (0.1, 0.2, 1.5)), spacing_seed=2)
    p = newton_params(max_relative_shift=1e-12, linear_reduction=1e-13, linear_max_iter=2000, max_steps=30)
    ctx = Context(desc)
    ctx.set_solution(u0)
    ctx.set_prev_solution(u0)
    rep = ctx.newton_solve(0.0, p)
    assert rep["converged"]
    assert np.max(np.abs(ctx.solution() - exact)) <= 1e-9 * np.max(np.abs(exact))
    st, uo, orep = oracle.newton_solve(desc, u0, u0, 0.0, p)
    assert st == 0 and orep["iterations"] == rep["iterations"]
    assert "MPFA-O" in ctx.describe()


@pytest.mark.parametrize("cells", [(40, 40), (37, 70), (20, 9), (200, 300), (30, 600), (12, 1100)])
def test_mpfa_line_sweeps_equal_level_kernel(cells):
    """The 2D line sweeps, in one CTA (warp shuffles and a barrier per level) and over a
    cluster (four warps per CTA, up to nine CTAs here, point-to-point hand-offs), and the
    level-by-level kernel compute the same preconditioner bit for bit."""
    desc, u0, _ = problems.mpfa_convergence_problem(cells[0])
    if cells[0] != cells[1]:
        desc, u0, _ = problems.mpfa_linear_field_problem(cells=cells, spacing_seed=1)
    out = {}
    for kind in ("lanes", "wavefront", "levels"):
        ctx = Context(desc)
        ctx.set_ilu_kernel(kind)
        ctx.set_solution(u0)
        ctx.assemble_jacobian_and_residual()
        res = ctx.linear_solve(1e-12, 3000)
        assert res["converged"]
        out[kind] = (res["iterations"], ctx.update(), ctx.describe())
    assert "over a cluster" in out["lanes"][2] and "level by level" in out["levels"][2]
    if cells[1] <= 1024:
        assert "in one CTA" in out["wavefront"][2]
    for kind in ("lanes", "wavefront"):
        assert out[kind][0] == out["levels"][0]
        assert np.array_equal(out[kind][1], out["levels"][1])


@pytest.mark.parametrize("b,cells", [(1, (9, 7, 5)), (1, (6, 40, 3)), (1, (5, 5, 16)), (1, (4, 3, 20)),
                                     (2, (8, 6, 5)), (2, (6, 20, 4)), (2, (10, 40, 3)), (2, (32, 32, 16))])
def test_mpfa_3d_line_sweeps_equal_level_kernel(b, cells):
    """The 3D sweeps over a cluster (one z-plane per CTA, one lane per grid line and block
    row; (6, 40, 3) and (6, 20, 4) with b = 2 hand line histories between warps, (5, 5, 16) fills
    a 16-CTA cluster) and the level-by-level kernel compute the same preconditioner bit for
    bit; with more than 16 planes the sweeps fall back to the level kernel."""
    if b == 1:
        K = ((2.0, 0.3, 0.1), (0.3, 1.0, 0.2), (0.1, 0.2, 1.5))
        desc, u0, _ = problems.mpfa_linear_field_problem(cells=cells, K=K, spacing_seed=3)
        u = u0
    else:
        desc, u0 = problems.dnapl_2p_mpfa(cells=cells, seed=5)
        u = u0.reshape(-1, 2).copy()
        u[:, 1] = np.random.default_rng(4).uniform(0, 0.4, len(u))
        u = u.reshape(-1)
    out = {}
    for kind in ("lanes", "levels"):
        ctx = Context(desc)
        ctx.set_ilu_kernel(kind)
        ctx.set_solution(u)
        ctx.set_prev_solution(u0)
        if b == 2:
            ctx.set_time_step(250.0)
        ctx.assemble_jacobian_and_residual()
        res = ctx.linear_solve(1e-12, 3000)
        assert res["converged"]
        out[kind] = (res["iterations"], ctx.update(), ctx.describe())
    assert "level by level" in out["levels"][2]
    if cells[2] <= 16:
        assert "one z-plane per CTA" in out["lanes"][2]
    else:
        assert "level by level" in out["lanes"][2]
    assert out["lanes"][0] == out["levels"][0]
    assert np.array_equal(out["lanes"][1], out["levels"][1])


@pytest.mark.parametrize("b,cells", [(1, (9, 7, 5)), (2, (8, 6, 5)), (2, (5, 40, 4))])
def test_mpfa_3d_linear_solve_matches_oracle(b, cells):
    """ILU(0)-BiCGSTAB on a 3D MPFA-O Jacobian: the cluster factorisation (one warp per row of
    a level) and the cluster sweeps against the oracle's SeqILU + BiCGSTAB on the same matrix."""
    if b == 1:
        K = ((2.0, 0.3, 0.1), (0.3, 1.0, 0.2), (0.1, 0.2, 1.5))
        desc, u0, _ = problems.mpfa_linear_field_problem(cells=cells, K=K, spacing_seed=2)
        u = u0
    else:
        desc, u0 = problems.dnapl_2p_mpfa(cells=cells, seed=6)
        u = u0.reshape(-1, 2).copy()
        u[:, 1] = np.random.default_rng(9).uniform(0, 0.4, len(u))
        u = u.reshape(-1)
    ctx = Context(desc)
    ctx.set_solution(u)
    ctx.set_prev_solution(u0)
    if b == 2:
        ctx.set_time_step(250.0)
    ctx.assemble_jacobian_and_residual()
    res = ctx.linear_solve(1e-13, 1000)
    assert res["converged"] and "one z-plane per CTA" in ctx.describe()
    x = ctx.update()
    row_ptr, col, vals = ctx.jacobian()
    st, xo, ores = oracle.linear_solve(row_ptr, col, vals, ctx.residual(), b, reduction=1e-13, max_iter=1000)
    assert st == 0
    assert np.max(np.abs(x - xo)) <= 1e-8 * np.max(np.abs(xo))
    assert abs(res["iterations"] - ores.iterations) <= max(2, 0.1 * ores.iterations)


def test_mpfa_3d_cluster_sweep_wait_limit_expires_and_recovers():
    """The 3D cluster sweeps under a 1 us wait limit give up (each plane waits for the plane
    before far longer), the solve reports DXG_ERR_TIMEOUT, and with the limit restored the same
    context solves to the same bits."""
    desc, u0 = problems.dnapl_2p_mpfa(cells=(16, 16, 12), seed=5)
    ctx = Context(desc)
    ctx.set_ilu_kernel("lanes")
    ctx.set_solution(u0)
    ctx.set_prev_solution(u0)
    ctx.set_time_step(250.0)
    ctx.assemble_jacobian_and_residual()
    first = ctx.linear_solve(1e-12, 3000)
    assert first["converged"] and "one z-plane per CTA" in ctx.describe()
    x0 = ctx.update()
    ctx.set_wait_limit(1e-6)
    with pytest.raises(Exception, match="timed out"):
        ctx.linear_solve(1e-12, 3000)
    ctx.set_wait_limit(0.5)
    again = ctx.linear_solve(1e-12, 3000)
    assert again["iterations"] == first["iterations"] and np.array_equal(ctx.update(), x0)


def test_mpfa_cluster_sweep_wait_limit_expires_and_recovers():
    """A 1 us wait limit: the cluster line sweeps give up (later warps wait for their
    neighbours' first results far longer), the solve reports DXG_ERR_TIMEOUT, and with the
    limit restored the same context solves to the same bits."""
    desc, u0, _ = problems.mpfa_convergence_problem(300)
    ctx = Context(desc)
    ctx.set_ilu_kernel("lanes")
    ctx.set_solution(u0)
    ctx.assemble_jacobian_and_residual()
    first = ctx.linear_solve(1e-12, 3000)
    assert first["converged"] and "over a cluster" in ctx.describe()
    x0 = ctx.update()
    ctx.set_wait_limit(1e-6)
    with pytest.raises(Exception, match="timed out"):
        ctx.linear_solve(1e-12, 3000)
    ctx.set_wait_limit(0.5)
    again = ctx.linear_solve(1e-12, 3000)
    assert again["iterations"] == first["iterations"] and np.array_equal(ctx.update(), x0)


@pytest.mark.parametrize("cells", [(1, 7), (7, 1), (1, 1), (2, 2), (1, 1, 3), (3, 1, 1), (2, 1, 2)])
def test_mpfa_degenerate_grids(cells):
    """Grids of one or two cells per axis: interaction volumes with one, two or four cells,
    every face a boundary face on some axis."""
    K = ((2.0, 0.5), (0.5, 1.0)) if len(cells) == 2 else ((2.0, 0.3, 0.1), (0.3, 1.0, 0.2), (0.1, 0.2, 1.5))
    desc, u0, exact = problems.mpfa_linear_field_problem(cells=cells, K=K)
    u = exact + 0.25
    ctx = Context(desc)
    ctx.set_solution(u)
    ctx.assemble_jacobian_and_residual()
    row_ptr, col, vals = ctx.jacobian()
    orow, ocol, ovals, r_orc = oracle.assemble(desc, u)
    assert np.array_equal(row_ptr, orow) and np.array_equal(col, ocol)
    assert np.array_equal(vals, ovals) and np.array_equal(ctx.residual(), r_orc)
    p = newton_params(max_relative_shift=1e-12, linear_reduction=1e-14, linear_max_iter=500, max_steps=30)
    ctx.set_solution(u0)
    ctx.set_prev_solution(u0)
    assert ctx.newton_solve(0.0, p)["converged"]
    assert np.max(np.abs(ctx.solution() - exact)) <= 1e-12 * np.max(np.abs(exact))


@pytest.fixture
def _cr_pow():
    prev = oracle.get_pow_mode()
    oracle.set_pow_mode(oracle.POW_CORRECTLY_ROUNDED)
    yield
    oracle.set_pow_mode(prev)


@pytest.mark.parametrize("cells", [(7, 5), (5, 4, 3)])
@pytest.mark.parametrize("method", [1, 0, -1, 5])
def test_mpfa_2p_residual_and_jacobian_equal_the_oracle(cells, method, _cr_pow):
    """2p MPFA-O with a rotated anisotropic tensor, gravity, Dirichlet and Neumann faces and
    the storage term: the device residual and Jacobian blocks bit for bit."""
    desc, u0 = problems.dnapl_2p_mpfa(cells=cells, seed=5)
    desc.numeric_difference_method = method
    u = u0.reshape(-1, 2).copy()
    u[:, 1] = np.random.default_rng(6).uniform(0.0, 0.5, len(u))
    u[:, 0] += np.random.default_rng(7).uniform(-100.0, 100.0, len(u))
    u = u.reshape(-1)
    ctx = Context(desc)
    ctx.set_solution(u)
    ctx.set_prev_solution(u0)
    ctx.set_time_step(250.0)
    ctx.assemble_jacobian_and_residual()
    row_ptr, col, vals = ctx.jacobian()
    orow, ocol, ovals, r_orc = oracle.assemble(desc, u, u0, 250.0)
    assert np.array_equal(row_ptr, orow) and np.array_equal(col, ocol)
    assert np.array_equal(ctx.residual(), r_orc)
    assert np.array_equal(vals, ovals)


def test_mpfa_2p_newton_matches_oracle(_cr_pow):
    desc, u0 = problems.dnapl_2p_mpfa(cells=(9, 6, 4), seed=8)
    p = newton_params(linear_reduction=1e-13, linear_max_iter=1000)
    ctx = Context(desc)
    ctx.set_solution(u0)
    ctx.set_prev_solution(u0)
    reps = []
    dt = 250.0
    for _ in range(3):
        reps.append(ctx.newton_solve(dt, p))
        ctx.advance_time_step()
        dt = min(ctx.suggest_time_step(reps[-1]["dt_used"], p), 250.0)
    u_orc, oreps = oracle.time_loop(desc, u0, 250.0, 3, params=p, max_dt=250.0)
    assert [r["iterations"] for r in reps] == [r["iterations"] for r in oreps]
    uo, ug = u_orc.reshape(-1, 2), ctx.solution().reshape(-1, 2)
    assert np.max(np.abs(ug[:, 0] - uo[:, 0])) <= 1e-9 * np.max(np.abs(uo[:, 0]))
    assert np.max(np.abs(ug[:, 1] - uo[:, 1])) <= 1e-9 * max(1e-3, np.max(np.abs(uo[:, 1])))
    assert np.max(uo[:, 1]) > 1e-3


def test_mpfa_2p_lens_on_the_device_matches_reference_vtu():
    """test_2p_incompressible_mpfa on the device: the lens to t = 3000 s against the
    reference file."""
    from test_oracle_vangenuchten import _compare_with_golden
    desc, u0 = problems.twop_lens_problem(analytic=False)
    desc.discretization = 1
    p = newton_params()
    ctx = Context(desc)
    ctx.set_solution(u0)
    ctx.set_prev_solution(u0)
    t, dt, times = 0.0, 250.0, []
    while t < 3000.0 - 1e-9:
        rep = ctx.newton_solve(dt, p)
        t += rep["dt_used"]
        times.append(t)
        ctx.advance_time_step()
        dt = min(ctx.suggest_time_step(rep["dt_used"], p), 3000.0 - t)
    assert len(times) == 7 and abs(times[4] - 2054.01) < 5e-3
    err_p, err_s, small = _compare_with_golden(ctx.solution())
    assert err_p <= 2e-5 and err_s <= 1e-4 and small <= 1e-6, (err_p, err_s, small)
