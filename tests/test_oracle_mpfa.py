"""The MPFA-O restatement of the oracle against the reference's own MPFA tests.

* test/porousmediumflow/1p/incompressible, test_1p_incompressible_mpfa (CMakeLists.txt:41-51):
  the MPFA-O lens solution is compared with the same reference file as the TPFA test
  (test_1p_cc-reference.vtu): with an isotropic permeability on a Cartesian grid the
  O-method's face systems decouple and give the two-point fluxes;
* test/porousmediumflow/1p/convergence/analyticsolution, test_1p_convergence_analytic_mpfa_
  structured (CMakeLists.txt, convergencetest.py): a full permeability tensor and an analytic
  solution; the L2 error over refinements 10, 20, 40, 80 must converge at a mean rate >= 1.8;
* the O-method's consistency: a linear pressure field with a constant full tensor is
  reproduced exactly (its residual vanishes), also on non-uniform tensor grids.
"""
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN
from dumux_gb300 import newton_params, problems


def _load(name):
    return np.array([float(v) for v in open(os.path.join(GOLDEN, name)).read().split("\n")[1:] if v.strip()])


def _linear_step(desc, u0, reduction=1e-13):
    row_ptr, col, vals, r = oracle.assemble(desc, u0)
    st, dx, res = oracle.linear_solve(row_ptr, col, vals, r, 1, reduction=reduction, max_iter=2000)
    assert st == 0 and res.converged
    return u0 - dx, (row_ptr, col, vals, r)


def test_mpfa_lens_matches_reference_vtu_and_tpfa():
    ref = _load("onep_lens_p.txt")
    desc, u0 = problems.onep_lens_problem(numeric_epsilon=True, discretization="mpfa")
    p, (row_ptr, col, _, r) = _linear_step(desc, u0)
    assert np.max(np.abs(p - ref)) <= 0.5 + 1e-9     # Float32 printed with 6 digits
    # the 3x3 stencil of every interior cell
    assert row_ptr[-1] == sum(min(i + 2, 10) - max(i - 1, 0) for i in range(10)) ** 2
    dt, ut = problems.onep_lens_problem(numeric_epsilon=True)
    pt, _ = _linear_step(dt, ut)
    assert np.max(np.abs(p - pt)) <= 1e-9 * np.max(np.abs(pt))


def test_mpfa_convergence_rate_of_the_reference_analytic_problem():
    p = newton_params(min_steps=1, max_steps=1, max_relative_shift=1e300, linear_reduction=1e-12,
                      max_time_step_divisions=0, linear_max_iter=2000)
    errs, dofs = [], []
    for cells in (10, 20, 40, 80):
        desc, u0, exact = problems.mpfa_convergence_problem(cells)
        st, u, rep = oracle.newton_solve(desc, u0, u0, 0.0, p)
        assert st == 0
        h = 1.0 / cells
        errs.append(np.sqrt(np.sum(h * h * (u - exact) ** 2)))
        dofs.append(cells * cells)
    rates = [np.log(errs[i] / errs[i + 1]) / np.log(np.sqrt(dofs[i + 1] / dofs[i])) for i in range(3)]
    assert np.mean(rates) >= 1.8, rates          # convergencetest.py: mean rate >= 1.8
    assert errs[0] < 1e-2


@pytest.mark.parametrize("cells,K", [((6, 5), ((2.0, 0.5), (0.5, 1.0))),
                                     ((5, 4, 3), ((2.0, 0.3, 0.1), (0.3, 1.0, 0.2), (0.1, 0.2, 1.5)))])
@pytest.mark.parametrize("seed", [None, 3])
def test_mpfa_reproduces_linear_pressure_fields(cells, K, seed):
    desc, u0, exact = problems.mpfa_linear_field_problem(cells=cells, K=K, spacing_seed=seed)
    _, _, vals, r_exact = oracle.assemble(desc, exact)
    scale = np.max(np.abs(vals)) * np.max(np.abs(exact))
    assert np.max(np.abs(r_exact)) <= 1e-13 * scale
    # Newton from zero lands on the linear field
    p = newton_params(max_relative_shift=1e-12, linear_reduction=1e-14, linear_max_iter=2000)
    st, u, rep = oracle.newton_solve(desc, u0, u0, 0.0, p)
    assert st == 0
    assert np.max(np.abs(u - exact)) <= 1e-9 * np.max(np.abs(exact))


def test_mpfa_gravity_neumann_and_source_are_consistent():
    """3D, gravity, a Neumann side and a source: the numeric Jacobian against central
    differences of the residual column by column, and the linear solve's residual."""
    rng = np.random.default_rng(4)
    cells = (4, 3, 3)
    desc, u0, _ = problems.mpfa_linear_field_problem(cells=cells, K=((2.0, 0.3, 0.1), (0.3, 1.0, 0.2),
                                                                       (0.1, 0.2, 1.5)), gravity=True,
                                                      spacing_seed=5)
    desc.bc_type[:12] = 2                       # -x side Neumann
    desc.bc_values[:12] = rng.uniform(-1e-3, 1e-3, 12)
    desc.source = rng.uniform(-1e-2, 1e-2, desc.num_cells)
    u = 1e5 + rng.uniform(-1e3, 1e3, desc.num_cells)
    row_ptr, col, vals, r = oracle.assemble(desc, u)
    J = np.zeros((desc.num_cells, desc.num_cells))
    for i in range(desc.num_cells):
        J[i, col[row_ptr[i]:row_ptr[i + 1]]] = vals[row_ptr[i]:row_ptr[i + 1]]
    for j in range(desc.num_cells):
        e = np.zeros_like(u)
        e[j] = 1.0
        rp = oracle.assemble(desc, u + e, jacobian=False)
        rm = oracle.assemble(desc, u - e, jacobian=False)
        # a linear residual: central differences of step 1 are exact up to rounding; the forward
        # difference of the assembler (eps = 1e-10 (|p| + 1)) carries the residual's rounding
        np.testing.assert_allclose(J[:, j], (rp - rm) / 2.0, rtol=1e-4, atol=1e-6 * np.max(np.abs(J)))
    # one linear step removes the residual up to the forward difference's accuracy; Newton
    # iterations (the residual is exactly linear) drive it to rounding
    p1, _ = _linear_step(desc, u, reduction=1e-14)
    r1 = oracle.assemble(desc, p1, jacobian=False)
    assert np.max(np.abs(r1)) <= 1e-4 * np.max(np.abs(r))
    prm = newton_params(max_relative_shift=1e-12, linear_reduction=1e-14, linear_max_iter=2000, max_steps=30)
    st, un, rep = oracle.newton_solve(desc, u, u, 0.0, prm)
    assert st == 0
    rn = oracle.assemble(desc, un, jacobian=False)
    assert np.max(np.abs(rn)) <= 1e-10 * np.max(np.abs(r))


def test_mpfa_analytic_jacobian_equals_numeric_differences():
    """The analytic Jacobian of the incompressible 1p MPFA-O residual (transmissibility times
    density / viscosity) against central differences of the residual; the lens with it (the
    reference test's own configuration) against the reference file."""
    desc, u0, _ = problems.mpfa_linear_field_problem(cells=(5, 4, 3), K=((2.0, 0.3, 0.1), (0.3, 1.0, 0.2),
                                                                         (0.1, 0.2, 1.5)), gravity=True,
                                                      spacing_seed=5)
    desc.bc_type[:12] = 2
    u = 1e5 + np.random.default_rng(9).uniform(-1e3, 1e3, desc.num_cells)
    desc.analytic = True
    row_ptr, col, va, r = oracle.assemble(desc, u)
    desc.analytic = False
    desc.numeric_difference_method = 0
    _, _, vn, rn = oracle.assemble(desc, u)
    assert np.array_equal(r, rn)
    np.testing.assert_allclose(va, vn, rtol=1e-5, atol=1e-6 * np.max(np.abs(va)))
    ref = _load("onep_lens_p.txt")
    dl, ul = problems.onep_lens_problem(numeric_epsilon=True, discretization="mpfa")
    dl.analytic = True
    p, _ = _linear_step(dl, ul)
    assert np.max(np.abs(p - ref)) <= 0.5 + 1e-9


def test_mpfa_2p_lens_matches_reference_vtu():
    """test/porousmediumflow/2p/incompressible, test_2p_incompressible_mpfa (CMakeLists.txt:
    93-102): the 2p lens with MPFA-O against the same reference file as the TPFA test, to its
    print precision; with isotropic cell permeabilities the O-method's fluxes are the
    two-point ones, so Newton takes the TPFA run's iterations."""
    from test_oracle_vangenuchten import _compare_with_golden
    desc, u0 = problems.twop_lens_problem(analytic=False)
    desc.discretization = 1
    u, reps = oracle.time_loop(desc, u0, 250.0, 100, newton_params(), t_end=3000.0)
    times = [r["time"] for r in reps]
    assert len(times) == 7 and abs(times[-1] - 3000.0) < 1e-6 and abs(times[4] - 2054.01) < 5e-3
    err_p, err_s, small = _compare_with_golden(u)
    assert err_p <= 2e-5 and err_s <= 1e-4 and small <= 1e-6, (err_p, err_s, small)
    dt, ut = problems.twop_lens_problem(analytic=False)
    ut_end, reps_t = oracle.time_loop(dt, ut, 250.0, 100, newton_params(), t_end=3000.0)
    assert [r["iterations"] for r in reps] == [r["iterations"] for r in reps_t]
    assert np.max(np.abs(u - ut_end)) <= 1e-9 * np.max(np.abs(ut_end))


@pytest.mark.parametrize("cells", [(6, 5), (4, 3, 3)])
def test_mpfa_2p_jacobian_equals_central_differences(cells):
    """2p with a rotated anisotropic tensor, gravity, Dirichlet and Neumann faces, a
    transient storage term: the Jacobian columns against forward differences of larger steps
    wherever the residual is smooth (two step sizes agree: upwind switches at near-zero
    fluxes make it kinked), and Newton from the previous state converging superlinearly."""
    desc, u0 = problems.dnapl_2p_mpfa(cells=cells, seed=3)
    u = u0.reshape(-1, 2).copy()
    u[:, 1] = np.random.default_rng(4).uniform(0.05, 0.5, len(u))
    u = u.reshape(-1)
    row_ptr, col, vals, r = oracle.assemble(desc, u, u0, 250.0)
    n = desc.num_dofs
    J = np.zeros((n, n))
    for i in range(desc.num_cells):
        for k in range(row_ptr[i], row_ptr[i + 1]):
            J[2 * i:2 * i + 2, 2 * col[k]:2 * col[k] + 2] = vals[4 * k:4 * k + 4].reshape(2, 2)
    checked = 0
    for j in range(n):
        cols = []
        # forward differences (the side of the assembler's own perturbation: a flux that is
        # zero at u makes the residual kinked there) with two step sizes
        for h in ((1e-4, 1e-5) if j % 2 == 0 else (1e-8, 1e-9)):
            e = np.zeros(n)
            e[j] = h
            rp = oracle.assemble(desc, u + e, u0, 250.0, jacobian=False)
            cols.append((rp - r) / h)
        scale = np.max(np.abs(J[:, j])) + 1e-300
        smooth = np.abs(cols[0] - cols[1]) <= 1e-4 * scale
        np.testing.assert_allclose(J[smooth, j], cols[1][smooth], rtol=1e-3, atol=1e-5 * scale)
        checked += int(np.count_nonzero(smooth & (J[:, j] != 0)))
    assert checked > 0.5 * np.count_nonzero(J)
    p = newton_params(max_relative_shift=1e-10)
    st, un, rep = oracle.newton_solve(desc, u0, u0, 250.0, p)
    assert st == 0 and rep["iterations"] <= 8
    sh = rep["shift"][:rep["iterations"]]
    assert sh[-1] <= 1e-10 and sh[-1] < 1e-3 * sh[-3]
