"""The CPU oracle against the reference's own golden vectors and known-answer tests."""
import math
import os

import numpy as np
import pytest

import oracle
from dumux_gb300 import problems
from conftest import GOLDEN


def _load(name):
    return np.array([float(v) for v in open(os.path.join(GOLDEN, name)).read().split("\n")[1:] if v.strip()])


def test_onep_lens_matches_reference_vtu():
    # test/porousmediumflow/1p/incompressible (numdiff variant with params.input's
    # Assembly.NumericDifference.PriVarMagnitude = 1e5, BaseEpsilon = 0.1):
    # assembleJacobian, assembleResidual, one linear solve (reduction 1e-13 =
    # LinearSolverParameters default), x -= deltaX
    ref = _load("onep_lens_p.txt")
    desc, u0 = problems.onep_lens_problem(numeric_epsilon=True)
    row_ptr, col, vals, r = oracle.assemble(desc, u0)
    st, dx, res = oracle.linear_solve(row_ptr, col, vals, r, 1, reduction=1e-13)
    assert st == 0 and res.converged
    p = u0 - dx
    # the reference file stores Float32 printed with 6 significant digits
    assert np.max(np.abs(p - ref)) <= 0.5 + 1e-9
    # the residual of the solved linear problem vanishes
    r1 = oracle.assemble(desc, p, jacobian=False)
    assert np.linalg.norm(r1) < 1e-10 * np.linalg.norm(r)


def test_onep_lens_gravity_matters():
    # guards the gravity default (Problem.EnableGravity = true): without it the field
    # misses the golden file by far more than its print precision
    ref = _load("onep_lens_p.txt")
    desc, u0 = problems.onep_lens_problem()
    desc.enable_gravity = False
    row_ptr, col, vals, r = oracle.assemble(desc, u0)
    _, dx, _ = oracle.linear_solve(row_ptr, col, vals, r, 1)
    assert np.max(np.abs(u0 - dx - ref)) > 100.0


def test_brooks_corey_pc_matches_reference_dat():
    # test/material/fluidmatrixinteractions/2p/test_material_2p_brookscorey.cc:40-64
    ref = _load("pcsw_brookscorey.txt")
    n = 100
    delta = (1.0 - 0.0) / (n - 1)
    sw = np.array([0.0 + i * delta for i in range(n)])
    pc = oracle.brooks_corey([1e4, 2.0, 0.1, 0.1, 0.01], "pc", sw)
    assert np.max(np.abs(pc - ref) / np.abs(ref)) < 1e-13
    assert np.count_nonzero(pc == ref) >= 80


def test_brooks_corey_regularisation_branches():
    prm = [500.0, 2.0, 0.05, 0.0, 0.01]
    sw = np.array([0.0, 0.05, 0.0595, 0.5, 0.999, 1.0, 1.1])
    krw = oracle.brooks_corey(prm, "krw", sw)
    krn = oracle.brooks_corey(prm, "krn", sw)
    pc = oracle.brooks_corey(prm, "pc", sw)
    assert krw[0] == 0.0 and krw[-1] == 1.0 and krw[-2] == 1.0
    assert krn[0] == 1.0 and krn[-1] == 0.0
    assert pc[5] == 500.0            # entry pressure at swe = 1
    assert pc[6] < 500.0             # linear continuation above swe = 1
    assert np.all(np.diff(pc) < 0)   # strictly decreasing, no kink


def test_numeric_differentiation_known_answers():
    # test/common/numericdifferentiation/test_numericdifferentiation.cc:118-130
    base = math.sqrt(np.finfo(float).eps)
    dfunc = lambda x: 1.0 / 6.0 * x ** 3 + 0.5 * x * x + x + 1.0
    for method, eps, tol in [(1, base, 100 * base), (-1, base, 100 * base), (0, base, base),
                             (5, 1e6 * base, base * base)]:
        assert abs(oracle.numdiff_poly(method, eps, 1.0) - dfunc(1.0)) < tol


@pytest.mark.parametrize("line_search", [0, 1])
def test_newton_scalar_mock(line_search):
    # test/nonlinear/newton/test_newton.cc:31-111: x^2 - 5 = 0 from 0.1 to 1e-13
    st, x, it = oracle.newton_scalar(0.1, use_line_search=line_search)
    assert st == 0
    assert abs(x - math.sqrt(5.0)) <= 1e-13 * math.sqrt(5.0)
