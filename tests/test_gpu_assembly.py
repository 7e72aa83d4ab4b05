"""Device residual and numeric-difference Jacobian against the CPU oracle."""
import numpy as np
import pytest

import oracle
from dumux_gb300 import Context, problems

pytestmark = pytest.mark.gpu


def _random_2p_state(desc, u0, seed, sn_max=0.9):
    rng = np.random.default_rng(seed)
    u = u0.reshape(-1, 2).copy()
    u[:, 0] += rng.uniform(-2e3, 2e3, len(u))
    u[:, 1] = rng.uniform(0.0, sn_max, len(u))
    # hit the regularised branches too
    u[::7, 1] = 0.0
    u[3::11, 1] = 0.96
    return u.reshape(-1)


def _cases():
    out = []
    d, u0 = problems.onep_lens_problem()
    rng = np.random.default_rng(0)
    out.append(("1p-lens-2d", d, u0 + 1e5 + rng.uniform(-5e4, 5e4, u0.size), None, 0.0))
    d, u0 = problems.darcy_1p(cells=(7, 6, 5), seed=3, enable_gravity=True)
    d.source = np.random.default_rng(1).uniform(-1e-3, 1e-3, d.num_dofs)
    up = u0 + 10.0
    out.append(("1p-3d-transient-source", d, u0 + rng.uniform(-1e3, 1e3, u0.size), up, 50.0))
    for dims, name in [((12, 8), "2p-2d"), ((6, 5, 4), "2p-3d")]:
        d, u0 = problems.dnapl_2p(cells=dims, extent=(6.0, 4.0, 1.0)[:len(dims)], seed=5)
        u = _random_2p_state(d, u0, 7)
        up = _random_2p_state(d, u0, 8)
        out.append((name, d, u, up, 250.0))
    return out


CASES = _cases()


@pytest.fixture(params=[oracle.POW_CORRECTLY_ROUNDED, oracle.POW_LIBM], ids=["crpow", "libm"])
def pow_mode(request):
    """The oracle's pow: the correctly rounded one (the device's) or the C library's (the
    reference's std::pow, not correctly rounded in ~0.1% of arguments)."""
    with oracle.pow_mode(request.param):
        yield request.param


def _compare(desc, u, up, dt):
    ctx = Context(desc)
    ctx.set_solution(u)
    if up is not None:
        ctx.set_prev_solution(up)
    ctx.set_time_step(dt)
    ctx.assemble_jacobian_and_residual()
    r_gpu = ctx.residual()
    row_ptr, col, vals = ctx.jacobian()
    orow, ocol, ovals, r_orc = oracle.assemble(desc, u, up, dt)
    assert np.array_equal(row_ptr, orow) and np.array_equal(col, ocol)
    return r_gpu, r_orc, vals, ovals


@pytest.mark.parametrize("name,desc,u,up,dt", CASES, ids=[c[0] for c in CASES])
def test_residual_and_jacobian_match_oracle(name, desc, u, up, dt, pow_mode):
    r_gpu, r_orc, J_gpu, J_orc = _compare(desc, u, up, dt)
    b = desc.num_eq
    if b == 1 or pow_mode == oracle.POW_CORRECTLY_ROUNDED:
        # identical operation sequence and the same pow -> identical bits
        assert np.array_equal(r_gpu, r_orc)
        assert np.array_equal(J_gpu, J_orc)
        return
    # the C library's pow differs from the correctly rounded one by an ulp in ~0.1% of
    # the arguments; the numeric derivative divides such an ulp by epsilon ~1e-10
    assert np.max(np.abs(r_gpu - r_orc)) <= 1e-13 * np.max(np.abs(r_orc))
    assert np.max(np.abs(J_gpu - J_orc)) <= 1e-7 * np.max(np.abs(J_orc))


@pytest.mark.parametrize("method", [1, -1, 0, 5])
def test_numeric_difference_methods(method):
    # forward, backward, central differences and the five-point stencil
    # (NumericDifferentiation::partialDerivative, dumux/common/numericdifferentiation.hh:67-123)
    d, u0 = problems.dnapl_2p(cells=(5, 4, 3), seed=9)
    d.numeric_difference_method = method
    u = _random_2p_state(d, u0, 3)
    with oracle.pow_mode(oracle.POW_CORRECTLY_ROUNDED):
        r_gpu, r_orc, J_gpu, J_orc = _compare(d, u, u, 100.0)
    assert np.array_equal(r_gpu, r_orc)
    assert np.array_equal(J_gpu, J_orc)


def test_residual_only_equals_full_assembly():
    d, u0 = problems.dnapl_2p(cells=(6, 5, 4), seed=11)
    u = _random_2p_state(d, u0, 4)
    ctx = Context(d)
    ctx.set_solution(u)
    ctx.set_prev_solution(u0)
    ctx.set_time_step(250.0)
    ctx.assemble_jacobian_and_residual()
    r1 = ctx.residual()
    ctx.assemble_residual()
    assert np.array_equal(r1, ctx.residual())
