"""The numpy restatements that check the red-black ILU(0) and the AMG solver variants on the
GPU, pinned on the CPU: inside the same BiCGSTAB iteration they solve the oracle's
assembled system to the oracle's own ILU(0)-BiCGSTAB solution, and they need no more
iterations than it (the property that makes the variants worth having on the device)."""
import numpy as np
import pytest

import oracle
from dumux_gb300 import problems

import test_gpu_amg as amg
import test_gpu_redblack as rb


def _system(dims, seed):
    d, u0 = problems.dnapl_2p(cells=dims, extent=(6.0, 4.0, 1.0)[:len(dims)], seed=seed)
    u = u0.reshape(-1, 2).copy()
    u[:, 1] = np.random.default_rng(seed).uniform(0, 0.5, len(u))
    row_ptr, col, vals, r = oracle.assemble(d, u.reshape(-1), u0, 250.0)
    st, x_ilu, res = oracle.linear_solve(row_ptr, col, vals, r, 2, reduction=1e-10, max_iter=1000)
    assert st == 0 and res.converged
    return d, row_ptr, col, vals, r, x_ilu, res.iterations


@pytest.mark.parametrize("dims", [(11, 9), (12, 9, 7), (21, 13, 6)])
def test_amg_restatement_solves_the_oracle_system(dims):
    d, row_ptr, col, vals, r, x_ilu, it_ilu = _system(dims, 7)
    A = amg._csr(d, row_ptr, col, vals)
    it, x = amg._bicgstab(A, amg._Amg(A, d.cells[:d.dim], 2), r, 1e-10, 1000)
    assert it > 0
    assert it <= it_ilu
    assert np.max(np.abs(x - x_ilu)) <= 1e-7 * np.max(np.abs(x_ilu))


@pytest.mark.parametrize("dims", [(11, 9), (12, 9, 7)])
def test_redblack_restatement_solves_the_oracle_system(dims):
    d, row_ptr, col, vals, r, x_ilu, it_ilu = _system(dims, 8)
    A, mask, offs = rb._slots(d, row_ptr, col, vals)
    it, x = rb._bicgstab(A, mask, offs, rb._redblack(d, A, mask, offs), r.reshape(-1, 2), 1e-10, 1000)
    assert it > 0
    assert np.max(np.abs(x.reshape(-1) - x_ilu)) <= 1e-7 * np.max(np.abs(x_ilu))
