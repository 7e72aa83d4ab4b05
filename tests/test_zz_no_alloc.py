"""dxg_norm2_noalloc: the allocation-free Euclidean norm, against dxg_residual_norm.

Collected last on purpose (file name): if it fails, a run that stops at the first
failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from dumux_gb300 import Context, problems

pytestmark = pytest.mark.gpu

MAX_ENTRIES = 4096 * 256 * 8


def test_norm_without_allocation_matches_residual_norm(gpu_lib):
    torch = pytest.importorskip("torch")
    f = gpu_lib.dxg_norm2_noalloc
    f.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    desc, u0 = problems.dnapl_2p(cells=(20, 16, 12), seed=7)
    ctx = Context(desc)
    u = u0.reshape(-1, 2).copy()
    u[:, 1] = np.random.default_rng(3).uniform(0.0, 0.5, len(u))
    ctx.set_solution(u.reshape(-1))
    ctx.set_prev_solution(u0)
    ctx.set_time_step(250.0)
    ctx.assemble_residual()
    expected = ctx.residual_norm()           # the existing entry point
    r = ctx.residual()
    x = torch.tensor(r, dtype=torch.float64, device="cuda:0")
    out = torch.empty(1, dtype=torch.float64, device="cuda:0")
    stream = torch.cuda.current_stream(0).cuda_stream
    for _ in range(2):                       # two calls in a row share the scratch
        out.fill_(-1.0)
        assert f(x.data_ptr(), x.numel(), out.data_ptr(), stream) == 0
        torch.cuda.synchronize()
        got = float(out.item())
        assert got == pytest.approx(expected, rel=1e-12)
        assert got == pytest.approx(float(np.linalg.norm(r)), rel=1e-12)
    # a length beyond the fixed scratch is refused before any launch
    assert f(x.data_ptr(), MAX_ENTRIES + 1, out.data_ptr(), stream) == 11   # DXG_ERR_SIZE


def test_norm_without_allocation_edges_and_no_device_memory_taken(gpu_lib):
    """The longest vector the fixed scratch covers (4096 blocks, the last one summing all
    partials), the empty vector, and no device memory taken by the calls."""
    torch = pytest.importorskip("torch")
    f = gpu_lib.dxg_norm2_noalloc
    f.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    stream = torch.cuda.current_stream(0).cuda_stream
    host = np.random.default_rng(11).uniform(-1.0, 1.0, MAX_ENTRIES)
    x = torch.tensor(host, dtype=torch.float64, device="cuda:0")
    out = torch.empty(1, dtype=torch.float64, device="cuda:0")
    assert f(x.data_ptr(), MAX_ENTRIES, out.data_ptr(), stream) == 0   # warm-up (module load, address look-up)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(0)
    alloc0 = torch.cuda.memory_allocated(0)
    for _ in range(3):
        out.fill_(-1.0)
        assert f(x.data_ptr(), MAX_ENTRIES, out.data_ptr(), stream) == 0
        torch.cuda.synchronize()
        assert float(out.item()) == pytest.approx(float(np.linalg.norm(host)), rel=1e-12)
    out.fill_(-1.0)
    assert f(x.data_ptr(), 0, out.data_ptr(), stream) == 0
    torch.cuda.synchronize()
    assert float(out.item()) == 0.0
    free1, _ = torch.cuda.mem_get_info(0)
    assert free1 == free0 and torch.cuda.memory_allocated(0) == alloc0
