"""The C ABI library builds for sm_103a, loads, and exports every declared symbol."""
import ctypes as C
import os
import re

import pytest

from conftest import ROOT


def _declared(header):
    txt = open(os.path.join(ROOT, "include", header)).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(dxg_\w+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(gpu_lib):
    names = _declared("dumux_gb300.h")
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(gpu_lib, n)]
    assert not missing, missing


def test_context_creation_fails_loudly_without_gpu(gpu_lib):
    import dumux_gb300
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = os.path.exists("/dev/nvidia0")
    if has_gpu:
        pytest.skip("a GPU is present")
    with pytest.raises(dumux_gb300.DxgError) as e:
        dumux_gb300.Context()
    assert e.value.status == 10   # DXG_ERR_NO_DEVICE


def test_boundary_face_count(gpu_lib):
    from dumux_gb300 import problems
    from dumux_gb300.abi import num_boundary_faces
    desc, _ = problems.dnapl_2p(cells=(5, 4, 3))
    d = desc.c
    gpu_lib.dxg_num_boundary_faces.restype = C.c_int64
    assert gpu_lib.dxg_num_boundary_faces(C.byref(d)) == num_boundary_faces(3, [5, 4, 3]) == 2 * (12 + 15 + 20)


def test_batch_creation_fails_loudly_without_gpu(gpu_lib):
    import dumux_gb300
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = os.path.exists("/dev/nvidia0")
    if has_gpu:
        pytest.skip("a GPU is present")
    with pytest.raises(dumux_gb300.DxgError) as e:
        dumux_gb300.Batch()
    assert e.value.status == 10   # DXG_ERR_NO_DEVICE


def test_problem_device_bytes_scales_with_cells(gpu_lib):
    """Admission sizes: host-only arithmetic, ~linear in cells; the mixed form holds FP32
    copies of the Jacobian and factors beside the FP64 Jacobian and Krylov vectors."""
    from dumux_gb300 import problem_device_bytes, problems
    small, _ = problems.dnapl_2p(cells=(8, 8, 8))
    large, _ = problems.dnapl_2p(cells=(16, 16, 16))
    one_p, _ = problems.darcy_1p(cells=(20, 20))
    s_mixed = problem_device_bytes(small, "mixed")
    l_mixed = problem_device_bytes(large, "mixed")
    assert s_mixed > problem_device_bytes(small, "fp64") > 0
    assert 6.0 < (l_mixed - 64 * 1024) / (s_mixed - 64 * 1024) < 8.5
    # 2p cells need more state than 1p cells
    assert problem_device_bytes(one_p, "mixed") < s_mixed
    # at least the Jacobian (7 blocks of 2x2 doubles) per cell
    assert s_mixed > 512 * 7 * 4 * 8
