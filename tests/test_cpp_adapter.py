"""The C++ adapter (include/dumux_gb300.hh) compiles against the C ABI and drives a
DuMux-style problem class; on a GPU its solution equals the Python path's on the same
tabulated problem."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

SRC = os.path.join(ROOT, "tests", "cpp", "test_adapter.cc")
LIBDIR = os.path.join(ROOT, "dumux_gb300", "_lib")


def _build(tmp_path):
    exe = str(tmp_path / "test_adapter")
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
           f"-L{LIBDIR}", "-ldumux_gb300", f"-Wl,-rpath,{LIBDIR}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_adapter_compiles_and_links(gpu_lib, tmp_path):
    exe = _build(tmp_path)
    r = subprocess.run([exe, "6", "5", "4", "1", str(tmp_path / "u.bin")], capture_output=True, text=True)
    # without a GPU the adapter must fail loudly with DXG_ERR_NO_DEVICE, never fall back
    assert r.returncode in (0, 3), r.stderr
    if r.returncode == 3:
        assert r.stdout.strip() == "no-device"


@pytest.mark.gpu
def test_adapter_matches_python_path(gpu_lib, tmp_path):
    from dumux_gb300 import Context, newton_params, problems
    from dumux_gb300.abi import cell_centers
    exe = _build(tmp_path)
    cells, steps = (8, 6, 5), 2
    out = tmp_path / "u.bin"
    r = subprocess.run([exe, *map(str, cells), str(steps), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    u_cpp = np.fromfile(out, dtype=np.float64)
    # the same problem tabulated in Python: the adapter test's permeability polynomial
    coords = [problems.equidistant(0.0, e, n) for e, n in zip((6.0, 4.0, 1.0), cells)]
    cc = cell_centers(coords)
    K = 1e-11 * (1.0 + 0.3 * cc[:, 0] + 0.2 * cc[:, 1] * cc[:, 1] + 0.1 * cc[:, 2])
    desc, u0 = problems.dnapl_2p(cells=cells, lnk=np.log(K))
    desc.permeability = K
    ctx = Context(desc)
    ctx.set_solution(u0)
    ctx.set_prev_solution(u0)
    for _ in range(steps):
        ctx.newton_solve(250.0, newton_params())
        ctx.advance_time_step()
    u_py = ctx.solution()
    assert u_cpp.shape == u_py.shape
    assert np.max(np.abs(u_cpp - u_py)) <= 1e-12 * np.max(np.abs(u_py))
