"""VTU output and restart (VtkOutputModule / loadSolution wire format): round trip, and
the reference's restart test replayed on the oracle -- restart the 2p lens case from the
output at t = 2054.01 s with dt 603.14 s (test/porousmediumflow/2p/incompressible/
CMakeLists.txt:30-40) and compare the end state with the golden VTU (fuzzy, 1e-2)."""
import os

import numpy as np

import oracle
from conftest import GOLDEN
from dumux_gb300 import newton_params, problems
from dumux_gb300.vtu import load_solution, read_vtu, write_vtu


def test_roundtrip_float64_and_float32(tmp_path):
    desc, u0 = problems.dnapl_2p(cells=(5, 4, 3), seed=1)
    u = u0.copy().reshape(-1, 2)
    u[:, 1] = np.linspace(0.0, 0.7, len(u))
    u = u.reshape(-1)
    write_vtu(tmp_path / "a.vtu", desc, u, precision="Float64")
    assert np.array_equal(load_solution(tmp_path / "a.vtu", desc), u)
    write_vtu(tmp_path / "b.vtu", desc, u)
    v = load_solution(tmp_path / "b.vtu", desc)
    assert np.max(np.abs(v - u) / np.maximum(np.abs(u), 1e-30)) <= 6e-8
    f = read_vtu(tmp_path / "b.vtu")
    assert set(f) == {"S_aq", "p_aq", "S_napl"}
    d1, p1 = problems.darcy_1p(cells=(6, 4), seed=1)
    write_vtu(tmp_path / "c.vtu", d1, p1, extra={"K": d1.permeability}, precision="Float64")
    assert np.array_equal(load_solution(tmp_path / "c.vtu", d1), p1)


def test_cell_order_and_connectivity(tmp_path):
    desc, u0 = problems.dnapl_2p(cells=(3, 2), extent=(6.0, 4.0), seed=1)
    write_vtu(tmp_path / "g.vtu", desc, u0)
    txt = open(tmp_path / "g.vtu").read()
    assert 'NumberOfCells="6" NumberOfPoints="12"' in txt
    # first cell (0,0): vertices 0, 1, 5, 4 of the 4 x 3 vertex grid (x fastest)
    assert "0 1 5 4 1 2 6 5" in txt


def test_restart_replays_reference_restart_test(tmp_path):
    desc, u0 = problems.twop_lens_problem(analytic=True)
    p = newton_params()
    u5, reps = oracle.time_loop(desc, u0, 250.0, 5, p, t_end=3000.0)
    t5 = reps[-1]["time"]
    assert abs(t5 - 2054.01) < 5e-3
    write_vtu(tmp_path / "lens-00005.vtu", desc, u5)              # Float32, as the reference
    ur = load_solution(tmp_path / "lens-00005.vtu", desc)
    u, reps2 = oracle.time_loop(desc, ur, 603.14, 100, p, t_end=3000.0 - t5)
    assert len(reps2) == 2                                        # output 2 of the restart run
    g = np.loadtxt(os.path.join(GOLDEN, "twop_lens_tpfa.txt"))
    u = u.reshape(-1, 2)
    assert np.max(np.abs(u[:, 0] - g[:, 1]) / np.abs(g[:, 1])) <= 1e-2
    mask = np.abs(g[:, 0]) > 1e-2 * np.max(g[:, 0])
    assert np.max(np.abs(u[mask, 1] - g[mask, 0]) / g[mask, 0]) <= 1e-2
