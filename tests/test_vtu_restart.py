"""VTU output and restart (VtkOutputModule / loadSolution wire format): round trip, and
the reference's restart test replayed on the oracle -- restart the 2p lens case from the
output at t = 2054.01 s with dt 603.14 s (test/porousmediumflow/2p/incompressible/
CMakeLists.txt:30-40) and compare the end state with the golden VTU (fuzzy, 1e-2)."""
import os

import numpy as np
import pytest

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


def _gpu_time_loop(desc, u0, dt, num_steps, params, t_end):
    """The oracle's time_loop on the device: TimeLoop semantics with the Newton solver's
    step-size suggestion, stopping at t_end."""
    from dumux_gb300 import Context
    ctx = Context(desc)
    ctx.set_solution(u0)
    ctx.set_prev_solution(u0)
    t, reps = 0.0, []
    for _ in range(num_steps):
        rep = ctx.newton_solve(dt, params)
        assert rep["converged"]
        ctx.advance_time_step()
        t += rep["dt_used"]
        rep["time"] = t
        reps.append(rep)
        if t >= t_end:
            break
        dt = min(ctx.suggest_time_step(rep["dt_used"], params), t_end - t)
    return ctx.solution(), reps


@pytest.mark.gpu
def test_gpu_restart_from_vtu_matches_oracle_replay(tmp_path):
    """The reference's restart test on the device: run the lens case to output 5, write it as
    the reference does (Float32 VTU), load it back (loadSolution by primary-variable names,
    dumux/io/loadsolution.hh:91-193), continue in a fresh context from t = 2054.01 s with
    dt 603.14 s, and compare with the oracle restarted from the same file and with the
    reference's golden output."""
    desc, u0 = problems.twop_lens_problem(analytic=True)
    p = newton_params()
    u5, reps = _gpu_time_loop(desc, u0, 250.0, 5, p, 3000.0)
    t5 = reps[-1]["time"]
    assert abs(t5 - 2054.01) < 5e-3
    write_vtu(tmp_path / "lens-00005.vtu", desc, u5)
    ur = load_solution(tmp_path / "lens-00005.vtu", desc)
    u_gpu, reps_gpu = _gpu_time_loop(desc, ur, 603.14, 100, p, 3000.0 - t5)
    u_orc, reps_orc = oracle.time_loop(desc, ur, 603.14, 100, p, t_end=3000.0 - t5)
    assert [r["iterations"] for r in reps_gpu] == [r["iterations"] for r in reps_orc]
    assert np.max(np.abs(u_gpu - u_orc)) <= 1e-9 * np.max(np.abs(u_orc))
    g = np.loadtxt(os.path.join(GOLDEN, "twop_lens_tpfa.txt"))
    u = u_gpu.reshape(-1, 2)
    assert np.max(np.abs(u[:, 0] - g[:, 1]) / np.abs(g[:, 1])) <= 1e-2
    mask = np.abs(g[:, 0]) > 1e-2 * np.max(g[:, 0])
    assert np.max(np.abs(u[mask, 1] - g[mask, 0]) / g[mask, 0]) <= 1e-2
