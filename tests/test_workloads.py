"""The benchmark workload generators (CPU): seeded, deterministic, and drawn from the
distributions the workloads state (grid extents, parameter ranges, arrival process)."""
import numpy as np

from dumux_gb300 import problems


def test_ensemble_is_seeded_and_within_its_ranges():
    a = problems.ensemble_2p(count=6, seed=4)
    b = problems.ensemble_2p(count=6, seed=4)
    for (da, ua, ma), (db, ub, mb) in zip(a, b):
        assert ma == mb
        assert np.array_equal(da.permeability, db.permeability) and np.array_equal(ua, ub)
        assert all(16 <= n <= 64 for n in ma["cells"])
        assert da.num_cells == int(np.prod(ma["cells"])) and da.num_eq == 2
        assert 0.5 <= ma["sigma"] <= 2.0 and 3.0 <= ma["corr_len"] <= 10.0 and 0.01 <= ma["inflow"] <= 0.08
    assert len({m["cells"] for _, _, m in a}) > 1            # uneven grids


def test_served_stream_arrivals_mix_and_sizes():
    reqs = problems.served_requests(400, rate=200.0, seed=5)
    t = np.array([r["arrival"] for r in reqs])
    assert np.all(np.diff(t) > 0)
    assert abs(np.mean(np.diff(t)) - 1.0 / 200.0) < 0.25 / 200.0        # Poisson, mean 200/s
    frac_1p = np.mean([r["kind"] == "1p" for r in reqs])
    assert 0.2 < frac_1p < 0.4
    for r in reqs:
        n = r["cells"][0]
        assert r["cells"] == (n, n, n) and 10 <= n <= 100
        assert 1 <= r["steps"] <= 20 and r["t_end"] == r["steps"] * r["dt"]
    assert problems.served_requests(5, seed=5) == problems.served_requests(5, seed=5)


def test_request_problems_have_their_kind_and_grid():
    reqs = problems.served_requests(40, seed=7, n_max=2e4)
    one = next(r for r in reqs if r["kind"] == "1p")
    two = next(r for r in reqs if r["kind"] == "2p")
    d1, u1 = problems.make_request_problem(one)
    d2, u2 = problems.make_request_problem(two)
    assert d1.num_eq == 1 and tuple(d1.cells[:3]) == one["cells"] and len(u1) == d1.num_cells
    assert d2.num_eq == 2 and tuple(d2.cells[:3]) == two["cells"] and len(u2) == 2 * d2.num_cells


def test_lnk_field_has_the_stated_mean_and_spread():
    f = problems.gaussian_lnk_field((96, 96), mean=np.log(1e-10), sigma=1.0, corr_len=4.0, seed=3)
    assert abs(np.mean(f) - np.log(1e-10)) < 0.3
    assert 0.7 < np.std(f) < 1.3
