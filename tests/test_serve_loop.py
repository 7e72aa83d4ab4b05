"""The served loop's host logic on the CPU (dumux_gb300.serve.Server.serve) over a fake
engine: arrival replay, admission in arrival order under the memory budget, release of
finished problems, latency and throughput records.  The engine itself (batching, budget
check, Newton and time loops) is native and tested on the GPU."""
import pytest

from dumux_gb300.serve import Server, percentile


class FakeDesc:
    def __init__(self, cells):
        self.num_cells = cells


class FakeBatch:
    """Admits while the summed cell count stays within `budget`; a problem finishes after
    `iterations` engine iterations; each iterate() advances the fake clock by `tick`."""

    def __init__(self, budget, iterations, clock, tick=0.01):
        self.budget, self.iterations, self.clock, self.tick = budget, iterations, clock, tick
        self.live, self.next_id, self.admitted, self.removed = {}, 1, [], []

    def add(self, desc, u0, dt, t_end, params):
        if sum(c for c, _ in self.live.values()) + desc.num_cells > self.budget:
            return None
        pid = self.next_id
        self.next_id += 1
        self.live[pid] = [desc.num_cells, 0]
        self.admitted.append(u0)
        return pid

    def iterate(self):
        self.clock.t += self.tick
        for v in self.live.values():
            v[1] += 1
        return sum(1 for v in self.live.values() if v[1] < self.iterations)

    def info(self, pid):
        cells, it = self.live[pid]
        done = it >= self.iterations
        return {"state": "finished" if done else "active", "status": 0, "time_steps": 2,
                "newton_iterations": it}

    def remove(self, pid):
        self.removed.append(pid)
        del self.live[pid]


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t


def _server(batch):
    s = Server.__new__(Server)   # no device: the engine is replaced by the fake
    s.batch, s.params = batch, None
    return s


def _requests(n, cells, gap):
    return [{"index": k, "kind": "2p", "arrival": k * gap, "dt": 250.0, "t_end": 500.0, "cells": cells[k]}
            for k in range(n)]


def test_admission_in_arrival_order_under_the_budget():
    clock = FakeClock()
    batch = FakeBatch(budget=100, iterations=3, clock=clock)
    reqs = _requests(5, [60, 30, 50, 10, 40], 0.0)
    records, stats = _server(batch).serve(reqs, lambda r: (FakeDesc(r["cells"]), r["index"]), clock=clock)
    # all requests arrive at once; admission keeps arrival order and waits for memory
    assert batch.admitted == [0, 1, 2, 3, 4]
    assert stats["requests"] == 5 and stats["finished"] == 5 and stats["failed"] == 0
    assert sorted(batch.removed) == [1, 2, 3, 4, 5]
    first = {r["index"]: r for r in records}
    # 60 + 30 fit, 50 waits until the first two finish after 3 iterations
    assert first[0]["admitted"] == 0.0 and first[1]["admitted"] == 0.0
    assert first[2]["admitted"] > first[0]["finished"] - 1e-12
    for r in records:
        assert r["latency"] == pytest.approx(r["finished"] - r["arrival"])
        assert r["cell_newton_steps"] == r["cells"] * r["newton_iterations"]
    assert stats["latency_p50_s"] == pytest.approx(percentile([r["latency"] for r in records], 50))
    assert stats["cell_newton_steps_per_s"] == pytest.approx(
        sum(r["cell_newton_steps"] for r in records) / stats["makespan_s"])


def test_arrivals_are_replayed_in_time():
    clock = FakeClock()
    batch = FakeBatch(budget=1000, iterations=2, clock=clock, tick=0.05)
    reqs = _requests(3, [10, 10, 10], 0.1)   # arrivals at 0.0, 0.1, 0.2
    records, stats = _server(batch).serve(reqs, lambda r: (FakeDesc(r["cells"]), r["index"]), clock=clock)
    by = {r["index"]: r for r in records}
    for k in range(3):
        assert by[k]["admitted"] >= by[k]["arrival"] - 1e-12
    assert stats["engine_iterations"] >= 2


def test_a_request_larger_than_the_budget_alone_is_an_error():
    clock = FakeClock()
    batch = FakeBatch(budget=10, iterations=1, clock=clock)
    with pytest.raises(RuntimeError, match="alone exceeds the memory budget"):
        _server(batch).serve(_requests(1, [20], 0.0), lambda r: (FakeDesc(r["cells"]), r["index"]), clock=clock)
