"""Served form: a request loop with continuous batching on one GPU.

Requests (independent 1p / 2p problems with their own time loops) arrive over time.
The loop admits arrived requests in arrival order while the device-memory budget
allows (dxg_batch_add refuses with DXG_ERR_BUDGET beyond it), runs one Newton
iteration of every admitted problem per engine call (dxg_batch_iterate: problems of a
kind share each kernel launch), and releases a problem's device memory as soon as it
finishes, so waiting requests are admitted while others are still on the GPU.  State
stays on the device across a problem's time steps.

The engine (batching, admission check, per-problem Newton and time loop) is native
code in the CUDA library; this module only feeds it requests and keeps the clock.
"""
import time
from collections import deque

import numpy as np

from . import Batch, newton_params


def percentile(values, q):
    if not values:
        return None
    return float(np.percentile(np.asarray(values, dtype=np.float64), q))


class Server:
    """Continuous-batching request loop over one dxg_batch.

    memory_budget: bytes of device memory all admitted problems may hold (0: no limit).
    """

    def __init__(self, device=0, precision="mixed", memory_budget=0, params=None, graphs=True, autotune=True,
                 ilu="natural", solver="ilu"):
        self.batch = Batch(device=device, precision=precision, graphs=graphs, autotune=autotune,
                           memory_budget=memory_budget, ilu=ilu, solver=solver)
        default_iter = 1000 if ilu == "redblack" else 500
        self.params = params if params is not None else newton_params(linear_max_iter=default_iter)

    def serve(self, requests, problem_of, clock=time.perf_counter):
        """Serves `requests` (dicts with 'arrival' seconds from the start, 'dt', 't_end')
        whose problems `problem_of(req)` returns as (desc, u0).  Arrivals are replayed in
        real time.  Returns per-request records and summary statistics."""
        pending = deque(sorted(requests, key=lambda r: r["arrival"]))
        waiting = deque()
        active = {}
        records = []
        t0 = clock()
        iterations = 0
        while pending or waiting or active:
            now = clock() - t0
            while pending and pending[0]["arrival"] <= now:
                waiting.append(pending.popleft())
            # admit in arrival order while the budget allows
            while waiting:
                req = waiting[0]
                desc, u0 = problem_of(req)
                pid = self.batch.add(desc, u0, dt=req["dt"], t_end=req["t_end"], params=self.params)
                if pid is None:
                    if not active:
                        raise RuntimeError(f"request {req.get('index')} alone exceeds the memory budget")
                    break
                waiting.popleft()
                active[pid] = (req, desc.num_cells, clock() - t0)
            if not active:
                if pending:
                    time.sleep(max(0.0, pending[0]["arrival"] - (clock() - t0)))
                continue
            self.batch.iterate()
            iterations += 1
            done_at = clock() - t0
            for pid in list(active):
                info = self.batch.info(pid)
                if info["state"] == "active":
                    continue
                req, cells, admitted = active.pop(pid)
                records.append({
                    "index": req.get("index"), "kind": req.get("kind"), "cells": cells, "steps": info["time_steps"],
                    "state": info["state"], "status": info["status"], "arrival": req["arrival"],
                    "admitted": admitted, "finished": done_at, "latency": done_at - req["arrival"],
                    "newton_iterations": info["newton_iterations"],
                    "cell_newton_steps": cells * info["newton_iterations"],
                })
                self.batch.remove(pid)
        makespan = clock() - t0
        ok = [r for r in records if r["state"] == "finished"]
        lat = [r["latency"] for r in ok]
        work = sum(r["cell_newton_steps"] for r in ok)
        return records, {
            "requests": len(records), "finished": len(ok), "failed": len(records) - len(ok),
            "makespan_s": makespan, "solves_per_s": len(ok) / makespan if makespan > 0 else None,
            "time_step_solves_per_s": sum(r["steps"] for r in ok) / makespan if makespan > 0 else None,
            "cell_newton_steps_per_s": work / makespan if makespan > 0 else None,
            "latency_p50_s": percentile(lat, 50), "latency_p99_s": percentile(lat, 99),
            "engine_iterations": iterations,
        }
