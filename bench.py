"""Benchmark: cell*Newton-steps/s of the implicit cc-TPFA 2p hot path on one GB300.

Workload (default): 2p immiscible water-DNAPL (p_w, S_n), cc-TPFA, 3D 64x64x32 cells on
6x4x1 m, seeded ln K Gaussian field (mean ln 5e-11, sigma 1, correlation length 6 cells),
porosity 0.4, regularised Brooks-Corey (pe=500 Pa, lambda=2, Swr=0.05, Snr=0), hydrostatic
Dirichlet left/right, DNAPL inflow 0.04 kg/m^2/s on the top strip, implicit Euler
dt = 250 s, Newton MaxRelativeShift 1e-8, ILU(0)-BiCGSTAB with the Newton's linear
reduction 1e-6, plain FP64 path.  One "step" = one implicit-Euler time step (a full
Newton solve).  Synthetic inputs: the ln K field is generated from a seed.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--precision fp64|mixed] [--cells 64,64,32]

N > 1 (torchrun): every rank solves its own replica of the workload (weak scaling, no
collective on the data path); rank 0 prints the line.  --impl reference times the
reference algorithm's CPU implementation (the oracle restatement; DuMux/DUNE cannot be
built here) on the host cores.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell*Newton-steps/s (2p cc-TPFA, numeric-diff assembly + ILU0-BiCGSTAB + Newton)"
METRIC_ENSEMBLE = "cell*Newton-steps/s, batched ensemble of 2p cc-TPFA problems (engine-wide)"
METRIC_SERVE = "cell*Newton-steps/s of a served 1p/2p request stream (continuous batching)"


def metric_name():
    """The metric of the single-problem workloads (the default 2p one is the headline)."""
    if WORKLOAD == "mpfa":
        return "cell*Newton-steps/s (1p cc-MPFA-O, numeric-diff assembly + ILU0-BiCGSTAB + Newton)"
    if WORKLOAD == "mpfa2p":
        return "cell*Newton-steps/s (2p cc-MPFA-O, numeric-diff assembly + ILU0-BiCGSTAB + Newton)"
    if WORKLOAD == "1p":
        return "cell*Newton-steps/s (1p cc-TPFA, numeric-diff assembly + ILU0-BiCGSTAB + Newton)"
    return METRIC
UNIT = "cell*Newton-steps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=7)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--cells", default="64,64,32")
    ap.add_argument("--dt", type=float, default=250.0)
    ap.add_argument("--cpu-sample-iters", type=int, default=2)
    ap.add_argument("--workload", default="2p", choices=["2p", "1p", "mpfa", "mpfa2p", "ensemble", "serve",
                                                         "accuracy"],
                    help="2p: transient water-DNAPL (default); 1p: stationary Darcy, 100x100, one Newton step; "
                         "ensemble: 256 uneven 2p problems batched; serve: Poisson request stream, continuous batching; "
                         "accuracy: the 128x128x64 2p case over --steps time steps in plain FP64 and the GB300 forms, "
                         "field errors against FP64 (and against the oracle's first time step with --oracle-step)")
    ap.add_argument("--save-first-step", default="",
                    help="accuracy workload: write the FP64 solution after the first time step (.npy)")
    ap.add_argument("--oracle-step", action="store_true",
                    help="accuracy workload: also compare the first FP64 time step with the CPU oracle's")
    ap.add_argument("--diff", default="numeric", choices=["numeric", "analytic"],
                    help="Jacobian by numeric differentiation (default, the reference's default) or analytic")
    ap.add_argument("--ilu", default="natural", choices=["natural", "lanes", "wavefront", "redblack"],
                    help="ILU(0) of the single-problem workloads: natural order (the reference's SeqILU, "
                         "default; the context times the lane sweeps and the cluster wavefront and keeps "
                         "the faster), natural order forced onto the lane sweeps or onto the cluster "
                         "wavefront, or red-black (two parallel passes per sweep, more iterations)")
    ap.add_argument("--solver", default="ilu", choices=["ilu", "amg"],
                    help="ILU(0)-BiCGSTAB (default, the reference's ILUBiCGSTABIstlSolver) or "
                         "AMG-BiCGSTAB (AMGBiCGSTABIstlSolver)")
    ap.add_argument("--problems", type=int, default=256, help="ensemble size")
    ap.add_argument("--requests", type=int, default=48, help="served-stream length")
    ap.add_argument("--ticks-per-step", type=int, default=25, help="ensemble: engine ticks per timed step")
    ap.add_argument("--no-forms", action="store_true",
                    help="default workload: skip the forms, ensemble and served summaries")
    ap.add_argument("--plain-sample", type=int, default=8,
                    help="problems / requests of the workload also run alone on the plain FP64 path")
    return ap.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


WORKLOAD = "2p"
DIFF = "numeric"
ILU = "natural"
SOLVER = "ilu"


def reduce_over_ranks(seconds, sums, device):
    """Across the torchrun ranks (replicas): the maximum of the timed seconds and the
    sums of the work counters; identity on a single process."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(seconds), [float(v) for v in sums]
    t = torch.tensor([float(seconds)] + [float(v) for v in sums], device=device, dtype=torch.float64)
    mx = t[:1].clone()
    rest = t[1:].clone()
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    dist.all_reduce(rest, op=dist.ReduceOp.SUM)
    return float(mx[0]), [float(v) for v in rest]


# workloads of one stationary Newton step (LinearPDESolver semantics)
STATIONARY = ("1p", "mpfa")


def workload(cells, seed=2):
    from dumux_gb300 import problems
    if WORKLOAD == "1p":
        return problems.darcy_1p(cells=cells[:2], seed=seed - 1)
    if WORKLOAD == "mpfa":
        desc, u0, _ = problems.mpfa_convergence_problem(cells[0])
        return desc, u0
    if WORKLOAD == "mpfa2p":
        return problems.dnapl_2p_mpfa(cells=cells, seed=seed)
    return problems.dnapl_2p(cells=cells, seed=seed)


def workload_name(cells, precision):
    if WORKLOAD == "mpfa2p":
        return (f"2p water-DNAPL cc-MPFA-O {'x'.join(map(str, cells))} cells, rotated anisotropic permeability "
                "tensors (ratio 4), implicit Euler dt=250 s, Newton shift 1e-8, ILU0-BiCGSTAB reduction 1e-6, "
                f"{precision.upper()} linear system")
    if WORKLOAD == "mpfa":
        return (f"1p cc-MPFA-O {'x'.join(map(str, cells[:2]))} cells on [0,1]^2 with the full permeability "
                "tensor and analytic solution of the reference's MPFA convergence test (c = 0.9), stationary, "
                f"one Newton step, ILU0-BiCGSTAB reduction 1e-12, {precision.upper()} linear system")
    if WORKLOAD == "1p":
        return (f"1p incompressible Darcy cc-TPFA {'x'.join(map(str, cells[:2]))} cells on [0,1]^2, stationary, "
                f"one Newton step, ILU0-BiCGSTAB reduction 1e-12, {precision.upper()} linear system")
    return (f"2p water-DNAPL cc-TPFA {'x'.join(map(str, cells))} cells, implicit Euler dt=250 s, "
            f"Newton shift 1e-8, ILU0-BiCGSTAB reduction 1e-6, {precision.upper()} linear system"
            + (", analytic Jacobian" if DIFF == "analytic" else "")
            + (", red-black ordered ILU(0)" if ILU == "redblack" else "")
            + (", AMG-BiCGSTAB" if SOLVER == "amg" else ""))


def step_params():
    from dumux_gb300.abi import newton_params
    if WORKLOAD in STATIONARY:
        # LinearPDESolver semantics: one assembly, one solve, one update
        return newton_params(min_steps=1, max_steps=1, max_relative_shift=1e300, linear_reduction=1e-12,
                             max_time_step_divisions=0, linear_max_iter=1000 if ILU == "redblack" else 250)
    # the red-black preconditioner needs about twice the BiCGSTAB iterations: a higher cap
    return newton_params(linear_max_iter=1000) if ILU == "redblack" else newton_params()


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    def __init__(self, index):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._proc = None

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self._proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                           "-i", str(self.index), "-lms", "200"],
                                          stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self._proc = None
            return
        def reader():
            for line in self._proc.stdout:
                self.samples.append([v.strip() for v in line.split(",")])
        self._t = threading.Thread(target=reader, daemon=True)
        self._t.start()
        # nvidia-smi's start-up (NVML initialisation) stalls the driver for a moment: let it
        # pass before the timed region begins; the 200 ms samples continue through it
        deadline = time.perf_counter() + 2.0
        while not self.samples and time.perf_counter() < deadline:
            time.sleep(0.01)

    def stop(self):
        if self._proc:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except Exception:
                self._proc.kill()
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[1]) for s in self.samples if len(s) >= 9 and s[1].replace('.', '', 1).isdigit()]
        mx = [float(s[2]) for s in self.samples if len(s) >= 9 and s[2].replace('.', '', 1).isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            if len(s) < 9:
                continue
            for k, n in enumerate(names):
                if s[5 + k].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# dram__bytes_read.sum + dram__bytes_write.sum per ILU(0) apply (forward + backward sweep)
# of the 64x64x32 FP64 system, from ncu captures of the sweeps (cold-cache, serialised
# launches): the cluster wavefront kernels and the lane sweeps (register-ring form, the one
# the context picks at this size).
ILU_TRAFFIC_PER_APPLY_64x64x32 = 14537472 + 18714112
LANE_TRAFFIC_PER_APPLY_64x64x32 = 14520320 + 18721792
# DRAM bytes per cell of one batched FP32 apply (forward + backward sweep), from an ncu capture
# of a 32-problem ensemble (2,379,154 cells); traffic scales with the cells swept (each block
# and vector entry is moved once)
ENSEMBLE_SWEEP_TRAFFIC_PER_CELL = (136113408 + 9772544 + 174257152 + 10788608) / 2379154


def cpu_sample(desc, u0, dt, iters):
    """The oracle (restated reference algorithm) on the host cores: the first `iters`
    Newton iterations of the first time step; returns (cell*Newton-steps/s, seconds)."""
    import oracle
    from dumux_gb300.abi import newton_params
    # exactly `iters` iterations: the shift criterion is satisfied once MinSteps are done
    p = newton_params(min_steps=iters, max_steps=iters, max_relative_shift=1e300, max_time_step_divisions=0,
                      linear_reduction=1e-12 if WORKLOAD in STATIONARY else 1e-6)
    if WORKLOAD in STATIONARY:
        dt = 0.0
    t0 = time.perf_counter()
    st, u, rep = oracle.newton_solve(desc, u0, u0, dt, p)
    sec = time.perf_counter() - t0
    n = rep["iterations"] + rep["wasted_iterations"]
    if n == 0:
        n = iters
    return desc.num_cells * n / sec, sec, n


def bench_config(desc, steps, warmup, precision="fp64"):
    """The workload description both arms print (the GPU arm and the reference arm run
    exactly this work)."""
    stationary = WORKLOAD in STATIONARY
    return {"workload": workload_name(tuple(desc.cells[:desc.dim]), precision), "cells": int(desc.num_cells),
            "unknowns": int(desc.num_dofs),
            "time_steps": (f"{steps} timed stationary Newton steps from the same initial state after {warmup} "
                           "warm-up steps" if stationary else
                           f"time steps {warmup + 1}..{warmup + steps} of the seeded initial state "
                           f"({warmup} warm-up steps advance the simulation); TimeLoop.MaxTimeStepSize 250 s "
                           "and the Newton solver's step-size suggestion below it"),
            "l2": "GPU arm: flushed between timed steps (256 MiB write)"}


def run_reference(args, cells):
    """The reference arm: the oracle's restatement of the reference's CPU path on the host
    cores -- element assembly on all host threads (the reference's coloured threaded
    assembly), ILU(0)-BiCGSTAB sequential as dune-istl's SeqILU / BiCGSTABSolver -- over the
    same time steps as the GPU arm: the warm-up steps advance the simulation untimed, then
    exactly `steps` time steps are timed."""
    global WORKLOAD
    WORKLOAD = args.workload
    rank, world, _ = dist_info()
    if rank != 0:
        return 0
    import oracle
    metric = metric_name()
    name = None
    if WORKLOAD == "ensemble":
        from dumux_gb300 import problems
        desc, u0, _ = problems.ensemble_2p(count=1, seed=4)[0]
        WORKLOAD = "2p"
        metric, name = METRIC_ENSEMBLE, f"ensemble problem 0 ({desc.num_cells} cells) on the host"
    elif WORKLOAD == "serve":
        from dumux_gb300 import problems
        req = next(r for r in problems.served_requests(args.requests, seed=5) if r["kind"] == "2p")
        desc, u0 = problems.make_request_problem(req)
        WORKLOAD = "2p"
        metric, name = METRIC_SERVE, f"first 2p request ({desc.num_cells} cells) on the host"
    else:
        desc, u0 = workload(cells)
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    oracle.set_linear_threads(1)
    stationary = WORKLOAD in STATIONARY
    params = step_params()
    dt = 0.0 if stationary else args.dt
    u = np.array(u0, dtype=np.float64)

    def one_step(u, dt):
        st, u_new, rep = oracle.newton_solve(desc, u0 if stationary else u, u0 if stationary else u, dt, params)
        if st != 0:
            raise RuntimeError(f"oracle time step failed with status {st}")
        n = rep["iterations"] + rep["wasted_iterations"]
        # TimeLoop with MaxTimeStepSize: NewtonSolver::suggestTimeStepSize, capped
        dt_next = dt if stationary else min(oracle.suggest_time_step(rep["iterations"], rep["dt_used"], params),
                                            args.dt)
        return (u if stationary else u_new), n, dt_next

    for _ in range(args.warmup):
        u, _, dt = one_step(u, dt)
    t0 = time.perf_counter()
    work, iters = 0, []
    for _ in range(args.steps):
        u, n, dt = one_step(u, dt)
        iters.append(n)
        work += desc.num_cells * n
    total = time.perf_counter() - t0
    value = work / total
    sample = (f"the same {args.steps} {'stationary Newton steps' if stationary else 'time steps'} as the GPU arm "
              f"after {args.warmup} warm-up steps (assembly on {threads} OpenMP threads, ILU0-BiCGSTAB sequential "
              "as dune-istl SeqILU)")
    config = bench_config(desc, args.steps, args.warmup)
    if name:
        config = {"workload": name, "cells": int(desc.num_cells), "unknowns": int(desc.num_dofs)}
    line = {
        "impl": "reference", "metric": metric, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded ln K Gaussian field)", "config": config, "newton_iterations": iters,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "DuMux needs DUNE (not installed, no network): the reference arm runs the oracle's "
                "restatement of the same algorithm on the host cores",
    }
    print(json.dumps(line), flush=True)
    return 0


def stats_of(values):
    return {"p50": float(np.percentile(values, 50)), "p99": float(np.percentile(values, 99)),
            "mean": float(np.mean(values))} if values else None


def plain_fp64_steady(items, params, device, warm_steps, steps):
    """Each (desc, u0, dt) alone through one plain FP64 context (the single-problem drop-in
    path): context creation, upload and `warm_steps` time steps (launch-shape tuning
    included) untimed, then `steps` time steps timed with CUDA events on the context's
    stream.  Returns cell*Newton-steps/s and time-step solves/s over the sample."""
    import torch
    import dumux_gb300
    work, sec, solves = 0, 0.0, 0
    for desc, u0, dt in items:
        ctx = dumux_gb300.Context(desc, device=device, precision="fp64")
        ctx.set_solution(u0)
        ctx.set_prev_solution(u0)
        dtc = dt
        for _ in range(warm_steps):
            rep = ctx.newton_solve(dtc, params)
            ctx.advance_time_step()
            dtc = min(ctx.suggest_time_step(rep["dt_used"], params), dt)
        stream = torch.cuda.ExternalStream(ctx.stream_handle(), device=device)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        its = 0
        for _ in range(steps):
            rep = ctx.newton_solve(dtc, params)
            its += rep["iterations"] + rep["wasted_iterations"]
            ctx.advance_time_step()
            dtc = min(ctx.suggest_time_step(rep["dt_used"], params), dt)
        e1.record(stream)
        torch.cuda.synchronize()
        sec += e0.elapsed_time(e1) / 1e3
        work += desc.num_cells * its
        solves += steps
        ctx.close()
    return work / sec, solves / sec


def plain_fp64_alone(items, params, device):
    """Each (desc, u0, dt, t_end) alone through one plain FP64 context (the
    single-problem drop-in path, host time loop), as a request served alone: its service
    time runs from context creation to the result on the host.  Returns cell*Newton-steps/s
    over the sample and per-problem service seconds."""
    import dumux_gb300
    work, total, service = 0, 0.0, []
    for desc, u0, dt, t_end in items:
        t0 = time.perf_counter()
        ctx = dumux_gb300.Context(desc, device=device, precision="fp64")
        ctx.set_solution(u0)
        ctx.set_prev_solution(u0)
        t, dtc, its = 0.0, min(dt, t_end), 0
        while True:
            rep = ctx.newton_solve(dtc, params)
            its += rep["iterations"] + rep["wasted_iterations"]
            t += rep["dt_used"]
            ctx.advance_time_step()
            remaining = t_end - t
            if remaining <= 1e-9 * max(1.0, t_end):
                break
            dtc = min(ctx.suggest_time_step(rep["dt_used"], params), dt, remaining)
        ctx.solution()
        sec = time.perf_counter() - t0
        ctx.close()
        work += desc.num_cells * its
        total += sec
        service.append(sec)
    return work / total, service


# GB300 forms of the same problem measured beside the plain FP64 drop-in path: mixed
# precision (FP32 preconditioner and operator products inside the FP64 Krylov, residual and
# Newton), with the natural-order ILU(0), the red-black ordered ILU(0) or AMG-BiCGSTAB
FORMS = (("mixed", "mixed", "natural", "ilu"), ("mixed+redblack", "mixed", "redblack", "ilu"),
         ("mixed+amg", "mixed", "natural", "amg"))


def form_params(precision, ilu, solver):
    """Newton parameters of a form: the reference's defaults, with LinearSolver.MaxIterations
    1000 where an FP32 or red-black ILU(0) preconditioner needs more BiCGSTAB iterations than
    the default 250 allows (on the 128x128x64 case the FP32 ILU(0) needs up to ~270)."""
    from dumux_gb300.abi import newton_params
    if solver == "ilu" and (precision == "mixed" or ilu == "redblack"):
        return newton_params(linear_max_iter=1000)
    return newton_params()


def run_forms(desc, u_start, u_ref, dt_seq, device, plain_ms_per_step, plain_value, flush):
    """Each form of FORMS over the same time steps as the timed plain FP64 region: from
    the same state u_start, the implicit-Euler steps of sizes dt_seq timed with CUDA events on the
    context's stream (L2 flushed between steps); one untimed step from u_start first
    (kernel loading, launch-shape tuning, AMG setup).  Reports the speed-up per time step
    over plain FP64 and the error of p_w and S_n against the plain FP64 fields u_ref."""
    import torch
    import dumux_gb300
    from dumux_gb300.abi import newton_params
    b = desc.num_eq
    ref = u_ref.reshape(-1, b)
    out = {}
    for name, precision, ilu, solver in FORMS:
        ctx = dumux_gb300.Context(desc, device=device, precision=precision)
        params = form_params(precision, ilu, solver)
        if ilu == "redblack":
            ctx.set_ilu_kernel("redblack")
        if solver == "amg":
            ctx.set_linear_solver("amg")
        steps = len(dt_seq)
        ctx.set_solution(u_start)
        ctx.set_prev_solution(u_start)
        ctx.newton_solve(dt_seq[0], params)
        ctx.set_solution(u_start)
        ctx.set_prev_solution(u_start)
        stream = torch.cuda.ExternalStream(ctx.stream_handle(), device=device)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        its, work = [], 0
        for dt in dt_seq:
            rep = ctx.newton_solve(dt, params)
            ctx.advance_time_step()
            its.append(rep["iterations"] + rep["wasted_iterations"])
            work += desc.num_cells * its[-1]
            with torch.cuda.stream(stream):
                flush.zero_()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        u = ctx.solution().reshape(-1, b)
        ctx.close()
        entry = {"value": work / (ms / 1e3), "unit": UNIT, "ms_per_step": ms / steps,
                 "speedup_per_time_step": plain_ms_per_step / (ms / steps),
                 "speedup_metric": (work / (ms / 1e3)) / plain_value, "newton_iterations": its,
                 "precision": precision, "ilu": ilu, "linear_solver": solver}
        for k, fname in enumerate(("p_w", "S_n")[:b]):
            d = u[:, k] - ref[:, k]
            entry[f"max_rel_err_{fname}"] = float(np.max(np.abs(d)) / np.max(np.abs(ref[:, k])))
            entry[f"l2_rel_err_{fname}"] = float(np.linalg.norm(d) / np.linalg.norm(ref[:, k]))
        out[name] = entry
    return out


def ensemble_summary(device, count=64, T=25, warm=2, steps=2, plain_sample=4):
    """A smaller instance of the batched ensemble (`count` problems of the ensemble workload,
    mixed precision, natural ILU(0) and AMG-BiCGSTAB): time-step solves/s and
    cell*Newton-steps/s over `steps` x T ticks after `warm` x T warm-up ticks, beside the
    same problems alone on the plain FP64 path in steady state."""
    import torch
    import dumux_gb300
    from dumux_gb300 import problems
    from dumux_gb300.abi import newton_params
    params = newton_params()
    probs = problems.ensemble_2p(count=count, seed=4)
    out = {"problems": count, "cells_total": int(sum(d.num_cells for d, _, _ in probs)), "ticks_per_step": T,
           "steps": steps, "precision": "mixed"}
    for solver in ("ilu", "amg"):
        batch = dumux_gb300.Batch(device=device, precision="mixed", solver=solver)
        ids = [batch.add(d, u0, dt=250.0, t_end=1e12, params=params) for d, u0, _ in probs]
        for _ in range(warm * T):
            batch.iterate()
        before = {i: batch.info(i) for i in ids}
        stream = torch.cuda.ExternalStream(batch.stream_handle(), device=device)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps * T):
            batch.iterate()
        e1.record(stream)
        torch.cuda.synchronize()
        sec = e0.elapsed_time(e1) / 1e3
        after = {i: batch.info(i) for i in ids}
        work = sum(after[i]["cells"] * (after[i]["newton_iterations"] - before[i]["newton_iterations"]) for i in ids)
        solves = sum(after[i]["time_steps"] - before[i]["time_steps"] for i in ids)
        batch.close()
        out[solver] = {"value": work / sec, "unit": UNIT, "solves_per_s": solves / sec}
    sample = probs[::max(1, count // plain_sample)][:plain_sample]
    plain, plain_solves = plain_fp64_steady([(d, u0, 250.0) for d, u0, _ in sample], params, device, 1, steps)
    out["plain_fp64_same_problems"] = {"value": plain, "unit": UNIT, "solves_per_s": plain_solves,
                                       "sample": f"{len(sample)} of the problems alone, 1 untimed and {steps} "
                                                 "timed time steps each"}
    for solver in ("ilu", "amg"):
        out[solver]["speedup_vs_plain_fp64"] = out[solver]["value"] / plain
    return out


def serve_summary(device, requests=24, plain_sample=4):
    """A shorter served stream (the first `requests` requests of the served workload,
    mixed precision, AMG-BiCGSTAB): p50/p99 latency and solves/s, beside the same requests
    served alone one after another on the plain FP64 path."""
    import torch
    from dumux_gb300 import problems
    from dumux_gb300.abi import newton_params
    from dumux_gb300.serve import Server
    params = newton_params()
    reqs = problems.served_requests(requests, rate=200.0, seed=5)
    built = {r["index"]: problems.make_request_problem(r) for r in reqs}
    free, _ = torch.cuda.mem_get_info(device)
    server = Server(device=device, precision="mixed", memory_budget=int(0.8 * free), params=params, solver="amg")
    warm = problems.served_requests(3, rate=1e6, seed=99, n_max=2e4)
    server.serve(warm, problems.make_request_problem)
    records, st = server.serve(reqs, lambda r: built[r["index"]])
    server.batch.close()
    sample = reqs[::max(1, len(reqs) // plain_sample)][:plain_sample]
    items = [(built[r["index"]][0], built[r["index"]][1], r["dt"], r["t_end"]) for r in sample]
    plain, service = plain_fp64_alone(items, params, device)
    return {"requests": requests, "precision": "mixed", "linear_solver": "amg",
            "latency_p50_s": st["latency_p50_s"], "latency_p99_s": st["latency_p99_s"],
            "solves_per_s": st["solves_per_s"], "value": st["cell_newton_steps_per_s"], "unit": UNIT,
            "makespan_s": st["makespan_s"],
            "plain_fp64_alone": {"value": plain, "unit": UNIT, "service_s": stats_of(service),
                                 "sample": f"{len(sample)} of the requests, each alone through one FP64 context "
                                           "(creation to result)"},
            "speedup_vs_plain_fp64": st["cell_newton_steps_per_s"] / plain}


def fp64_peak(device):
    """The device's dense FP64 FMA rate, measured here with CUDA events (None if unavailable)."""
    import dumux_gb300
    try:
        rates = [dumux_gb300.fp64_fma_rate(device) for _ in range(3)]
    except Exception:
        return None
    return {"tflops": max(rates), "unit": "TFLOP/s", "source": "measured in this run (dxg_fp64_fma_rate)"}


def sweep_flops_per_apply(cells, b):
    """FP64 flops of one ILU(0) apply (forward + backward sweep) on a structured grid: a
    b x b block-vector product (2 b^2 flops) per off-diagonal block of L and of U (one each
    per interior face) and one per inverted pivot."""
    nx, ny, nz = (tuple(cells) + (1, 1))[:3]
    faces = (nx - 1) * ny * nz + nx * (ny - 1) * nz + nx * ny * (nz - 1)
    return 2.0 * b * b * (2 * faces + nx * ny * nz)


def fp64_roof(roofline, peak_tflops, flops_per_apply, launches, ms):
    """The FP64 side of the sweep's roofline: achieved FP64 rate, arithmetic intensity and
    the fraction of min(HBM bandwidth x intensity, FP64 peak)."""
    if not launches or not ms or not roofline.get("algorithmic_bytes"):
        return None
    sec = ms / launches / 1e3
    intensity = flops_per_apply / roofline["algorithmic_bytes"]
    bound = min(roofline["peak"] * 1e9 * intensity, peak_tflops * 1e12)
    achieved = flops_per_apply / sec
    return {"flops_per_launch": flops_per_apply, "intensity_flop_per_byte": intensity,
            "achieved_tflops": achieved / 1e12, "peak_tflops": peak_tflops,
            "bound_tflops": bound / 1e12, "bound_by": "fp64" if bound < roofline["peak"] * 1e9 * intensity else "hbm",
            "frac": achieved / bound}


def batch_roofline(batch):
    """Kernel-class timing of the batched launches -> kernels dict and the roofline of
    the class with the largest device time."""
    peak, peak_kind = measured_peaks()
    kernels = {}
    for kind in ("ilu_sweep", "assembly", "spmv"):
        n, kms, by = batch.kernel_timing(kind)
        kernels[kind] = {"launches": n, "ms": kms, "gbs": (by / (kms / 1e3) / 1e9) if kms else None,
                         "algorithmic_bytes_per_launch": (by / n) if n else None}
    top = max(kernels, key=lambda k: kernels[k]["ms"])
    total = sum(v["ms"] for v in kernels.values())
    names = {"ilu_sweep": "waveKernel (batched ILU(0) forward+backward sweeps, one cluster per problem)",
             "assembly": "volvarsKernel + rowKernel (batched numeric-diff assembly)",
             "spmv": "spmvKernel (batched block SpMV)"}
    a = kernels[top]["gbs"]
    roofline = {"kernel": names[top], "bound": "hbm", "achieved": a, "peak": peak, "unit": "GB/s",
                "frac": (a / peak) if a else None, "traffic": None,
                "algorithmic_bytes": kernels[top]["algorithmic_bytes_per_launch"],
                "peak_source": f"{peak_kind} hbm_gbs", "share_of_sweep_spmv_assembly": kernels[top]["ms"] / total
                if total else None}
    if top == "assembly":
        roofline["note"] = "assembly is FP64-pipe bound (numeric-diff flux evaluations), reported against HBM"
    return kernels, roofline


def run_ensemble(args):
    """Batched ensemble: `--problems` independent 2p problems (uneven grids 16..64 per
    axis, own ln K fields and inflow rates) resident together in one dxg_batch.
    Steady-state throughput: every problem keeps time-stepping (no end time inside the
    run), a step is `--ticks-per-step` engine ticks (each: one chunk of 8 BiCGSTAB
    iterations for every problem, plus the assemblies and updates of the problems whose
    Newton iteration starts or ends in it)."""
    rank, world, local = dist_info()
    import torch
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    import dumux_gb300
    from dumux_gb300 import problems
    from dumux_gb300.abi import newton_params
    params = newton_params(linear_max_iter=1000) if args.ilu == "redblack" else newton_params()
    dt = args.dt
    T = args.ticks_per_step
    t_end = 1e12                   # problems keep stepping through the whole run
    probs = problems.ensemble_2p(count=args.problems, seed=4 + 100003 * rank)
    for d, _, _ in probs:
        d.analytic = args.diff == "analytic"
    cells_total = sum(d.num_cells for d, _, _ in probs)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    def ticks(b, n):
        for _ in range(n):
            b.iterate()

    batch = dumux_gb300.Batch(device=local, precision=args.precision, ilu=args.ilu, solver=args.solver)
    ids = [batch.add(d, u0, dt=dt, t_end=t_end, params=params) for d, u0, _ in probs]
    cells_of = {pid: d.num_cells for pid, (d, _, _) in zip(ids, probs)}
    ticks(batch, args.warmup * T)            # includes the sweep autotuning
    # kernel-class timing over one step's ticks (events around the batched launches)
    batch.set_kernel_timing(True)
    ticks(batch, T)
    kernels, roofline = batch_roofline(batch)
    batch.set_kernel_timing(False)
    if roofline["kernel"].startswith("waveKernel") and args.precision == "mixed":
        roofline["traffic"] = ENSEMBLE_SWEEP_TRAFFIC_PER_CELL * cells_total
        roofline["traffic_note"] = "ncu dram bytes of a 32-problem ensemble apply, scaled by cells"

    sweep_shapes = batch.describe().strip()
    before = {i: batch.info(i) for i in ids}
    stream = torch.cuda.ExternalStream(batch.stream_handle(), device=local)
    launches0 = batch.kernel_launches()
    sampler = ClockSampler(local)
    barrier()
    torch.cuda.synchronize()
    sampler.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    ticks(batch, args.steps * T)
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clocks = sampler.stop()
    sec = ev0.elapsed_time(ev1) / 1e3
    launches = batch.kernel_launches() - launches0
    after = {i: batch.info(i) for i in ids}
    failed = sum(1 for i in ids if after[i]["state"] == "failed")
    work = sum(cells_of[i] * (after[i]["newton_iterations"] - before[i]["newton_iterations"]) for i in ids)
    solves = sum(after[i]["time_steps"] - before[i]["time_steps"] for i in ids)
    lin = sum(after[i]["linear_iterations"] - before[i]["linear_iterations"] for i in ids)
    newton = sum(after[i]["newton_iterations"] - before[i]["newton_iterations"] for i in ids)
    sec, (work, solves) = reduce_over_ranks(sec, [work, solves], f"cuda:{local}")
    batch.close()

    # ---- end to end through the C ABI: admit (tabulation + h2d), then per step T ticks
    # and the read-back of every problem's solution
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b2 = dumux_gb300.Batch(device=local, precision=args.precision, ilu=args.ilu, solver=args.solver)
    ids2 = [b2.add(d, u0, dt=dt, t_end=t_end, params=params) for d, u0, _ in probs]
    d2h = 0
    for _ in range(args.steps):
        ticks(b2, T)
        for i in ids2:
            d2h += b2.solution(i).size * 8
    e2e_sec = time.perf_counter() - t0
    e2e_work = sum(d.num_cells * b2.info(i)["newton_iterations"] for i, (d, _, _) in zip(ids2, probs))
    b2.close()
    h2d = sum(d.num_dofs * 8 + d.num_cells * 16 + d.bc_type.size + d.bc_values.size * 8 for d, _, _ in probs)
    e2e_sec, (e2e_work,) = reduce_over_ranks(e2e_sec, [e2e_work], f"cuda:{local}")
    e2e = {"value": e2e_work / e2e_sec, "unit": UNIT, "h2d_bytes_per_step": int(h2d / args.steps),
           "d2h_bytes_per_step": int(d2h / args.steps),
           "note": "fresh batch: admission of every problem (tabulation + upload) and, per step, "
                   f"{T} ticks and the read-back of all solutions"}

    value = work / sec
    line = {
        "metric": METRIC_ENSEMBLE, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": sec * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64" if args.precision == "mixed" else "f64",
        "data": "synthetic (seeded ln K Gaussian fields)",
        "config": {"workload": f"batched ensemble: {args.problems} independent 2p water-DNAPL problems, grids "
                               f"16..64 cells per axis (uniform integers), sigma U[0.5,2], corr. length U[3,10] "
                               f"cells, inflow U[0.01,0.08] kg/m^2/s, dt=250 s, {args.precision} precision",
                   "problems": args.problems, "cells_total": int(cells_total), "global_batch": world,
                   "ticks_per_step": T, "newton_iterations": newton, "linear_iterations": lin,
                   "failed_problems": failed,
                   "parallelism": f"replicas x{world}" if world > 1 else "1 GPU, one batched launch per kernel",
                   "l2": "inputs larger than L2 (all problems resident, GBs of state)",
                   "step": f"{T} engine ticks with every problem resident and time-stepping"},
        "ensemble_solves_per_s": solves / sec, "sweep_shapes": sweep_shapes,
        "e2e": e2e, "gpu_launches": int(launches), "clocks": clocks, "roofline": roofline, "kernels": kernels,
    }
    if rank == 0:
        if args.plain_sample > 0:
            sample = probs[::max(1, len(probs) // args.plain_sample)][:args.plain_sample]
            plain, plain_solves = plain_fp64_steady([(d, u0, dt) for d, u0, _ in sample], params, local,
                                                    args.warmup, args.steps)
            line["plain_fp64_same_problems"] = {
                "value": plain, "unit": UNIT, "solves_per_s": plain_solves,
                "sample": f"{len(sample)} of the problems alone through one FP64 context each: creation, upload "
                          f"and {args.warmup} time steps untimed, then {args.steps} time steps timed on the device",
                "speedup_of_batched": value / plain}
        if args.cpu_sample_iters > 0:
            desc0, u00, _ = probs[0]
            rate, sec_cpu, n_cpu = cpu_sample(desc0, u00, dt, args.cpu_sample_iters)
            import oracle
            line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": oracle.get_threads(), "kind": "port",
                                    "sample": f"problem 0 ({desc0.num_cells} cells): first {n_cpu} Newton "
                                              f"iterations of its first time step ({sec_cpu:.1f} s)"}
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_serve(args):
    """Served stream: Poisson arrivals (200/s) of a 30/70 1p/2p mix, cube grids log-uniform
    in [1e3, 1e6] cells, 1..20 time steps each, admitted by device-memory budget into a
    continuously batched engine."""
    rank, world, local = dist_info()
    import torch
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    from dumux_gb300 import problems
    from dumux_gb300.abi import newton_params
    from dumux_gb300.serve import Server
    params = newton_params(linear_max_iter=1000) if args.ilu == "redblack" else newton_params()
    reqs = problems.served_requests(args.requests, rate=200.0, seed=5 + 100003 * rank)
    built = {r["index"]: problems.make_request_problem(r) for r in reqs}
    free, _ = torch.cuda.mem_get_info(local)
    budget = int(0.8 * free)
    server = Server(device=local, precision=args.precision, memory_budget=budget, params=params, ilu=args.ilu,
                    solver=args.solver)
    # warm-up: small requests of both kinds (kernel loading, sweep autotuning)
    warm = problems.served_requests(max(3, args.warmup), rate=1e6, seed=99, n_max=2e4)
    server.serve(warm, problems.make_request_problem)
    launches0 = server.batch.kernel_launches()
    sampler = ClockSampler(local)
    torch.cuda.synchronize()
    sampler.start()
    records, st = server.serve(reqs, lambda r: built[r["index"]])
    torch.cuda.synchronize()
    clocks = sampler.stop()
    launches = server.batch.kernel_launches() - launches0
    h2d = sum(d.num_dofs * 8 + d.num_cells * 16 + d.bc_type.size + d.bc_values.size * 8 for d, _ in built.values())
    d2h = 0
    line = {
        "metric": METRIC_SERVE, "value": st["cell_newton_steps_per_s"], "unit": UNIT, "n_gpus": world,
        "steps": args.requests, "warmup": len(warm), "ms_per_step": st["makespan_s"] * 1e3 / max(1, len(records)),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64" if args.precision == "mixed" else "f64", "data": "synthetic (seeded request stream)",
        "config": {"workload": f"served stream: {args.requests} requests, Poisson arrivals 200/s, 30/70 1p/2p, "
                               "cube grids log-uniform 1e3..1e6 cells, 1..20 steps of 250 s, "
                               f"{args.precision} precision, HBM admission budget {budget / 1e9:.0f} GB",
                   "step": "one request (ms_per_step = makespan / requests)",
                   "l2": "inputs larger than L2", "parallelism": "1 GPU, continuous batching"},
        "serve": st, "solves_per_s": st["solves_per_s"],
        "latency_p50_s": st["latency_p50_s"], "latency_p99_s": st["latency_p99_s"],
        "e2e": {"value": st["cell_newton_steps_per_s"], "unit": UNIT,
                "h2d_bytes_per_step": int(h2d / max(1, len(records))), "d2h_bytes_per_step": d2h,
                "note": "the served loop is itself end to end: arrival replay, admission (tabulation + upload), "
                        "solve, release"},
        "gpu_launches": int(launches), "clocks": clocks,
    }
    if rank == 0 and args.plain_sample > 0:
        sample = reqs[::max(1, len(reqs) // args.plain_sample)][:args.plain_sample]
        items = [(built[r["index"]][0], built[r["index"]][1], r["dt"], r["t_end"]) for r in sample]
        plain, service = plain_fp64_alone(items, params, local)
        served_lat = {r["index"]: rec["latency"] for rec in records for r in sample if rec["index"] == r["index"]}
        line["plain_fp64_alone"] = {
            "value": plain, "unit": UNIT, "sample": f"{len(sample)} of the requests, each alone through one FP64 "
                                                     "context (no queueing)",
            "service_s": stats_of(service), "solves_per_s_sequential": len(service) / sum(service),
            "served_latency_of_same_requests_s": stats_of(list(served_lat.values())),
            "speedup_of_served": st["cell_newton_steps_per_s"] / plain}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def field_errors(u, ref, b=2):
    """Max and L2 relative errors of p_w and S_n of u against ref."""
    u, ref = u.reshape(-1, b), ref.reshape(-1, b)
    out = {}
    for k, name in enumerate(("p_w", "S_n")[:b]):
        d = u[:, k] - ref[:, k]
        out[f"max_rel_err_{name}"] = float(np.max(np.abs(d)) / np.max(np.abs(ref[:, k])))
        out[f"l2_rel_err_{name}"] = float(np.linalg.norm(d) / np.linalg.norm(ref[:, k]))
    return out


def run_accuracy(args, cells):
    """The 2p case at `cells` (default 128x128x64, 1,048,576 cells) over --steps implicit-Euler
    steps (TimeLoop.MaxTimeStepSize --dt with the Newton solver's suggestion below it) in
    plain FP64 and in the GB300 forms: per-step Newton iterations, time-step divisions and
    sizes, wall time, and the forms' field errors against FP64 at the end; with
    --oracle-step also the FP64 first time step against the CPU oracle's."""
    import torch
    import dumux_gb300
    from dumux_gb300.abi import newton_params
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    desc, u0 = workload(cells)
    params = newton_params()
    runs = {}
    first_step = None
    for name, precision, ilu, solver in (("fp64", "fp64", "natural", "ilu"),) + FORMS:
        ctx = dumux_gb300.Context(desc, device=local, precision=precision)
        p = form_params(precision, ilu, solver)
        if ilu == "redblack":
            ctx.set_ilu_kernel("redblack")
        if solver == "amg":
            ctx.set_linear_solver("amg")
        ctx.set_solution(u0)
        ctx.set_prev_solution(u0)
        dt, t = args.dt, 0.0
        steps = []
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(args.steps):
            rep = ctx.newton_solve(dt, p)
            ctx.advance_time_step()
            if k == 0 and name == "fp64":
                first_step = ctx.solution()
                if args.save_first_step:
                    np.save(args.save_first_step, first_step)
            t += rep["dt_used"]
            steps.append({"dt": dt, "dt_used": rep["dt_used"], "iterations": rep["iterations"],
                          "divisions": rep["time_step_divisions"], "wasted_iterations": rep["wasted_iterations"],
                          "linear_iterations": rep["linear_iterations"]})
            dt = min(ctx.suggest_time_step(rep["dt_used"], p), args.dt)
        torch.cuda.synchronize()
        runs[name] = {"seconds": time.perf_counter() - t0, "time": t, "steps": steps, "u": ctx.solution(),
                      "ilu_kernels": ctx.describe()}
        ctx.close()
    ref = runs["fp64"]["u"]
    out = {}
    for name, r in runs.items():
        e = {"seconds": r["seconds"], "simulated_time_s": r["time"], "steps": r["steps"], "ilu_kernels": r["ilu_kernels"],
             "newton_iterations": sum(s["iterations"] + s["wasted_iterations"] for s in r["steps"])}
        if name != "fp64":
            e.update(field_errors(r["u"], ref))
            e["same_time"] = r["time"] == runs["fp64"]["time"]
        out[name] = e
    line = {"workload": "accuracy", "config": {"workload": workload_name(cells, "fp64"), "cells": int(desc.num_cells),
                                               "time_steps": args.steps, "max_dt": args.dt},
            "runs": out}
    if args.oracle_step:
        import oracle
        oracle.set_threads(os.cpu_count() or 1)
        oracle.set_linear_threads(0)
        t0 = time.perf_counter()
        st, uo, orep = oracle.newton_solve(desc, u0, u0, args.dt, params)
        line["oracle_first_step"] = {
            "status": st, "seconds": time.perf_counter() - t0, "iterations": orep["iterations"],
            "divisions": orep["time_step_divisions"], "dt_used": orep["dt_used"],
            "gpu_iterations": runs["fp64"]["steps"][0]["iterations"],
            "gpu_divisions": runs["fp64"]["steps"][0]["divisions"], **field_errors(first_step, uo)}
    print(json.dumps(line), flush=True)
    return 0


def main():
    global WORKLOAD, DIFF, ILU, SOLVER
    args = parse()
    WORKLOAD = args.workload
    DIFF = args.diff
    ILU = args.ilu
    SOLVER = args.solver
    if args.workload in ("ensemble", "serve") and args.ilu in ("lanes", "wavefront"):
        sys.exit("--ilu lanes/wavefront applies to the single-problem workloads")
    if args.workload in ("ensemble", "serve") and args.impl == "gb300":
        if args.precision == "fp64" and "--precision" not in sys.argv:
            args.precision = "mixed"
        return run_ensemble(args) if args.workload == "ensemble" else run_serve(args)
    if args.workload == "1p" and args.cells == "64,64,32":
        args.cells = "100,100"
        args.cpu_sample_iters = 1
    if args.workload == "mpfa2p":
        if args.cells == "64,64,32":
            args.cells = "32,32,16"
        args.cpu_sample_iters = 1
        if args.ilu != "natural" or args.solver != "ilu" or args.precision != "fp64" or args.diff != "numeric":
            sys.exit("--workload mpfa2p: FP64, numeric Jacobian, natural-order ILU(0)-BiCGSTAB")
    if args.workload == "mpfa":
        if args.cells == "64,64,32":
            args.cells = "256,256"
        args.cpu_sample_iters = 1
        if args.ilu == "redblack" or args.solver != "ilu" or args.precision != "fp64" or args.diff != "numeric":
            sys.exit("--workload mpfa: FP64, numeric Jacobian, natural-order ILU(0)-BiCGSTAB "
                     "(--ilu natural: the context's choice, wavefront: one-CTA line sweeps, "
                     "lanes: cluster line sweeps)")
    cells = tuple(int(c) for c in args.cells.split(","))
    if args.workload in STATIONARY:
        args.dt = 0.0
    if args.impl == "reference":
        return run_reference(args, cells)
    if args.workload == "accuracy":
        WORKLOAD = "2p"
        if args.cells == "64,64,32" and "--cells" not in sys.argv:
            cells = (128, 128, 64)
        if "--steps" not in sys.argv:
            args.steps = 10
        return run_accuracy(args, cells)

    rank, world, local = dist_info()
    import torch
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)

    import dumux_gb300
    desc, u0 = workload(cells, seed=2 + rank)
    desc.analytic = args.diff == "analytic"
    ctx = dumux_gb300.Context(desc, device=local, precision=args.precision)
    if args.ilu != "natural":
        ctx.set_ilu_kernel(args.ilu)
    if args.solver == "amg":
        ctx.set_linear_solver("amg")
    params = step_params()
    stationary = args.workload in STATIONARY
    stream = torch.cuda.ExternalStream(ctx.stream_handle(), device=local)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    # the flush's first launch loads its kernel (tens of ms): once here, outside the timed regions
    with torch.cuda.stream(stream):
        flush.zero_()
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # warm-up time steps (advance the simulation)
    ctx.set_solution(u0)
    ctx.set_prev_solution(u0)

    def next_dt(dt, rep):
        # TimeLoop with MaxTimeStepSize: NewtonSolver::suggestTimeStepSize, capped
        return dt if stationary else min(ctx.suggest_time_step(rep["dt_used"], params), args.dt)

    dt = args.dt
    for _ in range(args.warmup):
        if stationary:
            ctx.set_solution(u0)
        rep = ctx.newton_solve(dt, params)
        ctx.advance_time_step()
        dt = next_dt(dt, rep)
    u_start = u0 if stationary else ctx.solution()
    dt_start = dt
    # one untimed pass over the steps the regions below time, from the same state: the first
    # pass after the warm-up steps ran ~10% slower than every later pass of the same steps
    # (GPU clocks still settling), so both timed regions measure the steady state
    dtr = dt
    for _ in range(args.steps):
        if stationary:
            ctx.set_solution(u0)
        rep = ctx.newton_solve(dtr, params)
        ctx.advance_time_step()
        dtr = next_dt(dtr, rep)
    ctx.set_solution(u_start)
    ctx.set_prev_solution(u_start)

    # ---- device-resident timed region
    launches0 = ctx.kernel_launches()
    sampler = ClockSampler(local)
    barrier()
    torch.cuda.synchronize()
    sampler.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    work = 0
    newton_iters = []
    dt_seq = []
    step_events = []
    for _ in range(args.steps):
        if stationary:
            ctx.set_solution(u0)            # each step solves the same stationary problem
        dt_seq.append(dt)
        rep = ctx.newton_solve(dt, params)
        ctx.advance_time_step()
        dt = next_dt(dt, rep)
        newton_iters.append(rep["iterations"] + rep["wasted_iterations"])
        work += ctx.num_cells * newton_iters[-1]
        step_events.append(torch.cuda.Event(enable_timing=True))
        step_events[-1].record(stream)
        with torch.cuda.stream(stream):
            flush.zero_()          # L2 flush between timed steps (256 MiB > 129 MB L2)
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier()
    ms = ev0.elapsed_time(ev1)
    step_ms = [ev0.elapsed_time(step_events[0])] + [step_events[k - 1].elapsed_time(step_events[k])
                                                    for k in range(1, len(step_events))]
    launches = ctx.kernel_launches() - launches0
    sec = ms / 1e3
    u_after = ctx.solution()
    sec, (work,) = reduce_over_ranks(sec, [work], f"cuda:{local}")
    value = work / sec

    # ---- end to end through the C ABI with host buffers (h2d + d2h inside the region)
    ctx.set_solution(u_start)
    ctx.set_prev_solution(u_start)
    host_u = np.array(u_start)
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_work = 0
    e2e_step_ms = []
    for k in range(args.steps):
        ts = time.perf_counter()
        ctx.set_solution(u0 if stationary else host_u)   # h2d: initial guess of the step
        rep = ctx.newton_solve(dt_seq[k], params)
        host_u = ctx.solution()             # d2h: result of the step
        ctx.advance_time_step()
        e2e_work += ctx.num_cells * (rep["iterations"] + rep["wasted_iterations"])
        e2e_step_ms.append((time.perf_counter() - ts) * 1e3)
    torch.cuda.synchronize()
    e2e_sec = time.perf_counter() - t0
    # the clock sampler ran through both timed regions, so both see its NVML polling
    clocks = sampler.stop()
    e2e_sec, (e2e_work,) = reduce_over_ranks(e2e_sec, [e2e_work], f"cuda:{local}")
    e2e = {"value": e2e_work / e2e_sec, "unit": UNIT, "h2d_bytes_per_step": int(ctx.num_dofs * 8),
           "d2h_bytes_per_step": int(ctx.num_dofs * 8)}

    # ---- per-kernel event timing: one more time step from the state after the timed
    # region, outside of it (events around every launch would perturb the timed region)
    ctx.set_solution(u0 if stationary else u_after)
    ctx.set_prev_solution(u_after)
    ctx.set_kernel_timing(True)
    ctx.newton_solve(dt, params)
    sweep_n, sweep_ms, sweep_bytes = ctx.kernel_timing("ilu_sweep")
    sweep_flops = sweep_flops_per_apply(cells, desc.num_eq)
    asm_n, asm_ms, asm_bytes = ctx.kernel_timing("assembly")
    spmv_n, spmv_ms, spmv_bytes = ctx.kernel_timing("spmv")
    fac_n, fac_ms, fac_bytes = ctx.kernel_timing("ilu_factor")
    ctx.set_kernel_timing(False)
    timed_ms = sweep_ms + asm_ms + spmv_ms

    peak, peak_kind = measured_peaks()
    achieved = (sweep_bytes / sweep_n) / (sweep_ms / sweep_n / 1e3) / 1e9 if sweep_n else None
    lanes = "lane wavefront" in ctx.describe().split(";")[0]
    traffic = ((LANE_TRAFFIC_PER_APPLY_64x64x32 if lanes else ILU_TRAFFIC_PER_APPLY_64x64x32)
               if (args.workload == "2p" and cells == (64, 64, 32) and args.precision == "fp64") else None)
    if args.solver == "amg":
        rkernel = "AMG V-cycle (amg.cu passes, one preconditioner application)"
        rnote = ("bandwidth-bound passes over each level; algorithmic bytes counted as one read of the "
                 "fine operator, pivots and vectors, which the V-cycle reads about three times")
    elif args.ilu == "redblack":
        rkernel = "rbApplyBlack + rbApplyRed (red-black ILU(0) apply, two parallel passes)"
        rnote = "bandwidth-bound passes, latency bound at small grids"
    elif args.workload in ("mpfa", "mpfa2p"):
        dsc = ctx.describe()
        kname = ("stencilLane3dKernel" if "one z-plane per CTA" in dsc else
                 "stencilLane2dKernel" if "over a cluster" in dsc else
                 "stencilWave2dKernel" if "line sweeps" in dsc else "stencilApplyKernel")
        rkernel = f"{kname} (ILU(0) forward+backward sweep of the MPFA-O stencil, one apply)"
        rnote = ("latency-bound natural-order sweeps (nx + 2 ny - 1 levels each), far below the HBM roof; "
                 "algorithmic bytes: every factor entry, pivot and vector entry once")
        traffic = None
    elif lanes:
        rkernel = "laneWaveKernel (ILU(0) forward+backward lane sweeps, one apply)"
        rnote = ("latency/FP64-bound wavefront (one dependent level per grid line step and plane), "
                 "far below the HBM roof")
    else:
        rkernel = "waveKernel (ILU(0) forward+backward sweep, one apply)"
        rnote = "latency/FP64-bound wavefront (nx+ny+nz-2 dependent levels), far below the HBM roof"
    if args.solver == "amg" or args.ilu == "redblack":
        traffic = None
    roofline = {"kernel": rkernel, "bound": "hbm",
                "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": (achieved / peak) if achieved else None,
                "traffic": traffic, "algorithmic_bytes": sweep_bytes / sweep_n if sweep_n else None,
                "peak_source": f"{peak_kind} hbm_gbs",
                "share_of_sweep_spmv_assembly": (sweep_ms / timed_ms) if timed_ms else None,
                "note": rnote}
    kernels = {
        # the preconditioner application: ILU(0) sweeps, red-black passes or the AMG V-cycle
        "ilu_sweep": {"launches": sweep_n, "ms": sweep_ms, "gbs": achieved},
        "assembly": {"launches": asm_n, "ms": asm_ms,
                     "gbs": (asm_bytes / (asm_ms / 1e3) / 1e9) if asm_ms else None},
        "spmv": {"launches": spmv_n, "ms": spmv_ms, "gbs": (spmv_bytes / (spmv_ms / 1e3) / 1e9) if spmv_ms else None},
        # the preconditioner setup: ILU(0) factorisation (red-black pivots, AMG hierarchy)
        "ilu_factor": {"launches": fac_n, "ms": fac_ms,
                       "gbs": (fac_bytes / (fac_ms / 1e3) / 1e9) if fac_ms else None},
    }

    line = {
        "metric": metric_name(), "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32+f64",
        "data": "synthetic (seeded ln K Gaussian field)",
        "config": bench_config(desc, args.steps, args.warmup, args.precision),
        "newton_iterations": newton_iters, "parallelism": f"replicas x{world}",
        "step": "one stationary Newton step from the same initial state (includes its 80 KB h2d reset)"
                if stationary else "one implicit-Euler time step",
        "ilu_kernels": ctx.describe(),
        "warm_pass": "one untimed pass over the timed steps, from the same state, precedes both timed regions",
        "step_ms": {"device": [round(t, 2) for t in step_ms], "e2e": [round(t, 2) for t in e2e_step_ms]},
        "e2e": e2e, "gpu_launches": int(launches), "clocks": clocks, "roofline": roofline, "kernels": kernels,
    }
    headline = (args.workload == "2p" and cells == (64, 64, 32) and args.precision == "fp64"
                and args.solver == "ilu" and args.ilu == "natural" and args.diff == "numeric")
    if rank == 0 and world == 1 and headline and not args.no_forms:
        # the GB300 forms of the same problem over the same time steps (from u_start), and
        # shorter instances of the batched and served workloads
        line["forms"] = run_forms(desc, u_start, u_after, dt_seq, local, ms / args.steps, value, flush)
        line["forms"]["note"] = ("each form from the state the timed FP64 region started from, over the same "
                                 f"{args.steps} time steps; errors against the FP64 fields at their end")
        line["ensemble"] = ensemble_summary(local)
        line["ensemble_solves_per_s"] = line["ensemble"]["amg"]["solves_per_s"]
        line["serve"] = serve_summary(local)
        line["fp64_peak"] = fp64_peak(local)
        if line["fp64_peak"]:
            line["roofline"]["fp64"] = fp64_roof(line["roofline"], line["fp64_peak"]["tflops"], sweep_flops, sweep_n,
                                                 sweep_ms)
    if rank == 0:
        rate, sec_cpu, n_cpu = cpu_sample(desc, u_start, dt_start, args.cpu_sample_iters)
        import oracle
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": oracle.get_threads(), "kind": "port",
                                "sample": f"first {n_cpu} Newton iterations of one time step "
                                          f"({sec_cpu:.1f} s; threaded assembly, sequential ILU0-BiCGSTAB)"}
        if args.cpu_sample_iters > 0:
            # the same sample on one core (the reference's assembly without coloured threads)
            threads = oracle.get_threads()
            oracle.set_threads(1)
            try:
                rate1, sec1, n1 = cpu_sample(desc, u_start, dt_start, 1)
            finally:
                oracle.set_threads(threads)
            line["cpu_baseline"]["single_core"] = {"value": rate1, "unit": UNIT,
                                                   "sample": f"first {n1} Newton iteration ({sec1:.1f} s)"}
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
