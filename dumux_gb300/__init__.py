"""GB300-native cell-centred TPFA porous-flow hot path (residual/Jacobian assembly by
numeric differentiation, Newton, ILU(0)-preconditioned BiCGSTAB) behind the C ABI of
include/dumux_gb300.h.

The compute path is the CUDA library dumux_gb300/_lib/libdumux_gb300.so (built by
dumux_gb300/build.py).  There is no CPU fallback: every entry point raises when the
library or a CUDA device is missing.

Python mirror of the reference interfaces (same method names and meaning):
    FVAssembler            dumux/assembly/fvassembler.hh
    ILUBiCGSTABIstlSolver  dumux/linear/istlsolvers.hh:635-642
    NewtonSolver           dumux/nonlinear/newtonsolver.hh
"""
import ctypes as C
import os

import numpy as np

from .abi import (DXG_BATCH_OPT_AMG, DXG_BATCH_OPT_AUTOTUNE, DXG_BATCH_OPT_GRAPHS, DXG_BATCH_OPT_ILU_REDBLACK,
                  DXG_ERR_BUDGET,
                  DXG_PRECISION_FP64, DXG_PRECISION_MIXED, STATUS_NAMES, BatchProblemInfoC, LinearResultC, NewtonParamsC, NewtonReportC,
                  ProblemDesc, ProblemDescC, newton_params)

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libdumux_gb300.so")
_lib = None


class DxgError(RuntimeError):
    def __init__(self, status, msg=""):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")


class NumericalProblem(DxgError):
    """Recoverable failure (linear breakdown / non-convergence), Dumux::NumericalProblem."""


def lib():
    """Loads the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run dumux_gb300/build.py (nvcc, sm_103a)")
        L = C.CDLL(LIB_PATH)
        dp = C.POINTER(C.c_double)
        vp = C.c_void_p
        L.dxg_num_boundary_faces.argtypes = [C.POINTER(ProblemDescC)]
        L.dxg_num_boundary_faces.restype = C.c_int64
        L.dxg_ctx_create.argtypes = [C.POINTER(vp), C.c_int]
        L.dxg_ctx_destroy.argtypes = [vp]
        L.dxg_last_error.argtypes = [vp]
        L.dxg_last_error.restype = C.c_char_p
        L.dxg_set_precision.argtypes = [vp, C.c_int]
        L.dxg_problem_upload.argtypes = [vp, C.POINTER(ProblemDescC)]
        L.dxg_sizes.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int32), C.POINTER(C.c_int64)]
        for name in ("dxg_set_solution", "dxg_get_solution", "dxg_set_prev_solution", "dxg_get_residual",
                     "dxg_get_update"):
            getattr(L, name).argtypes = [vp, dp]
        L.dxg_set_time_step.argtypes = [vp, C.c_double]
        L.dxg_assemble_jacobian_and_residual.argtypes = [vp]
        L.dxg_assemble_residual.argtypes = [vp]
        L.dxg_get_jacobian.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int32), dp]
        L.dxg_set_linear_system.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int32), dp, dp]
        L.dxg_linear_solve.argtypes = [vp, C.c_double, C.c_int32, C.POINTER(LinearResultC)]
        L.dxg_residual_norm.argtypes = [vp, dp]
        L.dxg_newton_default_params.argtypes = [C.POINTER(NewtonParamsC)]
        L.dxg_newton_default_params.restype = None
        L.dxg_newton_solve.argtypes = [vp, C.c_double, C.POINTER(NewtonParamsC), C.POINTER(NewtonReportC)]
        L.dxg_suggest_time_step.argtypes = [vp, C.c_double, C.POINTER(NewtonParamsC)]
        L.dxg_suggest_time_step.restype = C.c_double
        L.dxg_advance_time_step.argtypes = [vp]
        L.dxg_set_lane_ring.argtypes = [vp, C.c_int]
        L.dxg_set_ilu_kernel.argtypes = [vp, C.c_int]
        L.dxg_set_wait_limit.argtypes = [vp, C.c_double]
        L.dxg_set_linear_solver.argtypes = [vp, C.c_int]
        L.dxg_stream_handle.argtypes = [vp]
        L.dxg_stream_handle.restype = C.c_void_p
        L.dxg_set_kernel_timing.argtypes = [vp, C.c_int]
        L.dxg_get_kernel_timing.argtypes = [vp, C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_double),
                                            C.POINTER(C.c_double)]
        L.dxg_kernel_launch_count.argtypes = [vp]
        L.dxg_kernel_launch_count.restype = C.c_int64
        L.dxg_sync.argtypes = [vp]
        L.dxg_batch_create.argtypes = [C.POINTER(vp), C.c_int, C.c_int]
        L.dxg_batch_destroy.argtypes = [vp]
        L.dxg_batch_last_error.argtypes = [vp]
        L.dxg_batch_last_error.restype = C.c_char_p
        L.dxg_batch_set_option.argtypes = [vp, C.c_int, C.c_int]
        L.dxg_problem_device_bytes.argtypes = [C.POINTER(ProblemDescC), C.c_int]
        L.dxg_problem_device_bytes.restype = C.c_int64
        L.dxg_batch_set_memory_budget.argtypes = [vp, C.c_int64]
        L.dxg_batch_device_bytes.argtypes = [vp]
        L.dxg_batch_device_bytes.restype = C.c_int64
        L.dxg_batch_add.argtypes = [vp, C.POINTER(ProblemDescC), dp, C.c_double, C.c_double, C.c_double,
                                    C.POINTER(NewtonParamsC), C.POINTER(C.c_int64)]
        L.dxg_batch_iterate.argtypes = [vp, C.POINTER(C.c_int32)]
        L.dxg_batch_run.argtypes = [vp]
        L.dxg_batch_info.argtypes = [vp, C.c_int64, C.POINTER(BatchProblemInfoC)]
        L.dxg_batch_get_solution.argtypes = [vp, C.c_int64, dp]
        L.dxg_batch_remove.argtypes = [vp, C.c_int64]
        L.dxg_batch_launch_count.argtypes = [vp]
        L.dxg_batch_launch_count.restype = C.c_int64
        L.dxg_batch_set_kernel_timing.argtypes = [vp, C.c_int]
        L.dxg_batch_get_kernel_timing.argtypes = [vp, C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_double),
                                                  C.POINTER(C.c_double)]
        L.dxg_selftest_bounded_wait.argtypes = [C.c_int, C.c_int32, C.c_int64, C.POINTER(C.c_int32),
                                                C.POINTER(C.c_double)]
        L.dxg_device_pow.argtypes = [C.c_int, dp, dp, dp, C.c_int64]
        L.dxg_fp64_fma_rate.argtypes = [C.c_int, dp]
        L.dxg_batch_describe.argtypes = [vp, C.c_char_p, C.c_int64]
        L.dxg_describe.argtypes = [vp, C.c_char_p, C.c_int64]
        L.dxg_batch_stream.argtypes = [vp]
        L.dxg_batch_stream.restype = C.c_void_p
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Context:
    """One problem resident on one GPU (dxg_ctx)."""

    def __init__(self, desc=None, device=0, precision="fp64"):
        L = lib()
        h = C.c_void_p()
        st = L.dxg_ctx_create(C.byref(h), int(device))
        if st != 0:
            raise DxgError(st, L.dxg_last_error(None).decode())
        self._h = h
        self._L = L
        prec = {"fp64": DXG_PRECISION_FP64, "mixed": DXG_PRECISION_MIXED}[precision]
        self._check(L.dxg_set_precision(h, prec))
        self.precision = precision
        self.desc = None
        if desc is not None:
            self.upload(desc)

    def _check(self, st, recoverable=False):
        if st != 0:
            msg = self._L.dxg_last_error(self._h).decode()
            if recoverable and st in (5, 6, 7, 8):
                raise NumericalProblem(st, msg)
            raise DxgError(st, msg)

    def close(self):
        if getattr(self, "_h", None):
            self._L.dxg_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- problem / state ---------------------------------------------------------
    def upload(self, desc):
        self.desc = desc
        d = desc.c
        self._check(self._L.dxg_problem_upload(self._h, C.byref(d)))
        n = C.c_int64(); b = C.c_int32(); nnzb = C.c_int64()
        self._check(self._L.dxg_sizes(self._h, C.byref(n), C.byref(b), C.byref(nnzb)))
        self.num_cells, self.num_eq, self.num_blocks = n.value, b.value, nnzb.value
        self.num_dofs = self.num_cells * self.num_eq

    def _vec(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
        if a.size != self.num_dofs:
            raise ValueError(f"expected {self.num_dofs} values, got {a.size}")
        return a

    def set_solution(self, u):
        self._check(self._L.dxg_set_solution(self._h, _dp(self._vec(u))))

    def solution(self):
        out = np.empty(self.num_dofs)
        self._check(self._L.dxg_get_solution(self._h, _dp(out)))
        return out

    def set_prev_solution(self, u):
        self._check(self._L.dxg_set_prev_solution(self._h, _dp(self._vec(u))))

    def set_time_step(self, dt):
        self._check(self._L.dxg_set_time_step(self._h, float(dt)))

    def advance_time_step(self):
        self._check(self._L.dxg_advance_time_step(self._h))

    # -- assembler ---------------------------------------------------------------
    def assemble_jacobian_and_residual(self):
        self._check(self._L.dxg_assemble_jacobian_and_residual(self._h), recoverable=True)

    def assemble_residual(self):
        self._check(self._L.dxg_assemble_residual(self._h), recoverable=True)

    def residual(self):
        out = np.empty(self.num_dofs)
        self._check(self._L.dxg_get_residual(self._h, _dp(out)))
        return out

    def jacobian(self):
        """(row_ptr, col_idx, values) in BCRS layout, blocks row-major."""
        b = self.num_eq
        row_ptr = np.empty(self.num_cells + 1, dtype=np.int64)
        col = np.empty(self.num_blocks, dtype=np.int32)
        vals = np.empty(self.num_blocks * b * b)
        self._check(self._L.dxg_get_jacobian(self._h, row_ptr.ctypes.data_as(C.POINTER(C.c_int64)),
                                             col.ctypes.data_as(C.POINTER(C.c_int32)), _dp(vals)))
        return row_ptr, col, vals

    def set_linear_system(self, row_ptr, col, vals, rhs):
        row_ptr = np.ascontiguousarray(row_ptr, dtype=np.int64)
        col = np.ascontiguousarray(col, dtype=np.int32)
        vals = np.ascontiguousarray(vals, dtype=np.float64)
        self._check(self._L.dxg_set_linear_system(self._h, row_ptr.ctypes.data_as(C.POINTER(C.c_int64)),
                                                  col.ctypes.data_as(C.POINTER(C.c_int32)), _dp(vals),
                                                  _dp(self._vec(rhs))))

    # -- linear solver -----------------------------------------------------------
    def linear_solve(self, reduction=1e-13, max_iter=250, raise_on_failure=False):
        res = LinearResultC()
        st = self._L.dxg_linear_solve(self._h, float(reduction), int(max_iter), C.byref(res))
        if st not in (0, 6) or (raise_on_failure and st != 0):
            self._check(st, recoverable=True)
        return {"converged": bool(res.converged), "iterations": res.iterations, "reduction": res.reduction,
                "initial_defect": res.initial_defect, "final_defect": res.final_defect}

    def update(self):
        out = np.empty(self.num_dofs)
        self._check(self._L.dxg_get_update(self._h, _dp(out)))
        return out

    def residual_norm(self):
        v = C.c_double()
        self._check(self._L.dxg_residual_norm(self._h, C.byref(v)))
        return v.value

    # -- Newton ------------------------------------------------------------------
    def newton_solve(self, dt=0.0, params=None, raise_on_failure=True):
        p = params if params is not None else newton_params()
        rep = NewtonReportC()
        st = self._L.dxg_newton_solve(self._h, float(dt), C.byref(p), C.byref(rep))
        if st != 0 and raise_on_failure:
            self._check(st, recoverable=True)
        out = rep.as_dict()
        out["status"] = st
        return out

    def suggest_time_step(self, old_dt, params=None):
        p = params if params is not None else newton_params()
        return self._L.dxg_suggest_time_step(self._h, float(old_dt), C.byref(p))

    def set_lane_ring(self, form):
        """Form of the lane sweeps: 'auto' (timed at the first factorisation), 'registers' or
        'ring' (shared-memory prefetch ring); both give the same bits."""
        self._check(self._L.dxg_set_lane_ring(self._h, {"auto": 0, "registers": 1, "ring": 2}[form]))

    def set_ilu_kernel(self, kind):
        """'auto' / 'wavefront' (one cluster launch per sweep), 'lanes' (two lanes per grid line,
        one plane per CTA over several clusters; 3D 2x2 blocks) or 'levels' (one launch per
        level): the natural-order ILU(0) of the reference; 'redblack': ILU(0) of the red-black
        reordered matrix (a different preconditioner, two parallel passes per sweep)."""
        self._check(self._L.dxg_set_ilu_kernel(self._h, {"auto": 0, "wavefront": 1, "levels": 2,
                                                          "redblack": 3, "lanes": 4}[kind]))

    def set_wait_limit(self, seconds):
        """Limit of every bounded wait inside the ILU(0) sweeps (dxg_set_wait_limit)."""
        self._check(self._L.dxg_set_wait_limit(self._h, float(seconds)))

    def set_linear_solver(self, kind):
        """'ilu' (ILU(0)-BiCGSTAB, the default) or 'amg' (BiCGSTAB preconditioned by one
        V-cycle of the aggregation AMG, the reference's AMGBiCGSTAB solver type)."""
        self._check(self._L.dxg_set_linear_solver(self._h, {"ilu": 0, "amg": 1}[kind]))

    def stream_handle(self):
        """cudaStream_t of this context (as an int) for event timing by the caller."""
        return int(self._L.dxg_stream_handle(self._h) or 0)

    def set_kernel_timing(self, enable=True):
        self._check(self._L.dxg_set_kernel_timing(self._h, int(bool(enable))))

    def kernel_timing(self, kind):
        """(launches, total device ms, algorithmic bytes) of 'ilu_sweep' / 'assembly' / 'spmv' /
        'ilu_factor'."""
        k = {"ilu_sweep": 0, "assembly": 1, "spmv": 2, "ilu_factor": 3}[kind]
        n = C.c_int64(); ms = C.c_double(); by = C.c_double()
        self._check(self._L.dxg_get_kernel_timing(self._h, k, C.byref(n), C.byref(ms), C.byref(by)))
        return n.value, ms.value, by.value

    def describe(self):
        """The ILU(0) kernels in use and, once tuned, the time of every launch shape tried."""
        buf = C.create_string_buffer(1024)
        self._check(self._L.dxg_describe(self._h, buf, len(buf)))
        return buf.value.decode()

    def kernel_launches(self):
        return int(self._L.dxg_kernel_launch_count(self._h))

    def sync(self):
        self._check(self._L.dxg_sync(self._h))


# ---------------------------------------------------------------- reference-named mirror
class FVAssembler:
    """dumux/assembly/fvassembler.hh:101-662 over a device-resident problem."""

    def __init__(self, desc, prev_sol=None, dt=None, device=0, precision="fp64"):
        self.ctx = Context(desc, device=device, precision=precision)
        if prev_sol is not None:
            self.set_previous_solution(prev_sol)
        if dt is not None:
            self.ctx.set_time_step(dt)

    def is_stationary_problem(self):
        return self.ctx.desc is not None and not hasattr(self, "_dt")

    def set_previous_solution(self, u):
        self.ctx.set_prev_solution(u)

    def assemble_jacobian_and_residual(self, u):
        self.ctx.set_solution(u)
        self.ctx.assemble_jacobian_and_residual()

    def assemble_residual(self, u):
        self.ctx.set_solution(u)
        self.ctx.assemble_residual()

    def jacobian(self):
        return self.ctx.jacobian()

    def residual(self):
        return self.ctx.residual()

    assembleJacobianAndResidual = assemble_jacobian_and_residual
    assembleResidual = assemble_residual


class ILUBiCGSTABIstlSolver:
    """dumux/linear/istlsolvers.hh:635-642: ILU(0)-preconditioned BiCGSTAB."""

    def __init__(self, residual_reduction=1e-13, max_iter=250):
        self.reduction = residual_reduction
        self.max_iter = max_iter

    def set_residual_reduction(self, r):
        self.reduction = r

    def set_max_iter(self, n):
        self.max_iter = n

    def solve(self, assembler):
        """Solves the assembler's J x = r on the device; returns (converged, x)."""
        res = assembler.ctx.linear_solve(self.reduction, self.max_iter)
        return res["converged"], assembler.ctx.update()

    def norm(self, assembler):
        return assembler.ctx.residual_norm()

    setResidualReduction = set_residual_reduction


class NewtonSolver:
    """dumux/nonlinear/newtonsolver.hh: solve(x, dt) with dt halving, solve(x) stationary."""

    def __init__(self, assembler, linear_solver=None, **params):
        self.assembler = assembler
        self.params = newton_params(**params)
        if linear_solver is not None:
            self.params.linear_max_iter = linear_solver.max_iter
        self.last_report = None

    def solve(self, u, dt=0.0):
        ctx = self.assembler.ctx
        ctx.set_solution(u)
        self.last_report = ctx.newton_solve(dt, self.params)
        return ctx.solution()

    def suggest_time_step_size(self, old_dt):
        return self.assembler.ctx.suggest_time_step(old_dt, self.params)

    suggestTimeStepSize = suggest_time_step_size


def selftest_bounded_wait(kind="mbarrier", limit_ms=2.0, device=0):
    """Runs the sweeps' bounded wait on a condition nothing satisfies (dxg_selftest_bounded_wait);
    returns (kernel status name, milliseconds waited).  The expected status is DXG_ERR_TIMEOUT."""
    k = {"mbarrier": 0, "flag": 1}[kind]
    st = C.c_int32(-1)
    ms = C.c_double(0.0)
    rc = lib().dxg_selftest_bounded_wait(int(device), k, int(limit_ms * 1e6), C.byref(st), C.byref(ms))
    if rc != 0:
        raise DxgError(rc, "bounded-wait self-test did not run")
    return STATUS_NAMES.get(st.value, st.value), ms.value


def device_pow(x, y, device=0):
    """pow(x, y) element-wise on the device with the material laws' correctly rounded pow
    (dxg_device_pow); y broadcasts against x."""
    import numpy as np
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(np.broadcast_to(y, x.shape), dtype=np.float64)
    out = np.empty_like(x)
    rc = lib().dxg_device_pow(int(device), _dp(x), _dp(y), _dp(out), x.size)
    if rc != 0:
        raise DxgError(rc, "dxg_device_pow failed")
    return out


def fp64_fma_rate(device=0):
    """Dense FP64 FMA rate of the device in TFLOP/s (dxg_fp64_fma_rate)."""
    v = C.c_double(0.0)
    rc = lib().dxg_fp64_fma_rate(int(device), C.byref(v))
    if rc != 0:
        raise DxgError(rc, "dxg_fp64_fma_rate failed")
    return v.value


def problem_device_bytes(desc, precision="mixed"):
    """Device memory a problem takes once admitted (dxg_problem_device_bytes)."""
    prec = {"fp64": DXG_PRECISION_FP64, "mixed": DXG_PRECISION_MIXED}[precision]
    return int(lib().dxg_problem_device_bytes(C.byref(desc.c), prec))


class Batch:
    """Many independent problems advanced together on one GPU (dxg_batch).

    add() admits a problem (refused with DXG_ERR_BUDGET beyond the memory budget),
    iterate() runs one Newton iteration of every active problem, run() iterates until
    none is active.  Each problem follows its own time loop; its result does not
    depend on what else is in the batch.
    """

    def __init__(self, device=0, precision="mixed", graphs=True, autotune=True, memory_budget=0, ilu="natural",
                 solver="ilu"):
        L = lib()
        h = C.c_void_p()
        prec = {"fp64": DXG_PRECISION_FP64, "mixed": DXG_PRECISION_MIXED}[precision]
        st = L.dxg_batch_create(C.byref(h), int(device), prec)
        if st != 0:
            raise DxgError(st, L.dxg_batch_last_error(None).decode())
        self._h = h
        self._L = L
        self.precision = precision
        self._sizes = {}
        self._check(L.dxg_batch_set_option(h, DXG_BATCH_OPT_GRAPHS, int(bool(graphs))))
        self._check(L.dxg_batch_set_option(h, DXG_BATCH_OPT_AUTOTUNE, int(bool(autotune))))
        self._check(L.dxg_batch_set_option(h, DXG_BATCH_OPT_ILU_REDBLACK,
                                           {"natural": 0, "redblack": 1}[ilu]))
        self._check(L.dxg_batch_set_option(h, DXG_BATCH_OPT_AMG, {"ilu": 0, "amg": 1}[solver]))
        self._check(L.dxg_batch_set_memory_budget(h, int(memory_budget)))

    def _check(self, st):
        if st != 0:
            raise DxgError(st, self._L.dxg_batch_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._L.dxg_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, desc, u0, dt=0.0, t_end=0.0, params=None, max_dt=None):
        """Admits a problem; returns its id, or None when the memory budget refuses it.
        dt: initial time step; max_dt: TimeLoop.MaxTimeStepSize (default: dt, i.e. fixed
        steps unless Newton asks for smaller ones; 0: unlimited)."""
        u0 = np.ascontiguousarray(u0, dtype=np.float64).reshape(-1)
        if u0.size != desc.num_dofs:
            raise ValueError(f"u0 has {u0.size} entries, expected {desc.num_dofs}")
        p = params if params is not None else newton_params()
        pid = C.c_int64()
        mdt = float(dt) if max_dt is None else float(max_dt)
        st = self._L.dxg_batch_add(self._h, C.byref(desc.c), _dp(u0), float(dt), mdt, float(t_end), C.byref(p),
                                   C.byref(pid))
        if st == DXG_ERR_BUDGET:
            return None
        self._check(st)
        self._sizes[pid.value] = desc.num_dofs
        return pid.value

    def iterate(self):
        n = C.c_int32()
        self._check(self._L.dxg_batch_iterate(self._h, C.byref(n)))
        return n.value

    def run(self):
        self._check(self._L.dxg_batch_run(self._h))

    def info(self, pid):
        i = BatchProblemInfoC()
        self._check(self._L.dxg_batch_info(self._h, int(pid), C.byref(i)))
        return i.as_dict()

    def solution(self, pid):
        u = np.empty(self._sizes[pid], dtype=np.float64)
        self._check(self._L.dxg_batch_get_solution(self._h, int(pid), _dp(u)))
        return u

    def remove(self, pid):
        self._check(self._L.dxg_batch_remove(self._h, int(pid)))
        self._sizes.pop(pid, None)

    def device_bytes(self):
        return int(self._L.dxg_batch_device_bytes(self._h))

    def set_memory_budget(self, nbytes):
        self._check(self._L.dxg_batch_set_memory_budget(self._h, int(nbytes)))

    def kernel_launches(self):
        return int(self._L.dxg_batch_launch_count(self._h))

    def stream_handle(self):
        return self._L.dxg_batch_stream(self._h)

    def describe(self):
        """The groups of problems and their ILU(0) sweep launch shapes."""
        buf = C.create_string_buffer(8192)
        self._check(self._L.dxg_batch_describe(self._h, buf, len(buf)))
        return buf.value.decode()

    def set_kernel_timing(self, enable=True):
        self._check(self._L.dxg_batch_set_kernel_timing(self._h, int(bool(enable))))

    def kernel_timing(self, kind):
        """(launches, device ms, algorithmic bytes) of 'ilu_sweep', 'assembly', 'spmv' or 'ilu_factor'."""
        kc = {"ilu_sweep": 0, "assembly": 1, "spmv": 2, "ilu_factor": 3}[kind]
        n = C.c_int64(); ms = C.c_double(); by = C.c_double()
        self._check(self._L.dxg_batch_get_kernel_timing(self._h, kc, C.byref(n), C.byref(ms), C.byref(by)))
        return n.value, ms.value, by.value


__all__ = ["Context", "FVAssembler", "ILUBiCGSTABIstlSolver", "NewtonSolver", "ProblemDesc", "newton_params",
           "DxgError", "NumericalProblem", "lib", "LIB_PATH", "Batch", "problem_device_bytes",
           "selftest_bounded_wait", "device_pow", "fp64_fma_rate"]
