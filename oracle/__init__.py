"""ctypes wrapper of the CPU oracle.  TEST INFRASTRUCTURE ONLY.

Used by tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py as the
checker for the product's CUDA path.  The product package never imports this module.
"""
import ctypes as C
import os

import numpy as np

from dumux_gb300.abi import LinearResultC, NewtonReportC, ProblemDescC, NewtonParamsC, newton_params

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        dp = C.POINTER(C.c_double)
        i64p = C.POINTER(C.c_int64)
        i32p = C.POINTER(C.c_int32)
        PD = C.POINTER(ProblemDescC)
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_set_pow_mode.argtypes = [C.c_int]
        L.orc_set_linear_threads.argtypes = [C.c_int]
        L.orc_set_dot_order.argtypes = [C.c_int]
        L.orc_get_pow_mode.restype = C.c_int
        L.orc_pow_batch.argtypes = [C.c_int32, C.c_int64, dp, dp, dp]
        L.orc_get_threads.restype = C.c_int
        L.orc_num_blocks.argtypes = [PD, i64p]
        L.orc_pattern.argtypes = [PD, i64p, i32p]
        L.orc_assemble.argtypes = [PD, dp, dp, C.c_double, dp, dp]
        L.orc_linear_solve.argtypes = [C.c_int64, C.c_int32, i64p, i32p, dp, dp, dp, C.c_double, C.c_int32,
                                       C.POINTER(LinearResultC)]
        L.orc_newton_solve.argtypes = [PD, dp, dp, C.c_double, C.POINTER(NewtonParamsC), C.POINTER(NewtonReportC)]
        L.orc_suggest_time_step.argtypes = [C.c_int32, C.c_double, C.POINTER(NewtonParamsC)]
        L.orc_suggest_time_step.restype = C.c_double
        L.orc_brooks_corey.argtypes = [dp, C.c_int32, C.c_int64, dp, dp]
        L.orc_van_genuchten.argtypes = [dp, C.c_int32, C.c_int64, dp, dp]
        L.orc_numdiff_poly.argtypes = [C.c_int32, C.c_double, C.c_double]
        L.orc_numdiff_poly.restype = C.c_double
        L.orc_newton_scalar.argtypes = [C.c_double, C.POINTER(NewtonParamsC), dp, i32p]
        _lib = L
    return _lib


def _dp(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def set_threads(n):
    lib().orc_set_threads(int(n))


def get_threads():
    return lib().orc_get_threads()


def set_linear_threads(n):
    """Threads of the oracle's linear solve: 1 (default) sequential as dune-istl, 0 all host
    threads (level-scheduled ILU(0), row-parallel SpMV; results identical bit for bit)."""
    lib().orc_set_linear_threads(int(n))


def set_dot_order(order):
    """Summation order of the oracle's dot products: 0 sequential (dune-istl), 1 blocked."""
    lib().orc_set_dot_order(int(order))


POW_LIBM, POW_CORRECTLY_ROUNDED = 0, 1


def set_pow_mode(mode):
    """pow of the material laws: POW_LIBM (the C library's pow, as the reference calls it;
    the default) or POW_CORRECTLY_ROUNDED (the device's correctly rounded pow)."""
    lib().orc_set_pow_mode(int(mode))


def get_pow_mode():
    return lib().orc_get_pow_mode()


class pow_mode:
    """Context manager selecting the oracle's pow for a block of calls."""

    def __init__(self, mode):
        self.mode = mode

    def __enter__(self):
        self.prev = get_pow_mode()
        set_pow_mode(self.mode)
        return self

    def __exit__(self, *exc):
        set_pow_mode(self.prev)


def pow_batch(x, y, mode):
    """Element-wise pow(x, y) in the given mode (broadcast y)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(np.broadcast_to(y, x.shape), dtype=np.float64)
    out = np.empty_like(x)
    lib().orc_pow_batch(int(mode), x.size, _dp(x), _dp(y), _dp(out))
    return out


def pattern(desc):
    L = lib()
    d = desc.c
    nnzb = C.c_int64()
    assert L.orc_num_blocks(C.byref(d), C.byref(nnzb)) == 0
    row_ptr = np.zeros(desc.num_cells + 1, dtype=np.int64)
    col = np.zeros(nnzb.value, dtype=np.int32)
    assert L.orc_pattern(C.byref(d), row_ptr.ctypes.data_as(C.POINTER(C.c_int64)),
                         col.ctypes.data_as(C.POINTER(C.c_int32))) == 0
    return row_ptr, col


def assemble(desc, u, u_prev=None, dt=0.0, jacobian=True):
    """Residual r (N*b) and, if requested, BCRS values (nnzb*b*b) at u."""
    L = lib()
    d = desc.c
    b = desc.num_eq
    row_ptr, col = pattern(desc)
    u = np.ascontiguousarray(u, dtype=np.float64)
    up = None if u_prev is None else np.ascontiguousarray(u_prev, dtype=np.float64)
    r = np.zeros(desc.num_dofs)
    vals = np.zeros(len(col) * b * b) if jacobian else None
    st = L.orc_assemble(C.byref(d), _dp(u), _dp(up), float(dt), _dp(vals), _dp(r))
    assert st == 0, st
    return (row_ptr, col, vals, r) if jacobian else r


def linear_solve(row_ptr, col, vals, rhs, b, reduction=1e-13, max_iter=250):
    L = lib()
    n = len(row_ptr) - 1
    x = np.zeros(n * b)
    res = LinearResultC()
    st = L.orc_linear_solve(n, b, row_ptr.ctypes.data_as(C.POINTER(C.c_int64)),
                            col.ctypes.data_as(C.POINTER(C.c_int32)), _dp(np.ascontiguousarray(vals)),
                            _dp(np.ascontiguousarray(rhs)), _dp(x), reduction, max_iter, C.byref(res))
    return st, x, res


def newton_solve(desc, u, u_prev=None, dt=0.0, params=None):
    """One Newton solve; returns (status, u_new, report dict)."""
    L = lib()
    d = desc.c
    p = params if params is not None else newton_params()
    x = np.array(u, dtype=np.float64, copy=True)
    up = None if u_prev is None else np.ascontiguousarray(u_prev, dtype=np.float64)
    rep = NewtonReportC()
    st = L.orc_newton_solve(C.byref(d), _dp(x), _dp(up), float(dt), C.byref(p), C.byref(rep))
    return st, x, rep.as_dict()


def suggest_time_step(newton_iterations, old_dt, params=None):
    p = params if params is not None else newton_params()
    return lib().orc_suggest_time_step(int(newton_iterations), float(old_dt), C.byref(p))


def brooks_corey(params5, what, sw):
    sw = np.ascontiguousarray(sw, dtype=np.float64)
    out = np.zeros_like(sw)
    prm = np.ascontiguousarray(params5, dtype=np.float64)
    lib().orc_brooks_corey(_dp(prm), {"pc": 0, "krw": 1, "krn": 2}[what], len(sw), _dp(sw), _dp(out))
    return out


def van_genuchten(params9, what, sw):
    """Regularised Van Genuchten: what in pc, krw, krn, dpc_dsw, dkrw_dsw, dkrn_dsw."""
    sw = np.ascontiguousarray(sw, dtype=np.float64)
    prm = np.ascontiguousarray(params9, dtype=np.float64)
    out = np.zeros_like(sw)
    k = ["pc", "krw", "krn", "dpc_dsw", "dkrw_dsw", "dkrn_dsw"].index(what)
    assert lib().orc_van_genuchten(_dp(prm), k, sw.size, _dp(sw), _dp(out)) == 0
    return out


def numdiff_poly(method, eps, x0):
    return lib().orc_numdiff_poly(int(method), float(eps), float(x0))


def newton_scalar(x0, **kw):
    p = newton_params(**kw)
    x = C.c_double()
    it = C.c_int32()
    st = lib().orc_newton_scalar(float(x0), C.byref(p), C.byref(x), C.byref(it))
    return st, x.value, it.value


def time_loop(desc, u0, dt, num_steps, params=None, max_dt=None, t_end=None):
    """Implicit-Euler time loop with fixed or suggested steps (TimeLoop semantics:
    dt_{n+1} = min(suggestTimeStepSize(dt_n), MaxTimeStepSize, tEnd - t)).
    Returns (u, list of per-step reports)."""
    p = params if params is not None else newton_params()
    u = np.array(u0, dtype=np.float64, copy=True)
    reports = []
    t = 0.0
    for _ in range(num_steps):
        u_prev = u.copy()
        st, u, rep = newton_solve(desc, u, u_prev, dt, p)
        if st != 0:
            raise RuntimeError(f"oracle Newton failed with status {st}")
        t += rep["dt_used"]
        rep["time"] = t
        reports.append(rep)
        dt = suggest_time_step(rep["iterations"], rep["dt_used"], p)
        if max_dt is not None:
            dt = min(dt, max_dt)
        if t_end is not None:
            if t >= t_end:
                break
            dt = min(dt, t_end - t)
    return u, reports
