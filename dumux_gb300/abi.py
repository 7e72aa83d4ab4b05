"""ctypes mirror of the C ABI declared in include/dumux_gb300.h.

Only data layouts live here (no behaviour), so that the product wrapper and the
test-side oracle wrapper read and write the same structures.
"""
import ctypes as C

import numpy as np

DXG_OK = 0
STATUS_NAMES = {
    0: "DXG_OK", 1: "DXG_ERR_ARG", 2: "DXG_ERR_CUDA", 3: "DXG_ERR_OOM", 4: "DXG_ERR_STATE",
    5: "DXG_ERR_LINEAR_BREAKDOWN", 6: "DXG_ERR_LINEAR_NOT_CONVERGED", 7: "DXG_ERR_NAN",
    8: "DXG_ERR_NEWTON_NOT_CONVERGED", 9: "DXG_ERR_TIMEOUT", 10: "DXG_ERR_NO_DEVICE", 11: "DXG_ERR_SIZE",
    12: "DXG_ERR_BUDGET",
}
DXG_ERR_BUDGET = 12
DXG_BATCH_OPT_GRAPHS = 0
DXG_BATCH_OPT_AUTOTUNE = 1
DXG_BATCH_OPT_ILU_REDBLACK = 2
DXG_BATCH_OPT_AMG = 3
DXG_PRECISION_FP64 = 0
DXG_PRECISION_MIXED = 1
MAX_NEWTON_RECORD = 64

_dp = C.POINTER(C.c_double)


class ProblemDescC(C.Structure):
    _fields_ = [
        ("dim", C.c_int32),
        ("cells", C.c_int32 * 3),
        ("coords", _dp * 3),
        ("num_eq", C.c_int32),
        ("enable_gravity", C.c_int32),
        ("gravity", C.c_double * 3),
        ("density", C.c_double * 2),
        ("viscosity", C.c_double * 2),
        ("permeability", _dp),
        ("porosity", _dp),
        ("extrusion", _dp),
        ("material", C.POINTER(C.c_int32)),
        ("source", _dp),
        ("num_materials", C.c_int32),
        ("material_params", _dp),
        ("bc_type", C.POINTER(C.c_int8)),
        ("bc_values", _dp),
        ("base_epsilon", C.c_double),
        ("privar_magnitude", C.c_double * 2),
        ("numeric_difference_method", C.c_int32),
        ("upwind_weight", C.c_double),
        ("diff_method", C.c_int32),
        ("material_law", C.c_int32),
        ("discretization", C.c_int32),
        ("permeability_tensor", _dp),
    ]


class LinearResultC(C.Structure):
    _fields_ = [
        ("converged", C.c_int32),
        ("iterations", C.c_int32),
        ("reduction", C.c_double),
        ("initial_defect", C.c_double),
        ("final_defect", C.c_double),
    ]


class NewtonParamsC(C.Structure):
    _fields_ = [
        ("max_relative_shift", C.c_double),
        ("min_steps", C.c_int32),
        ("max_steps", C.c_int32),
        ("target_steps", C.c_int32),
        ("use_line_search", C.c_int32),
        ("line_search_min_relaxation", C.c_double),
        ("enable_residual_criterion", C.c_int32),
        ("residual_reduction", C.c_double),
        ("max_time_step_divisions", C.c_int32),
        ("retry_time_step_reduction", C.c_double),
        ("linear_reduction", C.c_double),
        ("linear_max_iter", C.c_int32),
        ("record_residual_norms", C.c_int32),
        ("enable_partial_reassembly", C.c_int32),
        ("reassembly_min_threshold", C.c_double),
        ("reassembly_max_threshold", C.c_double),
        ("reassembly_shift_weight", C.c_double),
    ]


class NewtonReportC(C.Structure):
    _fields_ = [
        ("converged", C.c_int32),
        ("iterations", C.c_int32),
        ("time_step_divisions", C.c_int32),
        ("dt_used", C.c_double),
        ("linear_iterations", C.c_int32),
        ("wasted_iterations", C.c_int32),
        ("initial_residual", C.c_double),
        ("shift", C.c_double * MAX_NEWTON_RECORD),
        ("residual_norm", C.c_double * MAX_NEWTON_RECORD),
        ("linear_iters", C.c_int32 * MAX_NEWTON_RECORD),
        ("time_assemble", C.c_double),
        ("time_solve", C.c_double),
        ("time_update", C.c_double),
    ]

    def as_dict(self):
        n = min(self.iterations, MAX_NEWTON_RECORD)
        return {
            "converged": bool(self.converged),
            "iterations": int(self.iterations),
            "time_step_divisions": int(self.time_step_divisions),
            "dt_used": float(self.dt_used),
            "linear_iterations": int(self.linear_iterations),
            "wasted_iterations": int(self.wasted_iterations),
            "initial_residual": float(self.initial_residual),
            "shift": [float(self.shift[i]) for i in range(n)],
            "residual_norm": [float(self.residual_norm[i]) for i in range(n)],
            "linear_iters": [int(self.linear_iters[i]) for i in range(n)],
            "time_assemble": float(self.time_assemble),
            "time_solve": float(self.time_solve),
            "time_update": float(self.time_update),
        }


class BatchProblemInfoC(C.Structure):
    _fields_ = [
        ("state", C.c_int32),
        ("status", C.c_int32),
        ("time_steps", C.c_int32),
        ("time_step_divisions", C.c_int32),
        ("newton_iterations", C.c_int64),
        ("linear_iterations", C.c_int64),
        ("cells", C.c_int64),
        ("time", C.c_double),
        ("seconds_admitted", C.c_double),
        ("seconds_finished", C.c_double),
    ]

    STATES = {0: "active", 1: "finished", 2: "failed"}

    def as_dict(self):
        return {
            "state": self.STATES.get(self.state, self.state),
            "status": int(self.status),
            "time_steps": int(self.time_steps),
            "time_step_divisions": int(self.time_step_divisions),
            "newton_iterations": int(self.newton_iterations),
            "linear_iterations": int(self.linear_iterations),
            "cells": int(self.cells),
            "time": float(self.time),
            "seconds_admitted": float(self.seconds_admitted),
            "seconds_finished": float(self.seconds_finished),
        }


def newton_params(**kw):
    """Reference defaults of NewtonSolver::initParams_ (dumux/nonlinear/newtonsolver.hh:1213-1247)
    and LinearSolver.ResidualReduction = 1e-6 as set by the Newton constructor (:232)."""
    p = NewtonParamsC()
    p.max_relative_shift = 1e-8
    p.min_steps = 2
    p.max_steps = 18
    p.target_steps = 10
    p.use_line_search = 0
    p.line_search_min_relaxation = 0.125
    p.enable_residual_criterion = 0
    p.residual_reduction = 1e-5
    p.max_time_step_divisions = 10
    p.retry_time_step_reduction = 0.5
    p.linear_reduction = 1e-6
    p.linear_max_iter = 250
    p.record_residual_norms = 0
    p.enable_partial_reassembly = 0
    p.reassembly_min_threshold = 0.0
    p.reassembly_max_threshold = 0.0
    p.reassembly_shift_weight = 1e-3
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p


def _ptr(a, ctype=C.c_double):
    if a is None:
        return C.cast(None, C.POINTER(ctype))
    return a.ctypes.data_as(C.POINTER(ctype))


class ProblemDesc:
    """Owns the numpy tables of a tabulated problem and exposes the C descriptor.

    Field meanings follow dxg_problem_desc in include/dumux_gb300.h.
    """

    def __init__(self, *, coords, num_eq, permeability, porosity, bc_type, bc_values,
                 enable_gravity=True, gravity=None, density=(1000.0, 1000.0),
                 viscosity=(1e-3, 1e-3), extrusion=None, material=None, source=None,
                 material_params=None, base_epsilon=1e-10, privar_magnitude=(-1.0, -1.0),
                 numeric_difference_method=1, upwind_weight=1.0, analytic=False, material_law="brooks-corey",
                 discretization="tpfa", permeability_tensor=None):
        self.coords = [np.ascontiguousarray(c, dtype=np.float64) for c in coords]
        self.dim = len(self.coords)
        self.cells = [len(c) - 1 for c in self.coords] + [1] * (3 - self.dim)
        self.num_cells = int(np.prod(self.cells))
        self.num_eq = int(num_eq)
        n = self.num_cells
        self.permeability = np.ascontiguousarray(permeability, dtype=np.float64).reshape(n)
        self.porosity = np.ascontiguousarray(porosity, dtype=np.float64).reshape(n)
        self.extrusion = None if extrusion is None else np.ascontiguousarray(extrusion, dtype=np.float64).reshape(n)
        self.material = None if material is None else np.ascontiguousarray(material, dtype=np.int32).reshape(n)
        self.source = None if source is None else np.ascontiguousarray(source, dtype=np.float64).reshape(n * self.num_eq)
        self.material_law = {"brooks-corey": 0, "van-genuchten": 1}[material_law]
        width = 5 if self.material_law == 0 else 9
        if material_params is None:
            material_params = np.zeros((1, width))
        self.material_params = np.ascontiguousarray(material_params, dtype=np.float64).reshape(-1, width)
        nb = num_boundary_faces(self.dim, self.cells)
        self.bc_type = np.ascontiguousarray(bc_type, dtype=np.int8).reshape(nb)
        self.bc_values = np.ascontiguousarray(bc_values, dtype=np.float64).reshape(nb * self.num_eq)
        self.enable_gravity = bool(enable_gravity)
        if gravity is None:
            gravity = [0.0] * 3
            gravity[self.dim - 1] = -9.81
        self.gravity = list(gravity) + [0.0] * (3 - len(gravity))
        self.density = tuple(density)
        self.viscosity = tuple(viscosity)
        self.base_epsilon = base_epsilon
        self.privar_magnitude = tuple(privar_magnitude)
        self.numeric_difference_method = numeric_difference_method
        self.upwind_weight = upwind_weight
        self.analytic = bool(analytic)
        self.discretization = {"tpfa": 0, "mpfa": 1}[discretization]
        self.permeability_tensor = (None if permeability_tensor is None else
                                    np.ascontiguousarray(permeability_tensor, dtype=np.float64)
                                    .reshape(n * self.dim * self.dim))
        self._c = None

    @property
    def c(self):
        d = ProblemDescC()
        d.dim = self.dim
        for a in range(3):
            d.cells[a] = self.cells[a]
            d.coords[a] = _ptr(self.coords[a]) if a < self.dim else _ptr(None)
        d.num_eq = self.num_eq
        d.enable_gravity = int(self.enable_gravity)
        for a in range(3):
            d.gravity[a] = self.gravity[a]
        for p in range(2):
            d.density[p] = self.density[p]
            d.viscosity[p] = self.viscosity[p]
            d.privar_magnitude[p] = self.privar_magnitude[p]
        d.permeability = _ptr(self.permeability)
        d.porosity = _ptr(self.porosity)
        d.extrusion = _ptr(self.extrusion)
        d.material = _ptr(self.material, C.c_int32)
        d.source = _ptr(self.source)
        d.num_materials = self.material_params.shape[0]
        d.material_params = _ptr(self.material_params)
        d.bc_type = _ptr(self.bc_type, C.c_int8)
        d.bc_values = _ptr(self.bc_values)
        d.base_epsilon = self.base_epsilon
        d.numeric_difference_method = self.numeric_difference_method
        d.upwind_weight = self.upwind_weight
        d.diff_method = 1 if self.analytic else 0
        d.material_law = self.material_law
        d.discretization = self.discretization
        d.permeability_tensor = _ptr(self.permeability_tensor)
        self._c = d          # keep alive while the caller uses it
        return d

    @property
    def num_dofs(self):
        return self.num_cells * self.num_eq


def side_sizes(dim, cells):
    out = []
    for f in range(2 * dim):
        a = f // 2
        cnt = 1
        for c in range(dim):
            if c != a:
                cnt *= cells[c]
        out.append(cnt)
    return out


def num_boundary_faces(dim, cells):
    return int(sum(side_sizes(dim, cells)))


def boundary_face_centers(dim, coords):
    """Face centres of all boundary faces in the order of dxg_problem_desc
    (sides -x,+x,-y,+y,-z,+z; lexicographic over the remaining axes, lower axis fastest)."""
    centers = [0.5 * (c[:-1] + c[1:]) for c in coords]
    out = []
    for f in range(2 * dim):
        a, s = divmod(f, 2)
        others = [k for k in range(dim) if k != a]
        grids = np.meshgrid(*[centers[k] for k in others], indexing="ij")
        # lexicographic with the lower axis fastest -> flatten in Fortran order
        pts = np.zeros((grids[0].size, 3))
        for gi, k in zip(grids, others):
            pts[:, k] = gi.flatten(order="F")
        pts[:, a] = coords[a][0] if s == 0 else coords[a][-1]
        out.append(pts)
    return np.concatenate(out, axis=0)


def cell_centers(coords):
    centers = [0.5 * (c[:-1] + c[1:]) for c in coords]
    dim = len(coords)
    grids = np.meshgrid(*centers, indexing="ij")
    pts = np.zeros((grids[0].size, 3))
    for a in range(dim):
        pts[:, a] = grids[a].flatten(order="F")
    return pts
