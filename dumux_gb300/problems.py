"""Tabulated problems: the reference's test problems and the benchmark workloads.

Each builder evaluates the problem's ``*AtPos`` callbacks at cell and face centres and
returns a :class:`dumux_gb300.abi.ProblemDesc` (the input of ``dxg_problem_upload``)
plus the initial solution.
"""
import numpy as np

from .abi import ProblemDesc, boundary_face_centers, cell_centers, num_boundary_faces

# SimpleH2O (dumux/material/components/simpleh2o.hh:265-267, 309) and
# Trichloroethene (dumux/material/components/trichloroethene.hh:148-171)
WATER_DENSITY, WATER_VISCOSITY = 1000.0, 1e-3
DNAPL_DENSITY, DNAPL_VISCOSITY = 1460.0, 5.7e-4


def equidistant(lower, upper, cells):
    """Vertex coordinates of a YaspGrid with EquidistantOffsetCoordinates: x_i = lower + i*h."""
    h = (upper - lower) / cells
    return lower + np.arange(cells + 1, dtype=np.float64) * h


def onep_lens_problem(cells=(10, 10), numeric_epsilon=True, discretization="tpfa"):
    """test/porousmediumflow/1p/incompressible (problem.hh, spatialparams.hh, params.input):
    unit square, lens [0.2,0.8]^2 with K=1e-12 in K=1e-10, Dirichlet top/bottom with
    p = 1e5 - 1e5*(y - ymax), no-flow left/right, gravity on, stationary.  With
    discretization="mpfa" it is the reference's test_1p_incompressible_mpfa, which compares
    against the same reference solution as the TPFA test (CMakeLists.txt:41-51)."""
    coords = [equidistant(0.0, 1.0, n) for n in cells]
    cc = cell_centers(coords)
    eps = 1.5e-7
    lens_lo, lens_hi = (0.2, 0.2), (0.8, 0.8)
    in_lens = np.ones(len(cc), dtype=bool)
    for a in range(2):
        in_lens &= (cc[:, a] >= lens_lo[a] + eps) & (cc[:, a] <= lens_hi[a] - eps)
    K = np.where(in_lens, 1e-12, 1e-10)
    fc = boundary_face_centers(2, coords)
    ymax = coords[1][-1]
    dirichlet = (fc[:, 1] < 1e-6) | (fc[:, 1] > ymax - 1e-6)
    bc_type = np.where(dirichlet, 1, 2).astype(np.int8)
    bc_values = np.where(dirichlet, 1.0e5 + (-1.0e5) * (fc[:, 1] - ymax), 0.0)
    desc = ProblemDesc(coords=coords, num_eq=1, permeability=K, porosity=np.full(len(cc), 0.4),
                       bc_type=bc_type, bc_values=bc_values, enable_gravity=True,
                       density=(WATER_DENSITY, WATER_DENSITY), viscosity=(WATER_VISCOSITY, WATER_VISCOSITY),
                       base_epsilon=0.1 if numeric_epsilon else 1e-10,
                       privar_magnitude=(1e5, -1.0) if numeric_epsilon else (-1.0, -1.0),
                       discretization=discretization)
    return desc, np.zeros(desc.num_dofs)


# test/porousmediumflow/1p/convergence/analyticsolution: omega = pi (spatialparams.hh:70)
_CONV_OMEGA = np.pi


def mpfa_convergence_exact(x, y):
    """Pressure of the analytic solution (problem.hh:125-139): (e^(y+1) + 2 - e^2) sin(w x) + 10."""
    return (np.exp(y + 1.0) + 2.0 - np.exp(2.0)) * np.sin(_CONV_OMEGA * x) + 10.0


def mpfa_convergence_problem(cells=10, c=0.9, discretization="mpfa"):
    """test/porousmediumflow/1p/convergence/analyticsolution (problem.hh, spatialparams.hh,
    params.input, properties.hh): unit square with `cells` x `cells` cells, the full
    permeability tensor K = [[1, -c/(2w) sin(w x)], [., e^-2 (1 + c cos(w x))]] at the cell
    centres, the source term of the analytic solution at the cell centres, Dirichlet values
    of the analytic solution at every boundary face centre, no gravity, a constant liquid of
    density 1 and kinematic viscosity 1 (dynamic viscosity 1).  Returns the description, the
    zero initial solution and the exact pressures at the cell centres."""
    coords = [equidistant(0.0, 1.0, cells) for _ in range(2)]
    cc = cell_centers(coords)
    x, y = cc[:, 0], cc[:, 1]
    w = _CONV_OMEGA
    K = np.zeros((len(cc), 2, 2))
    K[:, 0, 0] = 1.0
    K[:, 0, 1] = -c / (2 * w) * np.sin(w * x)
    K[:, 1, 0] = K[:, 0, 1]
    K[:, 1, 1] = np.exp(-2.0) * (1.0 + c * np.cos(w * x))
    cosx = np.cos(w * x)
    src = (-(c * cosx + 1.0) * np.exp(y - 1.0) + 1.5 * c * np.exp(y + 1.0) * cosx
           + w * w * (np.exp(y + 1.0) - np.exp(2.0) + 2.0)) * np.sin(w * x)
    fc = boundary_face_centers(2, coords)
    bc_values = mpfa_convergence_exact(fc[:, 0], fc[:, 1])
    desc = ProblemDesc(coords=coords, num_eq=1, permeability=np.ones(len(cc)), porosity=np.full(len(cc), 0.4),
                       bc_type=np.ones(len(fc), dtype=np.int8), bc_values=bc_values, enable_gravity=False,
                       density=(1.0, 1.0), viscosity=(1.0, 1.0), source=src,
                       permeability_tensor=K if discretization == "mpfa" else None,
                       discretization=discretization)
    return desc, np.zeros(desc.num_dofs), mpfa_convergence_exact(x, y)


def mpfa_linear_field_problem(cells=(6, 5), K=((2.0, 0.5), (0.5, 1.0)), grad=(1.0, -2.0, 0.5), p0=3.0,
                              spacing_seed=None, gravity=False):
    """A constant full permeability tensor and Dirichlet values of the linear pressure
    p = p0 + grad . x on every boundary face, no source: MPFA-O reproduces the linear
    field exactly at the cell centres (the O-method is exact for linear pressures on
    parallelepiped cells), TPFA does not once K has off-diagonal entries.  With
    `spacing_seed` the vertex coordinates are perturbed per axis (still a tensor grid)."""
    dim = len(cells)
    rng = np.random.default_rng(spacing_seed) if spacing_seed is not None else None
    coords = []
    for a, n in enumerate(cells):
        x = equidistant(0.0, 1.0, n)
        if rng is not None:
            x[1:-1] += rng.uniform(-0.3, 0.3, n - 1) / n
        coords.append(x)
    cc = cell_centers(coords)
    N = len(cc)
    Kt = np.tile(np.asarray(K, dtype=np.float64).reshape(1, dim, dim), (N, 1, 1))
    fc = boundary_face_centers(dim, coords)
    g = np.asarray(grad[:dim])
    bc_values = p0 + fc[:, :dim] @ g
    desc = ProblemDesc(coords=coords, num_eq=1, permeability=np.ones(N), porosity=np.full(N, 0.3),
                       bc_type=np.ones(len(fc), dtype=np.int8), bc_values=bc_values, enable_gravity=gravity,
                       density=(WATER_DENSITY, WATER_DENSITY), viscosity=(WATER_VISCOSITY, WATER_VISCOSITY),
                       permeability_tensor=Kt, discretization="mpfa")
    return desc, np.zeros(N), p0 + cc[:, :dim] @ g


def gaussian_lnk_field(cells, mean, sigma, corr_len, seed):
    """Stationary Gaussian random field with exponential covariance
    C(h) = sigma^2 exp(-|h|/corr_len) (|h| in cells), sampled by circulant embedding
    on a grid padded to twice the size in every axis (numpy PCG64 from `seed`)."""
    cells = tuple(int(c) for c in cells)
    pad = tuple(2 * c for c in cells)
    axes = [np.minimum(np.arange(p), p - np.arange(p)).astype(np.float64) for p in pad]
    grids = np.meshgrid(*axes, indexing="ij")
    dist = np.sqrt(sum(g * g for g in grids))
    cov = sigma * sigma * np.exp(-dist / corr_len)
    lam = np.real(np.fft.fftn(cov))
    lam = np.maximum(lam, 0.0)
    rng = np.random.Generator(np.random.PCG64(seed))
    xi = rng.standard_normal(pad) + 1j * rng.standard_normal(pad)
    field = np.fft.ifftn(np.sqrt(lam) * xi) * np.sqrt(np.prod(pad))
    f = np.real(field)[tuple(slice(0, c) for c in cells)]
    # index order (x, y, z) -> flatten x fastest
    return mean + f.flatten(order="F")


def darcy_1p(cells=(100, 100), seed=1, sigma=1.0, corr_len=8.0, mean_lnk=np.log(1e-10),
             enable_gravity=False, lnk=None):
    """1p incompressible Darcy on [0,1]^2: ln K Gaussian field, porosity 0.4, water,
    Dirichlet p=2e5 left / 1e5 right, no-flow top/bottom, one Newton step (stationary)."""
    dim = len(cells)
    coords = [equidistant(0.0, 1.0, n) for n in cells]
    if lnk is None:
        lnk = gaussian_lnk_field(cells, mean_lnk, sigma, corr_len, seed)
    K = np.exp(lnk)
    n = int(np.prod(cells))
    fc = boundary_face_centers(dim, coords)
    nb = num_boundary_faces(dim, list(cells) + [1] * (3 - dim))
    left = fc[:, 0] < 1e-6
    right = fc[:, 0] > coords[0][-1] - 1e-6
    bc_type = np.where(left | right, 1, 2).astype(np.int8)
    bc_values = np.zeros(nb)
    bc_values[left] = 2e5
    bc_values[right] = 1e5
    desc = ProblemDesc(coords=coords, num_eq=1, permeability=K, porosity=np.full(n, 0.4),
                       bc_type=bc_type, bc_values=bc_values, enable_gravity=enable_gravity,
                       density=(WATER_DENSITY, WATER_DENSITY), viscosity=(WATER_VISCOSITY, WATER_VISCOSITY))
    return desc, np.full(desc.num_dofs, 1e5)


def dnapl_2p(cells=(64, 64, 32), extent=(6.0, 4.0, 1.0), seed=2, sigma=1.0, corr_len=6.0,
             mean_lnk=np.log(5e-11), inflow=0.04, pe=500.0, lam=2.0, swr=0.05, snr=0.0,
             pc_low_swe=0.01, enable_gravity=True, lnk=None):
    """2p immiscible water-DNAPL (p_w, S_n), the 2p incompressible test problem
    (test/porousmediumflow/2p/incompressible/problem.hh:59-180) on a 2D or 3D box with
    the vertical axis last: hydrostatic Dirichlet left/right (alpha-scaled), DNAPL
    Neumann inflow on the top strip 0.5 < (xmax-x)/width < 2/3, Brooks-Corey default law,
    Gaussian ln K field."""
    dim = len(cells)
    coords = [equidistant(0.0, float(extent[a]), cells[a]) for a in range(dim)]
    if lnk is None:
        lnk = gaussian_lnk_field(cells, mean_lnk, sigma, corr_len, seed)
    K = np.exp(lnk)
    n = int(np.prod(cells))
    v = dim - 1                       # vertical axis
    g = -9.81 if enable_gravity else 0.0
    fc = boundary_face_centers(dim, coords)
    nb = len(fc)
    xmin, xmax = coords[0][0], coords[0][-1]
    vmin, vmax = coords[v][0], coords[v][-1]
    eps = 1e-6
    on_left = fc[:, 0] < xmin + eps
    on_right = fc[:, 0] > xmax - eps
    on_upper = fc[:, v] > vmax - eps
    width = xmax - xmin
    lam_x = (xmax - fc[:, 0]) / width
    on_inlet = on_upper & (0.5 < lam_x) & (lam_x < 2.0 / 3.0)
    dirichlet = on_left | on_right
    bc_type = np.where(dirichlet, 1, 2).astype(np.int8)
    bc_values = np.zeros((nb, 2))
    height = vmax - vmin
    depth = vmax - fc[:, v]
    alpha = 1 + 1.5 / height
    factor = (width * alpha + (1.0 - alpha) * fc[:, 0]) / width
    pw_dir = 1e5 - factor * WATER_DENSITY * g * depth
    bc_values[dirichlet, 0] = pw_dir[dirichlet]
    bc_values[dirichlet, 1] = 0.0
    bc_values[on_inlet & ~dirichlet, 1] = -inflow
    cc = cell_centers(coords)
    u0 = np.zeros((n, 2))
    u0[:, 0] = 1e5 - WATER_DENSITY * g * (vmax - cc[:, v])
    u0[:, 1] = 0.0
    desc = ProblemDesc(coords=coords, num_eq=2, permeability=K, porosity=np.full(n, 0.4),
                       bc_type=bc_type, bc_values=bc_values.reshape(-1), enable_gravity=enable_gravity,
                       density=(WATER_DENSITY, DNAPL_DENSITY), viscosity=(WATER_VISCOSITY, DNAPL_VISCOSITY),
                       material_params=np.array([[pe, lam, swr, snr, pc_low_swe]]))
    return desc, u0.reshape(-1)


def dnapl_2p_mpfa(cells=(12, 8), seed=2, anisotropy=4.0, angle=0.4, **kw):
    """The 2p water-DNAPL problem of dnapl_2p with a full permeability tensor per cell for the
    MPFA-O discretization: K_i = k_i R diag(1, 1/anisotropy, 1) R^T with R the rotation by
    `angle` in the x-z plane (x-y in 2D), k_i the seeded ln K field."""
    desc, u0 = dnapl_2p(cells=cells, seed=seed, **kw)
    dim = len(cells)
    c, s_ = np.cos(angle), np.sin(angle)
    R = np.eye(dim)
    v = dim - 1
    R[0, 0], R[0, v], R[v, 0], R[v, v] = c, -s_, s_, c
    D = np.ones(dim)
    D[v] = 1.0 / anisotropy
    base = R @ np.diag(D) @ R.T
    Kt = desc.permeability[:, None, None] * base[None, :, :]
    desc.permeability_tensor = np.ascontiguousarray(Kt.reshape(-1))
    desc.discretization = 1
    return desc, u0


def ensemble_2p(count=256, seed=4, n_min=16, n_max=64, extent=(6.0, 4.0, 1.0)):
    """Batched ensemble workload: `count` independent 2p DNAPL problems (dnapl_2p) with
    uneven grids, each axis drawn uniformly from the integers n_min..n_max, and per
    problem sigma ~ U[0.5, 2.0], correlation length ~ U[3, 10] cells and inflow
    ~ U[0.01, 0.08] kg/m^2/s; problem i draws from PCG64(seed + i).
    Returns a list of (desc, u0, meta)."""
    out = []
    for i in range(count):
        rng = np.random.Generator(np.random.PCG64(seed + i))
        cells = tuple(int(v) for v in rng.integers(n_min, n_max + 1, size=3))
        sigma = float(rng.uniform(0.5, 2.0))
        corr = float(rng.uniform(3.0, 10.0))
        inflow = float(rng.uniform(0.01, 0.08))
        desc, u0 = dnapl_2p(cells=cells, extent=extent, seed=1000 + seed + i, sigma=sigma, corr_len=corr,
                            inflow=inflow)
        out.append((desc, u0, {"cells": cells, "sigma": sigma, "corr_len": corr, "inflow": inflow}))
    return out


def served_requests(count, rate=200.0, seed=5, frac_1p=0.3, n_min=1e3, n_max=1e6, steps=(1, 20), dt=250.0):
    """Served-stream workload: `count` requests with Poisson arrivals (mean `rate` per s),
    a frac_1p / (1 - frac_1p) mix of 1p (darcy_1p) and 2p (dnapl_2p) problems, cell
    counts log-uniform in [n_min, n_max] on cube-like 3D grids (round(N^(1/3)) cells per
    axis, at least 10), seeded ln K fields (sigma ~ U[0.5, 2], correlation length
    ~ U[3, 10] cells), 1..20 implicit-Euler steps of `dt` each.
    Returns a list of dicts with arrival time, kind, desc, u0, dt and t_end (sorted by
    arrival).  Problems are built lazily by make() so that a long stream stays cheap."""
    rng = np.random.Generator(np.random.PCG64(seed))
    t = 0.0
    reqs = []
    for i in range(count):
        t += float(rng.exponential(1.0 / rate))
        kind = "1p" if rng.uniform() < frac_1p else "2p"
        n_cells = float(np.exp(rng.uniform(np.log(n_min), np.log(n_max))))
        n = max(10, int(round(n_cells ** (1.0 / 3.0))))
        sigma = float(rng.uniform(0.5, 2.0))
        corr = float(rng.uniform(3.0, 10.0))
        nsteps = int(rng.integers(steps[0], steps[1] + 1))
        inflow = float(rng.uniform(0.01, 0.08))
        reqs.append({"index": i, "arrival": t, "kind": kind, "cells": (n, n, n), "sigma": sigma, "corr_len": corr,
                     "steps": nsteps, "dt": dt, "t_end": nsteps * dt, "inflow": inflow, "seed": 5000 + seed + i})
    return reqs


def make_request_problem(req):
    """(desc, u0) of one served request from served_requests()."""
    if req["kind"] == "1p":
        return darcy_1p(cells=req["cells"], seed=req["seed"], sigma=req["sigma"], corr_len=req["corr_len"])
    return dnapl_2p(cells=req["cells"], seed=req["seed"], sigma=req["sigma"], corr_len=req["corr_len"],
                    inflow=req["inflow"])


# Van Genuchten parameter sets of the reference's 2p lens test (SpatialParams.Lens /
# SpatialParams.Outer of test/porousmediumflow/2p/incompressible/params.input; l, Snr and
# the regularisation thresholds at their defaults): alpha, n, l, Swr, Snr, pcLowSwe,
# pcHighSwe, krnLowSwe, krwHighSwe
LENS_VG = (0.00045, 7.3, 0.5, 0.18, 0.0, 0.01, 0.99, 0.1, 0.9)
OUTER_VG = (0.0037, 4.7, 0.5, 0.05, 0.0, 0.01, 0.99, 0.1, 0.9)


def twop_lens_problem(cells=(48, 32), analytic=False):
    """The reference's 2p incompressible cc-TPFA test (test/porousmediumflow/2p/
    incompressible: problem.hh, spatialparams.hh, params.input): [0,6]x[0,4] m, DNAPL
    lens [1,4]x[2,3] with K 9.05e-12 in 4.6e-10 m^2, regularised Van Genuchten laws,
    porosity 0.4, gravity, hydrostatic Dirichlet left/right, DNAPL inflow -0.04 kg/m^2/s on
    the top strip, p_w hydrostatic and S_n = 0 initially.  Run with dt 250 s and end time
    3000 s it is the case of test_2p_incompressible_tpfa(_analytic)."""
    base, u0 = dnapl_2p(cells=cells, extent=(6.0, 4.0), lnk=np.zeros(int(np.prod(cells))))
    coords = base.coords
    cc = cell_centers(coords)
    eps = 1.5e-7
    lo, hi = (1.0, 2.0), (4.0, 3.0)
    in_lens = np.ones(len(cc), dtype=bool)
    for a in range(2):
        in_lens &= ~((cc[:, a] < lo[a] + eps) | (cc[:, a] > hi[a] - eps))
    K = np.where(in_lens, 9.05e-12, 4.6e-10)
    desc = ProblemDesc(coords=coords, num_eq=2, permeability=K, porosity=np.full(len(cc), 0.4),
                       bc_type=base.bc_type, bc_values=base.bc_values, enable_gravity=True,
                       density=(WATER_DENSITY, DNAPL_DENSITY), viscosity=(WATER_VISCOSITY, DNAPL_VISCOSITY),
                       material=np.where(in_lens, 0, 1).astype(np.int32),
                       material_params=np.array([LENS_VG, OUTER_VG]), material_law="van-genuchten",
                       analytic=analytic)
    return desc, u0
