"""VTU field output and restart for structured cc-TPFA problems.

The wire format of the reference's output and restart files (VtkOutputModule,
dumux/io/vtkoutputmodule.hh:186; loadSolution, dumux/io/loadsolution.hh:91-193): a VTK XML
UnstructuredGrid with the grid's vertices as points, one quadrilateral (2D) or hexahedron
(3D) per cell in the grid's cell order (x fastest), and cell data arrays named after the
model's fields -- for 2p immiscible water-DNAPL "S_aq", "p_aq", "S_napl", "p_napl", for 1p
"p".  ASCII Float32 by default, as the reference writes (Vtk.Precision = Float32);
Float64 for bit-exact restarts.

load_solution() reads the primary variables back by name (p0s1: p_aq and S_napl), as
loadSolution does with the model's primary-variable names.
"""
import re

import numpy as np

_PHASES = ("aq", "napl")


def _vertices(desc):
    dim = desc.dim
    coords = desc.coords
    grids = np.meshgrid(*coords, indexing="ij")
    pts = np.zeros((grids[0].size, 3))
    for a in range(dim):
        pts[:, a] = grids[a].flatten(order="F")     # x fastest, as the grid's vertex order
    return pts


def _cells(desc):
    """Connectivity in VTK's node order: quad (VTK 9) / hexahedron (VTK 12)."""
    n = desc.cells[:desc.dim]
    nv = [c + 1 for c in n]
    if desc.dim == 2:
        i, j = np.meshgrid(np.arange(n[0]), np.arange(n[1]), indexing="ij")
        i, j = i.flatten(order="F"), j.flatten(order="F")
        v = lambda a, b: (i + a) + nv[0] * (j + b)
        conn = np.stack([v(0, 0), v(1, 0), v(1, 1), v(0, 1)], axis=1)
        return conn, 9
    i, j, k = np.meshgrid(np.arange(n[0]), np.arange(n[1]), np.arange(n[2]), indexing="ij")
    i, j, k = i.flatten(order="F"), j.flatten(order="F"), k.flatten(order="F")
    v = lambda a, b, c: (i + a) + nv[0] * ((j + b) + nv[1] * (k + c))
    conn = np.stack([v(0, 0, 0), v(1, 0, 0), v(1, 1, 0), v(0, 1, 0),
                     v(0, 0, 1), v(1, 0, 1), v(1, 1, 1), v(0, 1, 1)], axis=1)
    return conn, 12


def primary_fields(desc, u):
    """Cell fields of a solution vector: 1p {"p"}, 2p {"p_aq", "S_napl", "S_aq"}."""
    u = np.asarray(u, dtype=np.float64).reshape(-1, desc.num_eq)
    if desc.num_eq == 1:
        return {"p": u[:, 0]}
    return {"S_aq": 1.0 - u[:, 1], "p_aq": u[:, 0], "S_napl": u[:, 1]}


def write_vtu(path, desc, u, extra=None, precision="Float32"):
    """Writes the solution u (N*num_eq) and optional extra cell fields {name: array}."""
    fmt = {"Float32": (np.float32, "%.9g"), "Float64": (np.float64, "%.17g")}[precision]
    fields = primary_fields(desc, u)
    if extra:
        fields.update({k: np.asarray(v, dtype=np.float64).reshape(-1) for k, v in extra.items()})
    pts = _vertices(desc)
    conn, vtk_type = _cells(desc)
    ncell, nper = conn.shape

    def arr(values, dtype):
        v = np.asarray(values, dtype=dtype).reshape(-1)
        if np.issubdtype(dtype, np.floating):
            return " ".join(fmt[1] % x for x in v)
        return " ".join(str(int(x)) for x in v)

    out = ['<?xml version="1.0"?>',
           '<VTKFile type="UnstructuredGrid" version="0.1" byte_order="LittleEndian">',
           '  <UnstructuredGrid>',
           f'    <Piece NumberOfCells="{ncell}" NumberOfPoints="{len(pts)}">',
           '      <CellData Scalars="%s">' % next(iter(fields))]
    for name, values in fields.items():
        out.append(f'        <DataArray type="{precision}" Name="{name}" NumberOfComponents="1" format="ascii">')
        out.append("          " + arr(values, fmt[0]))
        out.append('        </DataArray>')
    out += ['      </CellData>', '      <Points>',
            f'        <DataArray type="{precision}" Name="Coordinates" NumberOfComponents="3" format="ascii">',
            "          " + arr(pts, fmt[0]), '        </DataArray>', '      </Points>', '      <Cells>',
            '        <DataArray type="Int32" Name="connectivity" NumberOfComponents="1" format="ascii">',
            "          " + arr(conn, np.int32), '        </DataArray>',
            '        <DataArray type="Int32" Name="offsets" NumberOfComponents="1" format="ascii">',
            "          " + arr(np.arange(1, ncell + 1) * nper, np.int32), '        </DataArray>',
            '        <DataArray type="UInt8" Name="types" NumberOfComponents="1" format="ascii">',
            "          " + arr(np.full(ncell, vtk_type), np.int32), '        </DataArray>',
            '      </Cells>', '    </Piece>', '  </UnstructuredGrid>', '</VTKFile>', '']
    with open(path, "w") as f:
        f.write("\n".join(out))


def read_vtu(path):
    """Cell data arrays of an ASCII VTU file: {name: float64 array}."""
    txt = open(path).read()
    cell = re.search(r"<CellData[^>]*>(.*?)</CellData>", txt, re.S)
    if not cell:
        return {}
    out = {}
    for m in re.finditer(r'<DataArray[^>]*Name="([^"]+)"[^>]*>(.*?)</DataArray>', cell.group(1), re.S):
        out[m.group(1)] = np.array(m.group(2).split(), dtype=np.float64)
    return out


def load_solution(path, desc):
    """loadSolution for the p0s1 formulation: primary variables by name (1p: "p";
    2p: "p_aq", "S_napl"), returned as the flat N*num_eq solution vector."""
    f = read_vtu(path)
    names = ["p"] if desc.num_eq == 1 else ["p_aq", "S_napl"]
    missing = [n for n in names if n not in f]
    if missing:
        raise KeyError(f"{path} lacks the primary-variable fields {missing}")
    cols = [f[n] for n in names]
    if any(len(c) != desc.num_cells for c in cols):
        raise ValueError(f"{path} holds {len(cols[0])} cells, the problem {desc.num_cells}")
    return np.stack(cols, axis=1).reshape(-1)
