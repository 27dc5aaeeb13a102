"""VTU output of a solve, as WaveEquationProblem::output_results writes it
(explicit_wave.cc:336-436): the velocity and pressure and their errors
against the projected exact field, on patches of degree k per cell
(``DataOut::build_patches(mapping, fe_degree)``: (k+1)^dim equispaced
points per cell, k^dim linear sub-cells), as an XML unstructured grid.

The state is in the canonical layout [cell][field][point] with the Gauss
points of each cell in lexicographic order (x fastest); the fields are
u_0..u_{dim-1}, p.  Values at the patch points are the Lagrange interpolant
through the Gauss points, positions the multilinear map of the cell's
vertices (the mesh's geometry).  Host code: the state is copied to the
host once per call.
"""
import base64
import os
import xml.etree.ElementTree as ET

import numpy as np

VTK_QUAD, VTK_HEXAHEDRON = 9, 12


def gauss_nodes(n):
    """Gauss-Legendre points on [0, 1]."""
    x, _ = np.polynomial.legendre.leggauss(n)
    return 0.5 * (x + 1.0)


def lagrange_matrix(nodes, pts):
    """L[m, j] = l_j(pts[m]) for the Lagrange basis through ``nodes``."""
    nodes = np.asarray(nodes, dtype=np.float64)
    pts = np.asarray(pts, dtype=np.float64)
    L = np.ones((pts.size, nodes.size))
    for j in range(nodes.size):
        for l in range(nodes.size):
            if l != j:
                L[:, j] *= (pts - nodes[l]) / (nodes[j] - nodes[l])
    return L


def _tensor_apply(I, arr, dim):
    """Apply the 1-D matrix I along each of the last ``dim`` axes of arr
    (axes ordered [.., i_{dim-1}, .., i_0])."""
    for ax in range(dim):
        arr = np.moveaxis(np.tensordot(arr, I, axes=([arr.ndim - dim + ax], [1])), -1,
                          arr.ndim - dim + ax)
    return arr


def patch_coordinates(degree, dim):
    """Reference coordinates of the patch points, (k+1)^dim x dim, x fastest."""
    n = degree + 1
    s = np.linspace(0.0, 1.0, n)
    p = np.arange(n ** dim)
    return np.stack([s[(p // n ** d) % n] for d in range(dim)], axis=1)


def patch_points(vertices, degree):
    """Physical patch points of every cell, (cells, (k+1)^dim, dim): the
    multilinear map of the cell's 2^dim vertices (lexicographic order)."""
    v = np.asarray(vertices, dtype=np.float64)
    dim = v.shape[2]
    xi = patch_coordinates(degree, dim)  # (P, dim)
    phi = np.ones((xi.shape[0], 1 << dim))
    for corner in range(1 << dim):
        for d in range(dim):
            bit = (corner >> d) & 1
            phi[:, corner] *= xi[:, d] if bit else 1.0 - xi[:, d]
    return np.einsum("pv,cvd->cpd", phi, v)


def patch_values(state, n_cells, dim, degree):
    """Field values at the patch points, (cells, dim+1, (k+1)^dim)."""
    n = degree + 1
    u = np.asarray(state, dtype=np.float64).reshape((n_cells, dim + 1) + (n,) * dim)
    I = lagrange_matrix(gauss_nodes(n), np.linspace(0.0, 1.0, n))
    return _tensor_apply(I, u, dim).reshape(n_cells, dim + 1, -1)


def sub_cells(n_cells, dim, degree):
    """Connectivity of the k^dim linear sub-cells of every patch (VTK order)."""
    n = degree + 1
    corners = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0),
               (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)][:1 << dim]
    idx = []
    for c in np.ndindex(*([degree] * dim)):
        c = c[::-1]  # (i0, i1, i2), x fastest
        idx.append([sum((c[d] + corner[d]) * n ** d for d in range(dim)) for corner in corners])
    local = np.array(idx, dtype=np.int64)
    offs = (np.arange(n_cells, dtype=np.int64) * n ** dim)[:, None, None]
    return (local[None] + offs).reshape(-1, 1 << dim)


def _to_host(x):
    if hasattr(x, "detach"):
        x = x.detach().cpu().numpy()
    return np.asarray(x, dtype=np.float64)


def _data_array(name, arr, ncomp, vtype, fmt):
    head = '<DataArray type="%s" Name="%s" NumberOfComponents="%d" format="%s">' % (
        vtype, name, ncomp, fmt)
    a = np.ascontiguousarray(arr)
    if fmt == "ascii":
        body = " ".join(repr(float(x)) if a.dtype.kind == "f" else str(int(x)) for x in a.ravel())
    else:
        raw = a.tobytes()
        body = base64.b64encode(np.uint32(len(raw)).tobytes() + raw).decode("ascii")
    return head + body + "</DataArray>\n"


def write_vtu(path, mesh, degree, state, exact=None, cell_data=None, binary=True):
    """Write the solve's state (and, with ``exact`` in the same layout, the
    error exact - state, as explicit_wave.cc:370-378) to ``path``.
    ``cell_data``: optional {name: per-cell values}.  Returns the path."""
    dim = mesh.dim
    nc = mesh.n_cells
    fmt = "binary" if binary else "ascii"
    vals = patch_values(_to_host(state), nc, dim, degree)
    pts = patch_points(mesh.vertices, degree)
    P = pts.shape[1]
    xyz = np.zeros((nc * P, 3))
    xyz[:, :dim] = pts.reshape(-1, dim)
    conn = sub_cells(nc, dim, degree)
    n_sub = conn.shape[0]
    nv = 1 << dim
    point_data = []

    def add_fields(v, vel_name, p_name):
        vel = np.zeros((nc * P, 3))
        vel[:, :dim] = np.moveaxis(v[:, :dim, :], 1, 2).reshape(-1, dim)
        point_data.append(_data_array(vel_name, vel, 3, "Float64", fmt))
        point_data.append(_data_array(p_name, v[:, dim, :].reshape(-1), 1, "Float64", fmt))

    add_fields(vals, "solution_velocity", "solution_pressure")
    if exact is not None:
        err = patch_values(_to_host(exact), nc, dim, degree) - vals
        add_fields(err, "error_velocity", "error_pressure")
    cells_out = []
    for name, v in (cell_data or {}).items():
        v = np.asarray(v, dtype=np.float64).reshape(nc)
        cells_out.append(_data_array(name, np.repeat(v, n_sub // nc), 1, "Float64", fmt))
    parts = ['<?xml version="1.0"?>\n',
             '<VTKFile type="UnstructuredGrid" version="0.1" byte_order="LittleEndian" '
             'header_type="UInt32">\n<UnstructuredGrid>\n',
             '<Piece NumberOfPoints="%d" NumberOfCells="%d">\n' % (nc * P, n_sub),
             "<Points>\n", _data_array("Points", xyz, 3, "Float64", fmt), "</Points>\n",
             "<Cells>\n", _data_array("connectivity", conn, 1, "Int64", fmt),
             _data_array("offsets", np.arange(1, n_sub + 1, dtype=np.int64) * nv, 1, "Int64", fmt),
             _data_array("types", np.full(n_sub, VTK_QUAD if dim == 2 else VTK_HEXAHEDRON,
                                          dtype=np.uint8), 1, "UInt8", fmt),
             "</Cells>\n", "<PointData>\n"] + point_data + ["</PointData>\n"]
    if cells_out:
        parts += ["<CellData>\n"] + cells_out + ["</CellData>\n"]
    parts.append("</Piece>\n</UnstructuredGrid>\n</VTKFile>\n")
    d = os.path.dirname(path)
    if d:
        os.makedirs(d, exist_ok=True)
    with open(path, "w") as f:
        f.write("".join(parts))
    return path


def output_name(degree, operator_name, initial_case, n_refinements, output_step):
    """The reference's file name (explicit_wave.cc:396-406), without the
    per-process suffix: sol_deg<k>_<Name>_case<c>_ref<r>_step<NNN>.vtu."""
    return "sol_deg%d_%s_case%d_ref%d_step%03d.vtu" % (degree, operator_name, initial_case,
                                                       n_refinements, output_step)


def read_vtu(path):
    """Read a file written by ``write_vtu``: ({array name: (n, components)},
    number of points, number of cells)."""
    types = {"Float64": np.float64, "Int64": np.int64, "UInt8": np.uint8}
    root = ET.parse(path).getroot()
    out = {}
    for da in root.iter("DataArray"):
        dtype = types[da.get("type")]
        if da.get("format") == "ascii":
            a = np.array((da.text or "").split(), dtype=np.float64).astype(dtype)
        else:
            raw = base64.b64decode(da.text)
            n = int(np.frombuffer(raw[:4], dtype=np.uint32)[0])
            if n != len(raw) - 4:
                raise ValueError("%s: array %s has a bad length header" % (path, da.get("Name")))
            a = np.frombuffer(raw[4:], dtype=dtype)
        out[da.get("Name")] = a.reshape(-1, int(da.get("NumberOfComponents")))
    piece = root.find("UnstructuredGrid/Piece")
    return out, int(piece.get("NumberOfPoints")), int(piece.get("NumberOfCells"))
