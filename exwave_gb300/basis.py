"""Per-cell change of nodal basis between another set of 1-D support points
and this library's Gauss-point layout (``ew_nodal_to_gauss`` /
``ew_gauss_to_nodal``, host code).

The reference's FE_DGQ(k) (explicit_wave.cc:162) holds each field by its
values at k+1 equidistant points per direction; FEEvaluation interpolates
them to QGauss(k+1) before the operator (wave_equation_operations.cc:411-419).
Both span Q_k, so the conversion is exact in both directions.  Arrays are
[cell][field][point] with the points lexicographic, x fastest."""
import numpy as np

from . import _lib


def equidistant_nodes(degree):
    """FE_DGQ(k)'s 1-D support points on [0, 1]."""
    return np.linspace(0.0, 1.0, degree + 1)


def _convert(fn, dim, degree, values, nodes, n_fields):
    L = _lib.load()
    nodes = np.ascontiguousarray(equidistant_nodes(degree) if nodes is None else nodes,
                                 dtype=np.float64)
    src = np.ascontiguousarray(values, dtype=np.float64)
    per_cell = n_fields * (degree + 1) ** dim
    if nodes.size != degree + 1 or src.size % per_cell:
        raise ValueError("values must hold whole cells of %d fields x (k+1)^dim points" % n_fields)
    dst = np.empty_like(src)
    rc = getattr(L, fn)(dim, degree, src.size // per_cell, n_fields, nodes.ctypes.data,
                        src.ctypes.data, dst.ctypes.data)
    if rc != 0:
        raise _lib.EwError(rc, "%s: invalid arguments" % fn)
    return dst


def nodal_to_gauss(dim, degree, values, nodes=None, n_fields=None):
    """Values at ``nodes`` (default: FE_DGQ's equidistant points) -> values at
    the Gauss points, per cell and field (n_fields defaults to dim + 1)."""
    return _convert("ew_nodal_to_gauss", dim, degree, values, nodes,
                    dim + 1 if n_fields is None else n_fields)


def gauss_to_nodal(dim, degree, values, nodes=None, n_fields=None):
    """The inverse of ``nodal_to_gauss``."""
    return _convert("ew_gauss_to_nodal", dim, degree, values, nodes,
                    dim + 1 if n_fields is None else n_fields)
