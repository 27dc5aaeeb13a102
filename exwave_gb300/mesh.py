"""Meshes of one solve: the flattened problem definition handed to the
operator (vertices, face neighbours with boundary ids, per-cell material).

``hypercube`` restates the reference's ``input_geometry_description``
(input_parameters.h:60-88) through the native generator
``ew_hypercube_mesh``; materials default to the reference's single
material c = rho = 1 (input_parameters.cc:22-29).
"""
import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib

TRANSFORMS = {"reference": 0, "sine_all": 1}


@dataclass
class Mesh:
    dim: int
    vertices: np.ndarray   # (n_cells, 2^dim, dim) float64
    neighbors: np.ndarray  # (n_cells, 2*dim) int32; <0: -boundary id
    speed: np.ndarray      # (n_cells,) float64
    density: np.ndarray    # (n_cells,) float64
    cells_per_direction: int = 0

    @property
    def n_cells(self):
        return self.speed.shape[0]

    def centers(self):
        return self.vertices.mean(axis=1)

    def min_vertex_distance(self):
        """Per cell, the minimum distance between any two vertices
        (TriaAccessor::minimum_vertex_distance)."""
        v = self.vertices
        nv = v.shape[1]
        best = np.full(v.shape[0], np.inf)
        for a in range(nv):
            for b in range(a + 1, nv):
                best = np.minimum(best, np.sqrt(((v[:, a] - v[:, b]) ** 2).sum(axis=1)))
        return best


def hypercube(dim, n_intervals, n_refinements=0, transform_factor=0.0, transform="reference",
              boundary_ids=2, speed=1.0, density=1.0):
    """Structured mesh of [0,1]^dim: ``n_intervals`` coarse cells per
    direction, vertex transform, ``n_refinements`` global refinements.
    ``boundary_ids`` is one id for every boundary face (the reference) or a
    list per domain face (x=0, x=1, y=0, y=1, z=0, z=1)."""
    L = _lib.load()
    desc = _lib.HypercubeDesc()
    desc.dim = dim
    desc.n_intervals = n_intervals
    desc.n_refinements = n_refinements
    desc.transform = TRANSFORMS[transform]
    desc.transform_factor = transform_factor
    ids = [boundary_ids] * 6 if np.isscalar(boundary_ids) else list(boundary_ids) + [2] * 6
    for i in range(6):
        desc.boundary_ids[i] = int(ids[i])
    n = L.ew_hypercube_n_cells(ctypes.byref(desc))
    if n <= 0:
        raise ValueError("invalid hypercube description")
    verts = np.zeros((n, 1 << dim, dim), dtype=np.float64)
    nbr = np.zeros((n, 2 * dim), dtype=np.int32)
    _lib.check(L.ew_hypercube_mesh(ctypes.byref(desc), verts.ctypes.data, nbr.ctypes.data))
    sp = np.full(n, speed, dtype=np.float64) if np.isscalar(speed) else np.asarray(speed, np.float64)
    de = np.full(n, density, dtype=np.float64) if np.isscalar(density) else np.asarray(density, np.float64)
    return Mesh(dim, verts, nbr, sp, de, n_intervals << n_refinements)


def layered_materials(mesh, z_split, below, above, axis=None):
    """Two-layer medium: (c, rho) = ``below`` for cell centres with
    x_axis <= z_split, ``above`` otherwise (axis defaults to the last one)."""
    axis = mesh.dim - 1 if axis is None else axis
    upper = mesh.centers()[:, axis] > z_split
    mesh.speed = np.where(upper, above[0], below[0]).astype(np.float64)
    mesh.density = np.where(upper, above[1], below[1]).astype(np.float64)
    return mesh


def time_step_size(mesh, cfl_scaled):
    """compute_time_step_size (explicit_wave.cc:529-545): cfl * min over cells
    of (minimum vertex distance / speed); ``cfl_scaled`` already divided by
    k^1.5 (parameters.cc:195)."""
    return float(cfl_scaled * np.min(mesh.min_vertex_distance() / mesh.speed))
