"""CPU-side checks of the C ABI: the library loads, exports every entry
point that include/exwave_gb300.h declares, and rejects invalid meshes in
ew_create before touching a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from exwave_gb300 import build, _lib
    build.build()
    return _lib


def declared_functions():
    with open(os.path.join(ROOT, "include", "exwave_gb300.h")) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ew_[a-z0-9_]+)\s*\(", text)))


def test_exports_every_declared_symbol(lib):
    L = lib.load()
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(L, n), n
    assert sorted(lib.EXPORTS) == names


def _mesh_desc(lib, mesh, degree):
    keep = [np.ascontiguousarray(mesh.vertices), np.ascontiguousarray(mesh.neighbors),
            np.ascontiguousarray(mesh.speed), np.ascontiguousarray(mesh.density)]
    md = lib.MeshDesc()
    md.dim = mesh.dim
    md.degree = degree
    md.n_cells = mesh.n_cells
    md.vertices = keep[0].ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    md.neighbors = keep[1].ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    md.speed = keep[2].ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    md.density = keep[3].ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    return md, keep


def _create(lib, mesh, degree):
    md, keep = _mesh_desc(lib, mesh, degree)
    h = ctypes.c_void_p()
    rc = lib.load().ew_create(ctypes.byref(md), None, ctypes.byref(h))
    return rc, lib.load().ew_last_error(None).decode()


def test_create_rejects_bad_meshes(lib):
    import exwave_gb300 as ew
    m = ew.hypercube(2, 3)
    rc, msg = _create(lib, m, 13)     # the reference instantiates k = 1..12
    assert rc == -1 and "degree" in msg
    rc, msg = _create(lib, m, 0)
    assert rc == -1
    bad = ew.hypercube(2, 3)
    bad.neighbors[0, 1] = 5          # not symmetric
    rc, msg = _create(lib, bad, 2)
    assert rc == -1 and "symmetric" in msg
    bad = ew.hypercube(2, 3)
    bad.neighbors[0, 0] = -7         # unknown boundary id
    rc, msg = _create(lib, bad, 2)
    assert rc == -1 and "boundary id" in msg
    bad = ew.hypercube(2, 3)
    bad.neighbors[0, 1] = 100        # out of range
    rc, msg = _create(lib, bad, 2)
    assert rc == -1 and "range" in msg
    bad = ew.hypercube(2, 3)
    bad.speed[4] = -1.0
    rc, msg = _create(lib, bad, 2)
    assert rc == -1 and "positive" in msg
    bad = ew.hypercube(2, 3, transform_factor=0.1)
    bad.vertices[1, 0, 1] += 0.01    # face no longer matches its neighbour
    rc, msg = _create(lib, bad, 2)
    assert rc == -1


def test_create_rejects_degenerate_input(lib):
    import exwave_gb300 as ew
    L = lib.load()
    h = ctypes.c_void_p()
    # no mesh, no cells, missing arrays
    assert L.ew_create(None, None, ctypes.byref(h)) == -1
    m = ew.hypercube(2, 2)
    md, keep = _mesh_desc(lib, m, 2)
    md.n_cells = 0
    assert L.ew_create(ctypes.byref(md), None, ctypes.byref(h)) == -1
    md, keep = _mesh_desc(lib, m, 2)
    md.speed = None
    assert L.ew_create(ctypes.byref(md), None, ctypes.byref(h)) == -1
    # non-finite material, a collapsed cell
    bad = ew.hypercube(2, 2)
    bad.density[1] = float("nan")
    rc, msg = _create(lib, bad, 2)
    assert rc == -1 and "positive" in msg
    bad = ew.hypercube(2, 2)
    bad.vertices[2] = bad.vertices[2, 0]
    rc, msg = _create(lib, bad, 2)
    assert rc == -1


@pytest.mark.parametrize("dim,n,ref,f", [(2, 20, 0, 0.0), (2, 5, 2, 0.1), (3, 5, 0, 0.1),
                                         (3, 3, 0, 0.05), (2, 5, 3, 0.1), (3, 2, 2, 0.2)])
def test_hypercube_matches_oracle(lib, oracle_mod, dim, n, ref, f):
    import exwave_gb300 as ew
    m = ew.hypercube(dim, n, ref, f, boundary_ids=2)
    o = oracle_mod.Problem.hypercube(dim, 1, n, ref, f, 2)
    np.testing.assert_allclose(m.vertices, o.vertices(), rtol=0, atol=1e-15)
    np.testing.assert_array_equal(m.neighbors, o.neighbors())


def test_boundary_ids_per_face(lib):
    import exwave_gb300 as ew
    m = ew.hypercube(3, 4, boundary_ids=[1, 1, 1, 1, 1, 2])
    top = m.neighbors[:, 5]
    assert (top[top < 0] == -2).all() and (m.neighbors[:, :5][m.neighbors[:, :5] < 0] == -1).all()
    assert (m.neighbors < 0).sum() == 6 * 16


def test_time_step_and_control(lib, oracle_mod):
    import exwave_gb300 as ew
    m = ew.hypercube(3, 5, 0, 0.1)
    o = oracle_mod.Problem.hypercube(3, 4, 5, 0, 0.1, 2)
    cfl = 0.2 / 4 ** 1.5
    assert ew.time_step_size(m, cfl) == pytest.approx(o.time_step(cfl), rel=1e-15)
    # lsrk45r2_2d_cartesian: 20 intervals, k = 1, cfl 0.3; make_dofs resets
    # the rounded step to the unrounded one (explicit_wave.cc:222)
    dt = ew.time_step_size(ew.hypercube(2, 20), 0.3)
    tc = ew.TimeControl()
    tc.setup(1.0, 0.1, dt)
    assert "%g" % tc.time_step == "0.0149254"   # printed by the reference
    tc.set_time_step(dt)
    ticks = []
    while not tc.done():
        tc.advance_time_step()
        if tc.at_tick():
            ticks.append(tc.time_step_number)
    # the step numbers printed by the reference's lsrk45r2_2d_cartesian.output
    assert ticks == [7, 14, 21, 27, 34, 41, 47, 54, 61, 67]
