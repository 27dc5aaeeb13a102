"""VTU output (exwave_gb300.vtu, the analogue of output_results,
explicit_wave.cc:336-436) on the CPU: patch points on the mapped cells,
values equal to the oracle's point evaluation of the DG field, errors
against an exact field, and a file that parses as an XML unstructured grid
in both encodings."""
import numpy as np
import pytest

from exwave_gb300 import mesh as mesh_mod
from exwave_gb300 import vtu


@pytest.mark.parametrize("dim,k,n,f", [(2, 3, 3, 0.1), (3, 2, 2, 0.1), (2, 1, 2, 0.0)])
@pytest.mark.parametrize("binary", [True, False])
def test_vtu_matches_oracle_point_values(oracle_mod, tmp_path, dim, k, n, f, binary):
    m = mesh_mod.hypercube(dim, n, 0, f)
    o = oracle_mod.Problem.from_mesh(dim, k, m.vertices, m.neighbors, m.speed, m.density)
    rng = np.random.default_rng(3 + dim + k)
    u = rng.standard_normal(o.n_dofs)
    exact = rng.standard_normal(o.n_dofs)
    path = vtu.write_vtu(str(tmp_path / "out" / "s.vtu"), m, k, u, exact=exact,
                         cell_data={"speed": m.speed}, binary=binary)
    arr, npts, ncells = vtu.read_vtu(path)
    P = (k + 1) ** dim
    assert npts == m.n_cells * P and ncells == m.n_cells * k ** dim
    pts = arr["Points"][:, :dim]
    # patch corners are the cell vertices
    corners = [sum(((c >> d) & 1) * k * (k + 1) ** d for d in range(dim)) for c in range(1 << dim)]
    got = pts.reshape(m.n_cells, P, dim)[:, corners, :]
    assert np.abs(got - m.vertices).max() < 1e-14
    # pressure at interior patch points: the oracle's evaluation of the field
    xi = vtu.patch_coordinates(k, dim)
    inner = np.all((xi > 0) & (xi < 1), axis=1)
    if inner.any():
        sel = pts.reshape(m.n_cells, P, dim)[:, inner, :].reshape(-1, dim)
        ref = o.point_values(u, sel)
        mine = arr["solution_pressure"].reshape(m.n_cells, P)[:, inner].reshape(-1)
        assert np.abs(mine - ref).max() < 1e-12 * max(1.0, np.abs(ref).max())
    # every patch point: interpolation of a field that is a polynomial of
    # degree k in the reference coordinates is exact
    g = vtu.gauss_nodes(k + 1)
    q = np.arange((k + 1) ** dim)
    gx = np.stack([g[(q // (k + 1) ** d) % (k + 1)] for d in range(dim)], axis=1)
    poly = lambda x: 1.0 + x[:, 0] ** k - 0.5 * x[:, -1] ** max(k - 1, 0) * x[:, 0]
    w = np.zeros((m.n_cells, dim + 1, (k + 1) ** dim))
    w[:, dim, :] = poly(gx)[None, :]
    w[:, 0, :] = 2.0 * poly(gx)[None, :]
    path2 = vtu.write_vtu(str(tmp_path / "p.vtu"), m, k, w.reshape(-1), binary=binary)
    arr2, _, _ = vtu.read_vtu(path2)
    assert np.abs(arr2["solution_pressure"].reshape(m.n_cells, P) - poly(xi)[None]).max() < 1e-12
    assert np.abs(arr2["solution_velocity"][:, 0].reshape(m.n_cells, P) - 2 * poly(xi)[None]).max() \
        < 1e-12
    # errors: exact - solution at the same points
    err = arr["error_pressure"][:, 0] + arr["solution_pressure"][:, 0]
    ev = vtu.patch_values(exact, m.n_cells, dim, k)[:, dim, :].reshape(-1)
    assert np.abs(err - ev).max() < 1e-12
    # sub-cells: valid indices, positive measure (counter-clockwise / right-handed)
    conn = arr["connectivity"].reshape(-1, 1 << dim)
    assert conn.min() == 0 and conn.max() == npts - 1
    P0 = arr["Points"][conn[:, 0]]
    e1 = arr["Points"][conn[:, 1]] - P0
    e2 = arr["Points"][conn[:, 3]] - P0
    if dim == 2:
        assert (e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0] > 0).all()
    else:
        e3 = arr["Points"][conn[:, 4]] - P0
        assert (np.einsum("ij,ij->i", np.cross(e1, e2), e3) > 0).all()
    assert (arr["types"] == (9 if dim == 2 else 12)).all()
    assert np.array_equal(arr["speed"][:, 0], np.repeat(m.speed, k ** dim))


def test_output_name():
    assert vtu.output_name(4, "Runge-Kutta", 1, 0, 7) == "sol_deg4_Runge-Kutta_case1_ref0_step007.vtu"
