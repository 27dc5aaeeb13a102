"""Change of nodal basis on the host (ew_nodal_to_gauss / ew_gauss_to_nodal):
FE_DGQ(k)'s equidistant nodal values of a Q_k polynomial map to its values at
the Gauss points, the inverse maps back, and invalid arguments are refused."""
import numpy as np
import pytest

from exwave_gb300 import _lib, basis, vtu


def _poly_values(dim, k, pts1d, coef):
    """Q_k polynomial sum c_{abc} x^a y^b z^c at the tensor grid of pts1d
    (lexicographic, x fastest)."""
    n = k + 1
    p = np.arange(n ** dim)
    x = [pts1d[(p // n ** d) % n] for d in range(dim)]
    out = np.zeros(p.size)
    for idx in np.ndindex(*([n] * dim)):
        term = coef[idx]
        for d in range(dim):
            term = term * x[d] ** idx[d]
        out += term
    return out


@pytest.mark.parametrize("dim,k", [(2, 1), (2, 4), (3, 2), (3, 5), (3, 7)])
def test_equidistant_to_gauss_is_exact(dim, k):
    rng = np.random.default_rng(10 * dim + k)
    cells, F = 3, dim + 1
    eq = basis.equidistant_nodes(k)
    g = vtu.gauss_nodes(k + 1)
    coef = rng.standard_normal((cells, F) + (k + 1,) * dim)
    nodal = np.stack([np.stack([_poly_values(dim, k, eq, coef[c, f]) for f in range(F)])
                      for c in range(cells)])
    gauss = np.stack([np.stack([_poly_values(dim, k, g, coef[c, f]) for f in range(F)])
                      for c in range(cells)])
    mine = basis.nodal_to_gauss(dim, k, nodal.reshape(-1))
    scale = np.abs(gauss).max()
    assert np.abs(mine - gauss.reshape(-1)).max() < 1e-11 * scale
    back = basis.gauss_to_nodal(dim, k, mine)
    assert np.abs(back - nodal.reshape(-1)).max() < 1e-11 * scale
    # the Gauss values interpolate back to the patch points like the VTU writer
    pv = vtu.patch_values(mine, cells, dim, k)
    assert np.abs(pv.reshape(-1) - nodal.reshape(-1)).max() < 1e-11 * scale


def test_other_nodes_and_field_count():
    dim, k, F = 3, 3, 1
    nodes = np.array([0.0, 0.2, 0.7, 1.0])
    rng = np.random.default_rng(4)
    coef = rng.standard_normal((k + 1,) * dim)
    src = _poly_values(dim, k, nodes, coef)
    got = basis.nodal_to_gauss(dim, k, src, nodes=nodes, n_fields=F)
    ref = _poly_values(dim, k, vtu.gauss_nodes(k + 1), coef)
    assert np.abs(got - ref).max() < 1e-11 * np.abs(ref).max()


def test_invalid_arguments_are_refused():
    L = _lib.load()
    a = np.zeros(4 * 27)
    b = np.zeros_like(a)
    eq = basis.equidistant_nodes(2)
    dup = np.array([0.0, 0.5, 0.5])
    ok = L.ew_nodal_to_gauss(3, 2, 1, 4, eq.ctypes.data, a.ctypes.data, b.ctypes.data)
    assert ok == 0
    assert L.ew_nodal_to_gauss(4, 2, 1, 4, eq.ctypes.data, a.ctypes.data, b.ctypes.data) == -1
    assert L.ew_nodal_to_gauss(3, 0, 1, 4, eq.ctypes.data, a.ctypes.data, b.ctypes.data) == -1
    assert L.ew_nodal_to_gauss(3, 2, 1, 4, dup.ctypes.data, a.ctypes.data, b.ctypes.data) == -1
    assert L.ew_nodal_to_gauss(3, 2, 1, 4, None, a.ctypes.data, b.ctypes.data) == -1
    assert L.ew_gauss_to_nodal(3, 2, 1, 4, eq.ctypes.data, a.ctypes.data, a.ctypes.data) == -1
    assert L.ew_gauss_to_nodal(3, 2, 1, 0, eq.ctypes.data, a.ctypes.data, b.ctypes.data) == -1
    # no cells: nothing to do, null arrays allowed
    assert L.ew_gauss_to_nodal(3, 2, 0, 4, eq.ctypes.data, None, None) == 0
    with pytest.raises(ValueError):
        basis.nodal_to_gauss(3, 2, np.zeros(10))
