"""The inputs of the curved two-layer ADER configuration, on the CPU.

The reference knows one material and the membrane initial field
(input_parameters.cc:22-29, input_parameters.h:95-128); the Gaussian
pressure pulse and the two-layer medium have no counterpart there, so they
are checked here against their definitions:
- the oracle's Gaussian projection is the pulse sampled at the Gauss points
  (the collocation form of project_initial_field,
  wave_equation_operations.cc:902-935), with zero velocity;
- layered_materials gives (c, rho) of the lower layer to every cell whose
  centre lies at or below the split plane and the upper pair to the rest,
  and on the sine-mapped mesh the plane z = 0.5 stays a mesh plane, so every
  cell lies wholly on one side of it.
"""
import numpy as np
import pytest


def test_oracle_gaussian_is_the_sampled_pulse(oracle_mod):
    prob = oracle_mod.Problem.hypercube(3, 3, 3, 0, 0.05)
    x0 = np.array([0.41, 0.37, 0.28])
    width, amp = 0.12, 1.7
    u = prob.project_gaussian(x0, width, amp).reshape(prob.n_cells, 4, -1)
    xyz = prob.quadrature_points()
    want = amp * np.exp(-((xyz - x0) ** 2).sum(axis=2) / (2 * width ** 2))
    np.testing.assert_allclose(u[:, 3, :], want, rtol=1e-15, atol=1e-300)
    assert np.all(u[:, :3, :] == 0.0)
    # 2-D: only the first two coordinates of x0 count
    p2 = oracle_mod.Problem.hypercube(2, 4, 4, 1, 0.1)
    u2 = p2.project_gaussian([0.5, 0.25], 0.2).reshape(p2.n_cells, 3, -1)
    xy = p2.quadrature_points()
    want2 = np.exp(-((xy - np.array([0.5, 0.25])) ** 2).sum(axis=2) / (2 * 0.2 ** 2))
    np.testing.assert_allclose(u2[:, 2, :], want2, rtol=1e-15)


@pytest.mark.parametrize("n", [4, 6])
def test_layered_materials_split_on_a_mesh_plane(n):
    import exwave_gb300 as ew
    m = ew.hypercube(3, n, 0, 0.03, transform="sine_all", boundary_ids=[1, 1, 1, 1, 1, 2])
    ew.layered_materials(m, 0.5, below=(1.0, 1.0), above=(3.0, 2.0))
    upper = m.speed == 3.0
    assert np.all(m.density[upper] == 2.0)
    assert np.all((m.speed[~upper] == 1.0) & (m.density[~upper] == 1.0))
    assert upper.sum() == m.n_cells // 2
    z = m.vertices[:, :, 2]
    # the map x_i += 0.03 prod_d sin(2 pi x_d) vanishes on z = 0.5
    assert np.all(z[upper].min(axis=1) >= 0.5 - 1e-15)
    assert np.all(z[~upper].max(axis=1) <= 0.5 + 1e-15)
    # top face (z = 1) is the free surface (id 2), the others rigid walls (id 1)
    nb = m.neighbors
    assert set(np.unique(-nb[nb < 0])) == {1, 2}
    top = nb[:, 5] < 0
    assert np.all(nb[top, 5] == -2) and np.all(nb[:, :5][nb[:, :5] < 0] == -1)


def test_layered_materials_other_axis_and_threshold():
    import exwave_gb300 as ew
    m = ew.hypercube(2, 8)
    ew.layered_materials(m, 0.3, below=(2.0, 5.0), above=(1.0, 1.0), axis=0)
    cx = m.centers()[:, 0]
    np.testing.assert_array_equal(m.speed, np.where(cx > 0.3, 1.0, 2.0))
    np.testing.assert_array_equal(m.density, np.where(cx > 0.3, 1.0, 5.0))
