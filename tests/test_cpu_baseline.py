"""The CPU baseline for axis-aligned meshes (oracle/ew_cpu_cart.cpp, timed by
bench.py's CPU legs) against the oracle it restates in line form: operator
and LowStorageRK45Reg2 steps to 1e-13 relative, 2-D and 3-D, degrees 1..7,
heterogeneous materials and every boundary id."""
import numpy as np
import pytest

CASES = [
    # dim, degree, intervals, boundary ids
    (2, 1, 6, [1, 2, 3, 1]),
    (2, 4, 5, 2),
    (2, 7, 3, [3, 3, 1, 2]),
    (3, 2, 3, [1, 2, 3, 1, 2, 3]),
    (3, 5, 3, 2),
    (3, 7, 2, [2, 1, 3, 3, 1, 2]),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: "d%dk%d" % c[:2])
def test_cpu_baseline_matches_oracle(oracle_mod, case):
    import exwave_gb300 as ew
    dim, k, n, bids = case
    m = ew.hypercube(dim, n, 0, 0.0, boundary_ids=bids)
    rng = np.random.default_rng(k + 10 * dim)
    m.speed = rng.uniform(1.0, 4.0, m.n_cells)
    m.density = rng.uniform(1.0, 3.0, m.n_cells)
    o = oracle_mod.Problem.from_mesh(dim, k, m.vertices, m.neighbors, m.speed, m.density)
    c = oracle_mod.CartCPU(dim, k, m.vertices, m.neighbors, m.speed, m.density)
    u = rng.standard_normal(o.n_dofs)
    ref = o.apply(u)
    got = c.apply(u)
    assert np.abs(got - ref).max() / np.abs(ref).max() < 1e-13
    u0 = o.project_reference(2)
    dt = o.time_step(0.25 / k ** 1.5)
    a, b = u0.copy(), np.zeros_like(u0)
    x, y = u0.copy(), np.zeros_like(u0)
    for _ in range(3):
        o.lsrk45_step(dt, a, b)
        a, b = b, a
        c.lsrk45_step(dt, x, y)
        x, y = y, x
    assert np.abs(x - a).max() / np.abs(a).max() < 1e-13


def test_cpu_baseline_rejects_curved_cells(oracle_mod):
    import exwave_gb300 as ew
    m = ew.hypercube(2, 3, 0, 0.1)
    with pytest.raises(RuntimeError):
        oracle_mod.CartCPU(2, 3, m.vertices, m.neighbors, m.speed, m.density)
