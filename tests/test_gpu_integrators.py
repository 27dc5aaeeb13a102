"""The reference's other integrators on the GPU -- explicit Euler, classical
RK4, LSRK33R2 and LSRK59R2 (fused 2-register stages), LSRK45R3 and
SSPRK(4,8) (operator applications plus device vector updates) -- against the
oracle's restatements after a few steps.

Tolerances: FP64 and compensated (float-float operator) 1e-12 relative to
the largest entry; mixed (FP32 operator) 1e-5."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NAMES = ["ExplEuler", "clRK4", "LSRK33R2", "LSRK45R2", "LSRK45R3", "LSRK59R2", "SSPRK"]
CASES = [
    # dim, k, intervals, refinements, transform, boundary ids, heterogeneous
    (2, 4, 6, 0, 0.0, [1, 2, 3, 1], True),
    (3, 3, 3, 0, 0.1, 2, False),
]


@pytest.fixture(scope="module")
def env(oracle_mod):
    import torch
    from exwave_gb300 import build
    build.build()
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    import exwave_gb300 as ew
    from exwave_gb300 import driver
    return ew, driver, oracle_mod, torch


@pytest.mark.parametrize("case", CASES, ids=["d2k4_cart", "d3k3_curved"])
@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed_ff"])
@pytest.mark.parametrize("name", NAMES)
def test_integrator_matches_oracle(env, name, precision, case):
    ew, driver, oracle, torch = env
    dim, k, n, ref, f, bids, het = case
    m = ew.hypercube(dim, n, ref, f, boundary_ids=bids)
    if het:
        rng = np.random.default_rng(5)
        m.speed = rng.uniform(1.0, 4.0, m.n_cells)
        m.density = rng.uniform(1.0, 3.0, m.n_cells)
    op = ew.WaveEquationOperation(m, k, precision=precision)
    o = oracle.Problem.from_mesh(dim, k, m.vertices, m.neighbors, m.speed, m.density)
    u0 = o.project_reference(2)
    # explicit Euler is unstable for this operator: one short step only
    steps = 1 if name == "ExplEuler" else 4
    dt = o.time_step((0.05 if name == "ExplEuler" else 0.2) / k ** 1.5)
    a, b = u0.copy(), np.zeros_like(u0)
    vn = torch.from_numpy(u0.copy()).cuda()
    vnp = torch.zeros_like(vn)
    integ = driver.SUPPORTED[name]()
    for _ in range(steps):
        o.step(name, dt, a, b)
        a, b = b, a
        integ.perform_time_step(vn, vnp, dt, op)
        vn, vnp = vnp, vn
    op.synchronize()
    err = np.abs(vn.cpu().numpy() - a).max() / np.abs(a).max()
    # compensated (float-float, about 44 bits): FP64's bound on axis-aligned
    # cells, 1e-11 where the curved-cell metric terms enter
    tol = {"fp64": 1e-12, "mixed": 1e-5, "mixed_ff": 1e-12 if f == 0.0 else 1e-11}[precision]
    assert err < tol, err


def test_lsrk_step_rejects_unknown_scheme(env):
    ew, driver, oracle, torch = env
    from exwave_gb300.operator import _ptr
    op = ew.WaveEquationOperation(ew.hypercube(2, 2, 0, 0.0), 2)
    a, b = op.new_vector(), op.new_vector()
    assert op.L.ew_lsrk_step(op.ctx, 7, 0.01, _ptr(a), _ptr(b)) == -1  # EW_ERR_INVALID
    assert op.L.ew_lsrk_step(op.ctx, 0, 0.01, _ptr(a), _ptr(a)) == -1


@pytest.mark.parametrize("name", ["LSRK33R2", "LSRK45R3", "LSRK59R2", "SSPRK"])
def test_driver_runs_integrator(env, name):
    """The GPU time loop with the integrator against the oracle's replay of
    the reference's loop: time, step and every error column."""
    ew, driver, oracle, torch = env
    from exwave_gb300 import parameters
    p = parameters.parse_prm("set dimension = 2\nset fe_degree = 3\nset n_initial_intervals = 4\n"
                             "set grid_transform_factor = 0.0\nset time_integrator = %s\n"
                             "set cfl_number = 0.2\nset final_time = 0.2\n"
                             "set output_every_time = 0.1\n" % name)
    rows, dt = driver.run(p, precision="fp64")
    P = oracle.Problem.hypercube(2, 3, 4, 0, 0.0, p["boundary_id"])
    ref_rows, ref_dt = P.run_reference(name, p["cfl_number"], p["final_time"],
                                       p["output_every_time"], p["membrane_modes"],
                                       p["max_time_steps"])
    assert dt == pytest.approx(ref_dt, rel=1e-15)
    assert len(rows) == len(ref_rows)
    for mine, ref in zip(rows, ref_rows):
        assert mine[0] == pytest.approx(ref[0], rel=1e-14) and mine[1] == ref[1]
        for c in (2, 3, 4):
            assert mine[c] == pytest.approx(ref[c], rel=1e-9, abs=1e-15), (name, c, mine, ref)
        # error p post: CG to a relative residual of 1e-11 on both sides
        assert mine[5] == pytest.approx(ref[5], rel=1e-6), (name, mine, ref)


def test_aderadconfull_compensated_equals_fp64(env):
    """ADERADCONFULL (k+1 operator applications) in the compensated
    precision equals the FP64 path to 1e-12."""
    ew, driver, oracle, torch = env
    m = ew.hypercube(2, 6, 0, 0.0, boundary_ids=2)
    out = {}
    for prec in ("fp64", "mixed_ff"):
        op = ew.WaveEquationOperation(m, 3, precision=prec)
        u = op.project_membrane([1.0], [[1, 2]], 0.0)
        v = torch.zeros_like(u)
        dt = ew.time_step_size(m, 0.1 / 3 ** 1.5)
        for _ in range(4):
            op.aderadconfull_step(dt, u, v)
            u, v = v, u
        op.synchronize()
        out[prec] = u.cpu().numpy()
    err = abs(out["mixed_ff"] - out["fp64"]).max() / abs(out["fp64"]).max()
    assert err < 1e-12, err
