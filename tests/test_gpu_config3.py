"""The curved two-layer ADER configuration, small, against the oracle.

A replica of the 40^3 configuration at 6^3 cells: the vertex map
x_i += 0.03 prod_d sin(2 pi x_d), c = rho = 1 below z = 0.5 and c = 3,
rho = 2 above, free surface (id 2) on top and rigid walls (id 1) elsewhere,
a Gaussian pressure pulse of width 0.05 at a seeded point of the lower
layer, ADER of order k+1 with k = 4, CFL 0.15, 20 steps, 8 seeded receivers
sampled after every step.  Every precision is checked against the oracle's
FP64 run of the same inputs (ADER: ArbitraryHighOrderDG::perform_time_step,
time_integrators.cc:37-50, with WaveEquationOperationADER::apply_ader,
wave_equation_operations.cc:1346-1381):

- FP64: state and receiver traces to 1e-12 relative (round-off of reordered
  sums);
- compensated (float-float operator): 1e-11 relative;
- mixed (FP32 operator, FP64 state, float-pair Taylor sum): 2e-6 relative
  for the state and the traces after 20 steps (one FP32 operator
  application is accurate to about 2e-5 of its largest entry; the ADER
  update adds dt times that to the FP64 state).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-12, "mixed_ff": 1e-11, "mixed": 2e-6}


@pytest.fixture(scope="module")
def env(oracle_mod):
    import torch
    from exwave_gb300 import build
    build.build()
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    import exwave_gb300 as ew
    return ew, oracle_mod, torch


def config3_mesh(ew, n):
    m = ew.hypercube(3, n, 0, 0.03, transform="sine_all", boundary_ids=[1, 1, 1, 1, 1, 2])
    return ew.layered_materials(m, 0.5, below=(1.0, 1.0), above=(3.0, 2.0))


@pytest.mark.parametrize("dim,k,n,f", [(3, 4, 4, 0.03), (2, 5, 6, 0.1), (3, 2, 5, 0.0)])
def test_project_gaussian_matches_oracle(env, dim, k, n, f):
    """ew_project_gaussian equals the oracle's sampled pulse to 1e-14."""
    ew, oracle, torch = env
    m = ew.hypercube(dim, n, 0, f, transform="sine_all" if f else "reference")
    op = ew.WaveEquationOperation(m, k, precision="fp64")
    o = oracle.Problem.from_mesh(dim, k, m.vertices, m.neighbors, m.speed, m.density)
    x0 = [0.43, 0.31, 0.27][:dim]
    got = op.project_gaussian(x0, 0.08, 1.3)
    op.synchronize()
    ref = o.project_gaussian(x0, 0.08, 1.3)
    np.testing.assert_allclose(got.cpu().numpy(), ref, rtol=1e-14, atol=1e-14)


@pytest.mark.parametrize("precision", ["fp64", "mixed_ff", "mixed"])
def test_config3_replica_matches_oracle(env, precision):
    ew, oracle, torch = env
    k, n, steps = 4, 6, 20
    m = config3_mesh(ew, n)
    op = ew.WaveEquationOperation(m, k, precision=precision)
    o = oracle.Problem.from_mesh(3, k, m.vertices, m.neighbors, m.speed, m.density)
    rng = np.random.default_rng(3)
    x0 = [rng.uniform(0.2, 0.8), rng.uniform(0.2, 0.8), rng.uniform(0.15, 0.35)]
    pts = rng.uniform(0.1, 0.9, (8, 3))
    dt = ew.time_step_size(m, 0.15 / k ** 1.5)
    u = o.project_gaussian(x0, 0.05)
    vn = op.project_gaussian(x0, 0.05)
    vnp = torch.zeros_like(vn)
    op.set_receivers(pts)
    a, b = u.copy(), np.zeros_like(u)
    tr_gpu, tr_ref = [], []
    for _ in range(steps):
        o.ader_step(dt, a, b)
        a, b = b, a
        tr_ref.append(o.point_values(a, pts))
        op.ader_step(dt, vn, vnp)
        vn, vnp = vnp, vn
        tr_gpu.append(op.sample_receivers(vn)[:, 3].clone())
    op.synchronize()
    got = vn.cpu().numpy()
    err = np.abs(got - a).max() / np.abs(a).max()
    tg = torch.stack(tr_gpu).cpu().numpy()
    tref = np.array(tr_ref)
    terr = np.abs(tg - tref).max() / np.abs(tref).max()
    print("config-3 replica %s: state %.3e, traces %.3e" % (precision, err, terr))
    assert np.isfinite(got).all()
    assert err < TOL[precision], err
    assert terr < TOL[precision], terr
