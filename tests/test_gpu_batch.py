"""Batched solves on the GPU: point sources and receivers against the CPU
oracle, equality of a solve alone and in a mixed batch, agreement with the
single-solve context, graphs vs direct launches, admission by HBM budget."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env(oracle_mod):
    import torch
    from exwave_gb300 import build
    build.build()
    assert torch.cuda.is_available()
    import exwave_gb300 as ew
    from exwave_gb300 import batch
    return ew, batch, oracle_mod, torch


def hetero_mesh(ew, n, seed):
    m = ew.hypercube(3, n, boundary_ids=[1, 1, 3, 3, 1, 2])
    rng = np.random.default_rng(seed)
    m.speed = rng.uniform(1.0, 4.0, m.n_cells)
    m.density = rng.uniform(1.0, 3.0, m.n_cells)
    return m


RECEIVERS = np.array([[0.31, 0.52, 0.47], [0.73, 0.21, 0.66], [0.5, 0.5, 0.9]])
SOURCE = ([0.43, 0.57, 0.38], 6.0, 1.0 / 6.0 * 0.2, 3.0)


@pytest.mark.parametrize("precision", ["fp64", "mixed_ff"])
def test_source_and_receivers_match_oracle(env, precision):
    """FP64 and compensated batches with a Ricker source and receivers
    against the oracle: state to 1e-12, receiver traces to 1e-11."""
    ew, batch, oracle, torch = env
    m = hetero_mesh(ew, 5, 3)
    k = 3
    dt = ew.time_step_size(m, 0.25 / k ** 1.5)
    b = batch.Batch(precision=precision, hbm_budget_bytes=1 << 30)
    sid = b.add(batch.Solve(m, k, dt, 12, source=SOURCE, receivers=RECEIVERS))
    o = oracle.Problem.from_mesh(3, k, m.vertices, m.neighbors, m.speed, m.density)
    u, v = o.zeros(), o.zeros()
    ref_rec = []
    t = 0.0
    for _ in range(12):
        o.lsrk45_step_source(dt, t, u, v, SOURCE[0], SOURCE[3], SOURCE[1], SOURCE[2])
        u, v = v, u
        t += dt
        ref_rec.append(o.point_values(u, RECEIVERS))
    b.step(6)
    b.step(6)
    b.synchronize()
    got = b.get_state(sid, torch.zeros(o.n_dofs, dtype=torch.float64, device="cuda")).cpu().numpy()
    assert np.abs(u).max() > 0
    assert np.abs(got - u).max() / np.abs(u).max() < 1e-12
    rec = b.receivers(sid)
    ref_rec = np.array(ref_rec)
    assert rec.shape == ref_rec.shape
    assert np.abs(rec - ref_rec).max() / np.abs(ref_rec).max() < 1e-11


def test_alone_equals_mixed_batch(env):
    """Continuous-batching invariant: a solve's result does not depend on
    what else shares the device (bitwise, mixed precision)."""
    ew, batch, oracle, torch = env
    mA = hetero_mesh(ew, 6, 1)
    kA = 4
    dtA = ew.time_step_size(mA, 0.25 / kA ** 1.5)
    solveA = batch.Solve(mA, kA, dtA, 9, source=SOURCE, receivers=RECEIVERS)
    alone = batch.Batch(precision="mixed", hbm_budget_bytes=1 << 30)
    ia = alone.add(solveA)
    alone.step(9)
    alone.synchronize()
    nd = mA.n_cells * 4 * (kA + 1) ** 3
    ref_state = alone.get_state(ia, torch.zeros(nd, dtype=torch.float64, device="cuda")).cpu().numpy()
    ref_rec = alone.receivers(ia)
    mix = batch.Batch(precision="mixed", hbm_budget_bytes=2 << 30)
    mB = hetero_mesh(ew, 4, 2)
    mix.add(batch.Solve(mB, 3, ew.time_step_size(mB, 0.02), 20, source=SOURCE, receivers=RECEIVERS))
    mix.step(2)  # A is admitted while B is running
    ib = mix.add(batch.Solve(mA, kA, dtA, 9, source=SOURCE, receivers=RECEIVERS))
    mC = hetero_mesh(ew, 3, 5)
    mix.add(batch.Solve(mC, 6, ew.time_step_size(mC, 0.01), 30, receivers=RECEIVERS))
    for _ in range(3):
        mix.step(3)
    mix.synchronize()
    st = mix.get_state(ib, torch.zeros(nd, dtype=torch.float64, device="cuda")).cpu().numpy()
    assert np.array_equal(st, ref_state)
    assert np.array_equal(mix.receivers(ib), ref_rec)


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed_ff"])
def test_batch_matches_single_context(env, precision):
    ew, batch, oracle, torch = env
    m = ew.hypercube(3, 5)
    k = 5
    dt = ew.time_step_size(m, 0.25 / k ** 1.5)
    op = ew.WaveEquationOperation(m, k, precision=precision)
    u0 = op.project_membrane([1.0, 0.5], [[1, 1, 1], [2, 1, 3]])
    b = batch.Batch(precision=precision, hbm_budget_bytes=1 << 30)
    sid = b.add(batch.Solve(m, k, dt, 4))
    b.set_state(sid, u0)
    b.step(4)
    vn, vnp = u0.clone(), torch.zeros_like(u0)
    if precision == "mixed_ff":
        # one multi-step call: the state as float pairs between steps, like
        # the batch
        op.lsrk45_steps(dt, 4, vn, vnp)
        vn = vnp
    else:
        for _ in range(4):
            op.lsrk45_step(dt, vn, vnp)
            vn, vnp = vnp, vn
    op.synchronize()
    b.synchronize()
    got = b.get_state(sid, torch.zeros_like(u0))
    if precision in ("fp64", "mixed_ff"):
        # the same kernels on the same state between steps: bit-identical
        assert torch.equal(got, vn)
    else:
        # the batch carries the state's FP32 split between steps and runs
        # other kernel instantiations, whose FP32 operations may round
        # differently: agreement to FP32 round-off
        err = ((got - vn).abs().max() / vn.abs().max()).item()
        assert err < 1e-6, err


def test_graphs_equal_direct_launches(env):
    ew, batch, oracle, torch = env
    m = hetero_mesh(ew, 4, 9)
    res = []
    for graphs in (True, False):
        b = batch.Batch(precision="mixed", hbm_budget_bytes=1 << 30, use_graphs=graphs)
        sid = b.add(batch.Solve(m, 2, 1e-3, 7, source=SOURCE, receivers=RECEIVERS))
        b.step(7)
        b.synchronize()
        res.append(b.receivers(sid))
        assert b.kernel_launches() == 7 * 6
    assert np.array_equal(res[0], res[1])


def test_admission_by_budget(env):
    ew, batch, oracle, torch = env
    m = ew.hypercube(3, 8)
    s = batch.Solve(m, 4, 1e-3, 10)
    b0 = batch.Batch(precision="mixed", hbm_budget_bytes=1 << 30)
    need = b0.solve_bytes(s)
    b0.close()
    b = batch.Batch(precision="mixed", hbm_budget_bytes=int(need * 1.5))
    sid = b.add(s)
    with pytest.raises(Exception) as ei:
        b.add(batch.Solve(m, 4, 1e-3, 10))
    assert getattr(ei.value, "code", None) == -4
    b.remove(sid)
    b.add(batch.Solve(m, 4, 1e-3, 10))
    assert b.bytes_free() >= 0
