"""The post-processed pressure error ("error p post", compute_post_pressure,
wave_equation_operations.cc:784-848) on the GPU against the oracle, at the
edges of the per-cell kernel: k=1 in 2-D (9 points in a block of 32
threads), k=7 in 3-D (729 threads, 70 KB of shared memory), curved cells,
boundary faces of every kind; and the mixed context (FP32 operator for
du/dt) against the FP64 one.

Tolerances: FP64 1e-8 relative (both sides stop their CG at a relative
residual of 1e-11, so round-off can move the stopping iteration); mixed
1e-4 relative to the FP64 error."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [
    # dim, k, intervals, transform, boundary ids
    (2, 1, 4, 0.0, 2),
    (2, 4, 3, 0.1, [1, 2, 3, 1]),
    (3, 3, 2, 0.1, 2),
    (3, 7, 2, 0.0, [3, 1, 2, 2, 1, 3]),
]


@pytest.fixture(scope="module")
def env(oracle_mod):
    import torch
    from exwave_gb300 import build
    build.build()
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    import exwave_gb300 as ew
    return ew, oracle_mod, torch


@pytest.mark.parametrize("case", CASES, ids=lambda c: "d%dk%d_n%d_f%g" % c[:4])
def test_post_error_matches_oracle(env, case):
    ew, oracle, torch = env
    dim, k, n, f, bids = case
    m = ew.hypercube(dim, n, 0, f, boundary_ids=bids)
    o = oracle.Problem.from_mesh(dim, k, m.vertices, m.neighbors, m.speed, m.density)
    # a state with velocity and pressure: three LSRK45 steps from mode 2
    u = o.project_reference(2)
    dt = o.time_step(0.2 / k ** 1.5)
    a, b = u.copy(), np.zeros_like(u)
    for _ in range(3):
        o.lsrk45_step(dt, a, b)
        a, b = b, a
    t = 3 * dt
    ref = o.post_error_reference(a, 2, t)
    amps, kv = ew.reference_mode(dim, 2)
    errs = {}
    for prec in ("fp64", "mixed", "mixed_ff"):
        op = ew.WaveEquationOperation(m, k, precision=prec)
        errs[prec] = op.l2_error_post(torch.from_numpy(a.copy()).cuda(), amps, kv, t)
        op.close()
    assert ref > 0.0
    assert abs(errs["fp64"] - ref) <= 1e-8 * ref, (errs, ref)
    assert abs(errs["mixed"] - errs["fp64"]) <= 1e-4 * errs["fp64"], errs
    assert abs(errs["mixed_ff"] - errs["fp64"]) <= 1e-8 * errs["fp64"], errs


def test_post_error_rejects_null_state(env):
    ew, oracle, torch = env
    op = ew.WaveEquationOperation(ew.hypercube(2, 2, 0, 0.0), 2)
    out = np.zeros(1)
    amps = np.array([1.0])
    kv = np.array([[1, 1, 0]], dtype=np.int32)
    rc = op.L.ew_l2_error_post_membrane(op.ctx, None, 1, amps.ctypes.data, kv.ctypes.data, 0.0,
                                        out.ctypes.data)
    assert rc == -1
