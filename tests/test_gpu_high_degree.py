"""Degrees 8 to 12 against the oracle (the reference instantiates k = 1..12,
wave_equation_operations.cc:1695-1802; explicit_wave.cc:573-596).

In 2-D every kernel serves these degrees (the line kernel on axis-aligned
cells, the Cauchy-Kovalevskaya kernel for ADER).  In 3-D a cell has 9^3 to
13^3 Gauss points: the generic stage kernel runs them with several points
per thread, one cell per block, on axis-aligned and curved cells alike; ADER
(whose kernel keeps a whole cell's derivative levels in shared memory) is
built up to degree 7 there and answers EW_ERR_UNSUPPORTED above.

Tolerances as in the other parity tests: FP64 1e-12 relative to the largest
entry, compensated 1e-11; the FP32 operator's rounding grows with the size
of the derivative matrices (about k^2), so the mixed path is held to 1e-4
for one application at these degrees.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-12, "mixed_ff": 1e-11, "mixed": 1e-4}

CASES = [
    # dim, k, intervals, transform factor, boundary ids
    (2, 8, 3, 0.0, [1, 2, 3, 2]),
    (2, 10, 3, 0.1, 2),
    (2, 12, 2, 0.0, [3, 1, 2, 1]),
    (3, 8, 2, 0.05, [1, 2, 3, 1, 2, 3]),
    (3, 10, 2, 0.0, 2),
    (3, 12, 2, 0.05, [3, 3, 1, 2, 1, 2]),
]


def ids(c):
    return "d%dk%d_n%d_f%g" % c[:4]


@pytest.fixture(scope="module")
def env(oracle_mod):
    import torch
    from exwave_gb300 import build
    build.build()
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    import exwave_gb300 as ew
    return ew, oracle_mod, torch


def make(ew, oracle, dim, k, n, f, bids, seed):
    m = ew.hypercube(dim, n, 0, f, boundary_ids=bids)
    rng = np.random.default_rng(seed)
    m.speed = rng.uniform(1.0, 3.0, m.n_cells)
    m.density = rng.uniform(1.0, 2.0, m.n_cells)
    o = oracle.Problem.from_mesh(dim, k, m.vertices, m.neighbors, m.speed, m.density)
    return m, o


@pytest.mark.parametrize("case", CASES, ids=ids)
@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed_ff"])
def test_apply_high_degree(env, case, precision):
    ew, oracle, torch = env
    dim, k, n, f, bids = case
    m, o = make(ew, oracle, dim, k, n, f, bids, seed=k)
    op = ew.WaveEquationOperation(m, k, precision=precision)
    u = np.random.default_rng(100 + k).standard_normal(o.n_dofs)
    ref = o.apply(u)
    src = torch.from_numpy(u).cuda()
    dst = torch.zeros_like(src)
    op.apply(src, dst)
    op.synchronize()
    err = np.abs(dst.cpu().numpy() - ref).max() / np.abs(ref).max()
    print("apply %s %s: %.3e" % (ids(case), precision, err))
    assert err < TOL[precision], err


@pytest.mark.parametrize("case", CASES, ids=ids)
@pytest.mark.parametrize("precision", ["fp64", "mixed_ff"])
def test_lsrk45_high_degree(env, case, precision):
    """Three LSRK45 steps of a smooth field, single-step calls and one
    multi-step call, against the oracle's steps."""
    ew, oracle, torch = env
    dim, k, n, f, bids = case
    m, o = make(ew, oracle, dim, k, n, f, bids, seed=7 + k)
    op = ew.WaveEquationOperation(m, k, precision=precision)
    u0 = o.project_reference(2)
    dt = o.time_step(0.25 / k ** 1.5)
    a, b = u0.copy(), np.zeros_like(u0)
    for _ in range(3):
        o.lsrk45_step(dt, a, b)
        a, b = b, a
    vn = torch.from_numpy(u0.copy()).cuda()
    vnp = torch.zeros_like(vn)
    for _ in range(3):
        op.lsrk45_step(dt, vn, vnp)
        vn, vnp = vnp, vn
    x, y = torch.from_numpy(u0.copy()).cuda(), torch.zeros_like(vn)
    op.lsrk45_steps(dt, 3, x, y)
    op.synchronize()
    scale = np.abs(a).max()
    e1 = np.abs(vn.cpu().numpy() - a).max() / scale
    e2 = np.abs(y.cpu().numpy() - a).max() / scale
    print("lsrk45 %s %s: %.3e %.3e" % (ids(case), precision, e1, e2))
    assert e1 < TOL[precision] and e2 < TOL[precision], (e1, e2)


@pytest.mark.parametrize("k", [8, 12])
@pytest.mark.parametrize("precision", ["fp64", "mixed_ff"])
def test_ader_high_degree_2d(env, k, precision):
    """ADER of order k+1 in 2-D (the CK recursion through all its degree
    reductions) against the oracle, two steps on a curved mesh."""
    ew, oracle, torch = env
    m, o = make(ew, oracle, 2, k, 3, 0.1, [1, 2, 3, 1], seed=k)
    op = ew.WaveEquationOperation(m, k, precision=precision)
    u0 = o.project_reference(2)
    dt = o.time_step(0.2 / k ** 1.5)
    a, b = u0.copy(), np.zeros_like(u0)
    vn = torch.from_numpy(u0.copy()).cuda()
    vnp = torch.zeros_like(vn)
    for _ in range(2):
        o.ader_step(dt, a, b)
        a, b = b, a
        op.ader_step(dt, vn, vnp)
        vn, vnp = vnp, vn
    op.synchronize()
    err = np.abs(vn.cpu().numpy() - a).max() / np.abs(a).max()
    print("ader 2d k=%d %s: %.3e" % (k, precision, err))
    assert err < TOL[precision], err


def test_ader_3d_above_degree_7_is_unsupported(env):
    ew, oracle, torch = env
    from exwave_gb300 import _lib
    m = ew.hypercube(3, 2)
    op = ew.WaveEquationOperation(m, 8, precision="fp64")
    u = op.new_vector()
    v = op.new_vector()
    with pytest.raises(_lib.EwError) as ei:
        op.ader_step(1e-3, u, v)
    assert ei.value.code == -2 and "degrees up to 7" in str(ei.value)
