"""GPU parity: the CUDA kernels, called through the C ABI, against the CPU
oracle on the same meshes and seeded inputs.

Tolerances: FP64 path 1e-12 relative to the largest entry (round-off of
reordered sums); mixed path (FP32 operator, FP64 state) 2e-5 relative for a
single operator application; compensated path (float-float operator, FP64
state) 1e-12 on axis-aligned cells and 1e-11 where curved-cell metric terms or
the ADER derivative chain enter (float-float carries about 44 bits, a unit
round-off near 500 times FP64's)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
MIXED_TOL = 2e-5
FF_TOL = 1e-11
MIXED_ADER_TOL = 5e-5
MIXED_ADER_STEP_TOL = 1e-6


@pytest.fixture(scope="module")
def env(oracle_mod):
    import torch
    from exwave_gb300 import build
    build.build()
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    import exwave_gb300 as ew
    return ew, oracle_mod, torch


def make_case(ew, dim, n, ref, f, bids, hetero, seed):
    m = ew.hypercube(dim, n, ref, f, boundary_ids=bids)
    if hetero:
        rng = np.random.default_rng(seed)
        m.speed = rng.uniform(1.0, 4.0, m.n_cells)
        m.density = rng.uniform(1.0, 3.0, m.n_cells)
    return m


CASES = [
    # dim, k, intervals, refinements, transform, boundary ids, heterogeneous
    (2, 1, 20, 0, 0.0, 2, False),
    (2, 4, 16, 0, 0.0, 2, False),
    (2, 3, 5, 2, 0.1, 2, False),
    (2, 6, 5, 1, 0.0, [1, 2, 3, 1], True),
    (2, 2, 6, 0, 0.15, [3, 3, 1, 2], True),
    (2, 5, 4, 1, 0.1, [1, 1, 3, 3], True),
    (2, 7, 3, 0, 0.0, 2, True),
    (3, 1, 4, 0, 0.1, 2, False),
    (3, 2, 4, 0, 0.0, [1, 2, 3, 1, 2, 3], True),
    (3, 3, 3, 1, 0.1, [3, 1, 2, 2, 1, 3], True),
    (3, 4, 5, 0, 0.1, 2, False),
    (3, 5, 4, 0, 0.0, 2, True),
    (3, 6, 3, 0, 0.05, [1, 1, 1, 1, 1, 2], True),
    (3, 7, 3, 0, 0.05, 2, False),
]


def ids(c):
    return "d%dk%d_n%d_r%d_f%g_%s" % (c[0], c[1], c[2], c[3], c[4], "het" if c[6] else "hom")


@pytest.mark.parametrize("case", CASES, ids=ids)
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_apply(env, case, precision):
    ew, oracle, torch = env
    dim, k, n, ref, f, bids, het = case
    m = make_case(ew, dim, n, ref, f, bids, het, seed=k + 10 * dim)
    op = ew.WaveEquationOperation(m, k, precision=precision)
    o = oracle.Problem.from_mesh(dim, k, m.vertices, m.neighbors, m.speed, m.density)
    rng = np.random.default_rng(1234 + k)
    u = rng.standard_normal(o.n_dofs)
    ref_out = o.apply(u)
    src = torch.from_numpy(u).cuda()
    dst = torch.zeros_like(src)
    op.apply(src, dst)
    op.synchronize()
    got = dst.cpu().numpy()
    err = np.abs(got - ref_out).max() / np.abs(ref_out).max()
    assert err < (FP64_TOL if precision == "fp64" else MIXED_TOL), err


@pytest.mark.parametrize("case", [CASES[i] for i in (1, 2, 3, 9, 10, 12)], ids=ids)
def test_lsrk45_steps(env, case):
    ew, oracle, torch = env
    dim, k, n, ref, f, bids, het = case
    m = make_case(ew, dim, n, ref, f, bids, het, seed=7)
    op = ew.WaveEquationOperation(m, k, precision="fp64")
    o = oracle.Problem.from_mesh(dim, k, m.vertices, m.neighbors, m.speed, m.density)
    u0 = o.project_reference(2)
    dt = o.time_step(0.3 / k ** 1.5)
    a, b = u0.copy(), np.zeros_like(u0)
    vn = torch.from_numpy(u0.copy()).cuda()
    vnp = torch.zeros_like(vn)
    for _ in range(3):
        o.lsrk45_step(dt, a, b)
        a, b = b, a
        op.lsrk45_step(dt, vn, vnp)
        vn, vnp = vnp, vn
    op.synchronize()
    err = np.abs(vn.cpu().numpy() - a).max() / np.abs(a).max()
    assert err < FP64_TOL, err


@pytest.mark.parametrize("case", [CASES[i] for i in (1, 2, 3, 8, 11)], ids=ids)
@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed_ff"])
@pytest.mark.parametrize("n_steps", [1, 2, 5])
def test_lsrk45_steps_call(env, case, precision, n_steps):
    """ew_lsrk45_steps against n_steps calls of ew_lsrk45_step and the FP64
    oracle.  FP64: identical.  Mixed: on Cartesian meshes the call keeps the
    state as a float pair between its steps (exactly the FP64 state the
    single-step path would round to) and runs other kernel instantiations,
    whose FP32 operations may round differently; the two paths then agree to
    FP32 round-off (1e-6 relative after 5 steps) and stay as close to the
    FP64 oracle as the single-step path.  Compensated: on Cartesian meshes the
    call keeps the state as float pairs between its steps, where single steps
    round it to FP64 and split it again; the two agree to 1e-13 relative and
    both equal the oracle to the compensated tolerance."""
    ew, oracle, torch = env
    dim, k, n, ref, f, bids, het = case
    m = make_case(ew, dim, n, ref, f, bids, het, seed=3)
    op = ew.WaveEquationOperation(m, k, precision=precision)
    o = oracle.Problem.from_mesh(dim, k, m.vertices, m.neighbors, m.speed, m.density)
    u0h = o.project_reference(2)
    u0 = torch.from_numpy(u0h.copy()).cuda()
    dt = o.time_step(0.3 / k ** 1.5)
    vn, vnp = u0.clone(), torch.zeros_like(u0)
    for _ in range(n_steps):
        op.lsrk45_step(dt, vn, vnp)
        vn, vnp = vnp, vn
    a, b = u0.clone(), torch.full_like(u0, float("nan"))
    op.lsrk45_steps(dt, n_steps, a, b)
    op.synchronize()
    single, multi = vn.cpu().numpy(), b.cpu().numpy()
    scale = np.abs(single).max()
    if precision == "fp64":
        assert np.array_equal(multi, single)
        return
    if precision == "mixed_ff":
        assert np.abs(multi - single).max() / scale < 1e-13
        x, y = u0h.copy(), np.zeros_like(u0h)
        for _ in range(n_steps):
            o.lsrk45_step(dt, x, y)
            x, y = y, x
        assert np.abs(multi - x).max() / scale < FF_TOL
        return
    assert np.abs(multi - single).max() / scale < 1e-6
    x, y = u0h.copy(), np.zeros_like(u0h)
    for _ in range(n_steps):
        o.lsrk45_step(dt, x, y)
        x, y = y, x
    e_single = np.abs(single - x).max() / scale
    e_multi = np.abs(multi - x).max() / scale
    assert e_multi < 1e-5 and e_multi < 2.0 * e_single + 1e-9, (e_multi, e_single)


@pytest.mark.parametrize("case", [CASES[i] for i in (1, 2, 5, 9, 10, 13)], ids=ids)
@pytest.mark.parametrize("post", [False, True])
@pytest.mark.parametrize("precision", ["fp64", "mixed_ff", "mixed"])
def test_ader_step(env, case, post, precision):
    """apply_ader and two ADER steps (± post) against the oracle, on the FP64
    (1e-12 relative), the compensated float-float (1e-11 relative) and the
    mixed path (FP32 operator with a float-pair Taylor sum: 5e-5 relative for
    apply_ader, whose stage input T is itself rounded to FP32 -- measured up
    to 2.3e-5; 1e-6 relative for the FP64 state after two steps, which adds
    dt times such an application -- measured up to 1.4e-7)."""
    ew, oracle, torch = env
    dim, k, n, ref, f, bids, het = case
    m = make_case(ew, dim, n, ref, f, bids, het, seed=11)
    op = ew.WaveEquationOperation(m, k, precision=precision, use_ader_post=post)
    o = oracle.Problem.from_mesh(dim, k, m.vertices, m.neighbors, m.speed, m.density)
    o.set_ader_post(post)
    u0 = o.project_reference(2)
    dt = o.time_step(0.2 / k ** 1.5)
    # apply_ader (reference sign: dst = -M^-1 A(T))
    ref_dst = o.apply_ader(dt, u0)
    src = torch.from_numpy(u0.copy()).cuda()
    dst = torch.zeros_like(src)
    op.apply_ader(src, dst, dt)
    op.synchronize()
    tol = {"fp64": FP64_TOL, "mixed_ff": FF_TOL, "mixed": MIXED_ADER_TOL}[precision]
    err = np.abs(dst.cpu().numpy() - ref_dst).max() / np.abs(ref_dst).max()
    assert err < tol, err
    tol = {"fp64": FP64_TOL, "mixed_ff": FF_TOL, "mixed": MIXED_ADER_STEP_TOL}[precision]
    # two full steps
    a, b = u0.copy(), np.zeros_like(u0)
    vn = torch.from_numpy(u0.copy()).cuda()
    vnp = torch.zeros_like(vn)
    for _ in range(2):
        o.ader_step(dt, a, b)
        a, b = b, a
        op.ader_step(dt, vn, vnp)
        vn, vnp = vnp, vn
    op.synchronize()
    err2 = np.abs(vn.cpu().numpy() - a).max() / np.abs(a).max()
    print("ader %s post=%d: apply_ader %.3e, two steps %.3e" % (precision, post, err, err2))
    assert err2 < tol, err2


def test_rk_update_matches_reference_updater(env):
    ew, oracle, torch = env
    m = ew.hypercube(2, 4)
    op = ew.WaveEquationOperation(m, 2)
    rng = np.random.default_rng(5)
    v1, v2, v3 = (rng.standard_normal(op.n_dofs) for _ in range(3))
    for last in (0, 1):
        a1, a2, a3 = v1.copy(), v2.copy(), v3.copy()
        oracle.lib().ewo_rk_update(op.n_dofs, 0.3, -0.7, last, *(oracle._dp(x) for x in (a1, a2, a3)))
        g1, g2, g3 = (torch.from_numpy(x.copy()).cuda() for x in (v1, v2, v3))
        op.rk_update(0.3, -0.7, last, g1, g2, g3)
        op.synchronize()
        np.testing.assert_allclose(g2.cpu().numpy(), a2, rtol=1e-15, atol=1e-15)
        np.testing.assert_allclose(g3.cpu().numpy(), a3, rtol=1e-15, atol=1e-15)


def test_two_register_contract(env):
    """vec_np receives the new state; vec_n is a register; equal pointers are
    rejected (the in-place aliasing hazard of the fused update)."""
    ew, oracle, torch = env
    m = ew.hypercube(3, 3)
    op = ew.WaveEquationOperation(m, 3)
    u = op.project_membrane(*ew.reference_mode(3, 1))
    with pytest.raises(Exception):
        op.lsrk45_step(1e-3, u, u)
    with pytest.raises(Exception):
        op.ader_step(1e-3, u, u)


def test_projection_and_errors_match_oracle(env):
    ew, oracle, torch = env
    m = ew.hypercube(3, 4, 0, 0.1)
    o = oracle.Problem.from_mesh(3, 4, m.vertices, m.neighbors, m.speed, m.density)
    op = ew.WaveEquationOperation(m, 4)
    amps, kv = [1.0, 0.5], [[1, 1, 1], [2, 1, 3]]
    u = op.project_membrane(amps, kv, 0.3)
    ref = o.project_modes(amps, kv, 0.3)
    np.testing.assert_allclose(u.cpu().numpy(), ref, rtol=0, atol=1e-14)
    e_gpu = op.l2_errors(u * 1.01, amps, kv, 0.3)
    e_ref = o.errors_modes(ref * 1.01, amps, kv, 0.3)
    np.testing.assert_allclose(e_gpu, e_ref, rtol=1e-12)


EDGE = [
    # dim, k, intervals, transform, boundary ids, cells per block
    (2, 3, 1, 0.0, [1, 2, 3, 1], 1),      # one cell: every face a boundary
    (3, 2, 1, 0.1, [3, 1, 2, 2, 1, 3], 1),  # one curved cell
    (3, 5, 3, 0.0, 2, 4),                  # 27 cells, items of 4: the last holds 3
    (2, 4, 5, 0.0, [1, 1, 3, 3], 3),      # 25 cells, items of 3: the last holds 1
    (3, 3, 3, 0.1, 2, 5),                  # curved, 27 cells, items of 5
    # axis-aligned 3-D degrees whose neighbour arrays come by bulk copy
    (3, 3, 4, 0.0, [1, 2, 3, 1, 2, 3], 5),  # 64 cells, items of 5: the last holds 4
    (3, 6, 3, 0.0, [3, 1, 2, 2, 1, 3], 2),  # 27 cells, items of 2: the last holds 1
    (3, 7, 2, 0.0, [2, 3, 1, 1, 3, 2], 1),  # 8 cells, one per item
]


@pytest.mark.parametrize("case", EDGE, ids=lambda c: "d%dk%d_n%d_f%g_cb%d" % (c[0], c[1], c[2], c[3], c[5]))
@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed_ff"])
def test_ragged_work_lists_and_single_cells(env, case, precision):
    """Meshes of one cell (all faces on the boundary) and work lists whose
    last item is only partly filled: apply and three LSRK45 steps against
    the oracle."""
    ew, oracle, torch = env
    dim, k, n, f, bids, cb = case
    m = ew.hypercube(dim, n, 0, f, boundary_ids=bids)
    op = ew.WaveEquationOperation(m, k, precision=precision, cells_per_block=cb)
    o = oracle.Problem.from_mesh(dim, k, m.vertices, m.neighbors, m.speed, m.density)
    tol = {"fp64": FP64_TOL, "mixed": MIXED_TOL,
           "mixed_ff": FP64_TOL if f == 0.0 else FF_TOL}[precision]
    rng = np.random.default_rng(77 + k)
    u = rng.standard_normal(o.n_dofs)
    ref_out = o.apply(u)
    src = torch.from_numpy(u).cuda()
    dst = torch.zeros_like(src)
    op.apply(src, dst)
    op.synchronize()
    err = np.abs(dst.cpu().numpy() - ref_out).max() / np.abs(ref_out).max()
    assert err < tol, ("apply", err)
    dt = o.time_step(0.2 / k ** 1.5)
    a, b = u.copy(), np.zeros_like(u)
    for _ in range(3):
        o.lsrk45_step(dt, a, b)
        a, b = b, a
    vn, vnp = src.clone(), torch.zeros_like(src)
    op.lsrk45_steps(dt, 3, vn, vnp)
    op.synchronize()
    err = np.abs(vnp.cpu().numpy() - a).max() / np.abs(a).max()
    assert err < tol, ("lsrk45", err)


@pytest.mark.parametrize("case", [CASES[i] for i in (0, 1, 2, 3, 5, 6, 8, 9, 10, 11)], ids=ids)
def test_compensated_apply_and_steps(env, case):
    """EW_PREC_MIXED_FF on axis-aligned and curved meshes (FP64 inputs split exactly into
    float pairs, stage inputs kept as float pairs, the operator's arithmetic
    and coefficients in float-float): apply and three LSRK45 steps equal the
    FP64 oracle to 1e-12 relative on axis-aligned cells, the FP64 path's own
    bound, and to 1e-11 on curved cells."""
    ew, oracle, torch = env
    dim, k, n, ref, f, bids, het = case
    m = make_case(ew, dim, n, ref, f, bids, het, seed=k + 10 * dim)
    op = ew.WaveEquationOperation(m, k, precision="mixed_ff")
    o = oracle.Problem.from_mesh(dim, k, m.vertices, m.neighbors, m.speed, m.density)
    rng = np.random.default_rng(99 + k)
    u = rng.standard_normal(o.n_dofs)
    ref_out = o.apply(u)
    src = torch.from_numpy(u).cuda()
    dst = torch.zeros_like(src)
    op.apply(src, dst)
    op.synchronize()
    tol = FP64_TOL if f == 0.0 else FF_TOL
    err = np.abs(dst.cpu().numpy() - ref_out).max() / np.abs(ref_out).max()
    assert err < tol, err
    u0 = o.project_reference(2)
    dt = o.time_step(0.2 / k ** 1.5)
    a, b = u0.copy(), np.zeros_like(u0)
    for _ in range(3):
        o.lsrk45_step(dt, a, b)
        a, b = b, a
    vn = torch.from_numpy(u0.copy()).cuda()
    vnp = torch.zeros_like(vn)
    op.lsrk45_steps(dt, 3, vn, vnp)
    op.synchronize()
    err = np.abs(vnp.cpu().numpy() - a).max() / np.abs(a).max()
    assert err < tol, err


def test_compensated_rejects_static_step(env):
    ew, oracle, torch = env
    op = ew.WaveEquationOperation(ew.hypercube(2, 3, 0, 0.0), 2, precision="mixed_ff")
    a, b = op.new_vector(), op.new_vector()
    from exwave_gb300.operator import _ptr
    assert op.L.ew_lsrk45_step_static(op.ctx, 0.01, _ptr(a), _ptr(b)) == -2  # EW_ERR_UNSUPPORTED


@pytest.mark.parametrize("case", [CASES[i] for i in (1, 5, 10, 12, 13)], ids=ids)
@pytest.mark.parametrize("post", [False, True])
@pytest.mark.parametrize("precision", ["fp64", "mixed_ff", "mixed"])
def test_ader_step_without_spectral_evaluation(env, case, post, precision):
    """ADER with spectral_evaluation = false (the CK recursion at full degree
    throughout) against the oracle: two steps, the tolerances of test_ader_step."""
    ew, oracle, torch = env
    dim, k, n, ref, f, bids, het = case
    m = make_case(ew, dim, n, ref, f, bids, het, seed=12)
    op = ew.WaveEquationOperation(m, k, precision=precision, use_ader_post=post,
                                  spectral_evaluation=False)
    o = oracle.Problem.from_mesh(dim, k, m.vertices, m.neighbors, m.speed, m.density)
    o.set_ader_post(post)
    o.set_spectral(False)
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
    tol = {"fp64": FP64_TOL, "mixed_ff": FF_TOL, "mixed": MIXED_ADER_STEP_TOL}[precision]
    err = np.abs(vn.cpu().numpy() - a).max() / np.abs(a).max()
    assert err < tol, err


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed_ff"])
def test_neighbour_staging_layouts_agree(env, precision):
    """The line kernel's two shared-memory layouts of the neighbour data (the
    autotuner's layout knob) compute the same values in the same order:
    bitwise equal results, over three LSRK45 steps of a heterogeneous 3-D
    mesh of degree 5 with every boundary id."""
    ew, oracle, torch = env
    m = make_case(ew, 3, 4, 0, 0.0, [1, 2, 3, 1, 2, 3], True, seed=21)
    outs = []
    for staging in (1, 2):
        op = ew.WaveEquationOperation(m, 5, precision=precision, nb_staging=staging)
        u = op.project_membrane([1.0, 0.5], [[1, 1, 1], [2, 1, 3]])
        v = torch.zeros_like(u)
        dt = ew.time_step_size(m, 0.25 / 5 ** 1.5)
        op.lsrk45_steps(dt, 3, u, v)
        op.synchronize()
        outs.append(v.cpu().numpy())
        op.close()
    assert np.abs(outs[0]).max() > 0
    assert np.array_equal(outs[0], outs[1])
