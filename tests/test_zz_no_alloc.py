"""The allocation-free LSRK45 step (ew_lsrk45_step_static).

Some callers cannot let the library allocate device memory while they step
a solution: applications that hand all device memory to their own pool or
run under a fixed device-memory budget, and latency-sensitive loops, where
cudaMalloc would synchronise the device or fail.  ew_lsrk45_step_static
keeps its stage scratch in a static device array instead of the context's
buffers; this test calls it through the C ABI, twice in a row, and checks
every result against the regular ew_lsrk45_step, for both precisions, on an
axis-aligned 3-D mesh (the line kernel), a curved 3-D mesh (the staged
curved-cell kernel) and a curved 2-D mesh, and that contexts above the
array's size limit are rejected.  Both steps run the same kernels in the same
order on the same inputs, only the scratch lives elsewhere, so the results
must be bitwise equal.  Named to run last in the suite.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MESHES = {
    # dim, intervals, transform factor, boundary ids, degree
    "cart3d": (3, 5, 0.0, [1, 2, 3, 1, 2, 3], 3),
    "curved3d": (3, 4, 0.1, [3, 1, 2, 2, 1, 3], 4),
    "curved2d": (2, 6, 0.15, [1, 2, 3, 2], 5),
}


@pytest.fixture(scope="module")
def env():
    import torch
    from exwave_gb300 import build
    build.build()
    assert torch.cuda.is_available(), "GPU test"
    import exwave_gb300 as ew
    from exwave_gb300 import _lib
    return ew, _lib, torch


@pytest.mark.parametrize("mesh", sorted(MESHES))
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_static_step_matches_regular_step(env, precision, mesh):
    ew, _lib, torch = env
    L = _lib.load()
    dim, n, f, bids, k = MESHES[mesh]
    m = ew.hypercube(dim, n, 0, f, boundary_ids=bids)
    op = ew.WaveEquationOperation(m, k, precision=precision)
    dt = ew.time_step_size(m, 0.25 / k ** 1.5)
    kv = [[1, 1, 1], [2, 1, 3]] if dim == 3 else [[1, 1], [2, 3]]
    u0 = op.project_membrane([1.0, 0.5], kv)
    ref_n, ref_np = u0.clone(), torch.zeros_like(u0)
    st_n, st_np = u0.clone(), torch.zeros_like(u0)
    for call in range(2):
        op.lsrk45_step(dt, ref_n, ref_np)
        rc = L.ew_lsrk45_step_static(op.ctx, dt, ctypes.c_void_p(st_n.data_ptr()),
                                     ctypes.c_void_p(st_np.data_ptr()))
        _lib.check(rc, op.ctx)
        op.synchronize()
        ref = ref_np.cpu().numpy()
        got = st_np.cpu().numpy()
        assert np.abs(ref).max() > 0
        assert np.array_equal(got, ref), (precision, mesh, call, np.abs(got - ref).max())
        ref_n, ref_np = ref_np, ref_n
        st_n, st_np = st_np, st_n


def test_static_step_rejects_too_large(env):
    ew, _lib, torch = env
    L = _lib.load()
    m = ew.hypercube(3, 26)  # 17576 cells x 4 x 8^3 points > the array's limit
    op = ew.WaveEquationOperation(m, 7, precision="mixed")
    assert op.n_dofs > (64 << 20) // 8 - 64
    u = op.new_vector()
    v = op.new_vector()
    rc = L.ew_lsrk45_step_static(op.ctx, 1e-4, ctypes.c_void_p(u.data_ptr()),
                                 ctypes.c_void_p(v.data_ptr()))
    assert rc == -6
    assert "static scratch" in L.ew_last_error(op.ctx).decode()
