"""Failure detection without a GPU fault.  The staged kernels wait on
mbarriers with a bounded number of polls; when a wait gives up, the kernel
raises a time-out flag, waits (bounded) for its own copies and returns, and
the host reports EW_ERR_DEVICE.  The diagnostic entry point runs that wait
on a barrier nothing completes, with nothing in flight: the call reports the
time-out, and the context computes correctly afterwards."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_wait_timeout_reports_and_context_recovers(oracle_mod):
    import torch
    from exwave_gb300 import build
    build.build()
    import exwave_gb300 as ew
    from exwave_gb300 import _lib
    L = _lib.load()
    m = ew.hypercube(3, 3, 0, 0.0, boundary_ids=2)
    op = ew.WaveEquationOperation(m, 3, precision="mixed")
    rc = L.ew_check_wait_timeout(op.ctx, 64)
    assert rc == -5
    assert "timed out" in L.ew_last_error(op.ctx).decode()
    # the flag was cleared; the next operator application runs normally
    o = oracle_mod.Problem.from_mesh(3, 3, m.vertices, m.neighbors, m.speed, m.density)
    u = np.random.default_rng(1).standard_normal(o.n_dofs)
    src = torch.from_numpy(u).cuda()
    dst = torch.zeros_like(src)
    op.apply(src, dst)
    op.synchronize()
    ref = o.apply(u)
    assert np.abs(dst.cpu().numpy() - ref).max() / np.abs(ref).max() < 2e-5
    assert L.ew_check_wait_timeout(op.ctx, 0) == -1
