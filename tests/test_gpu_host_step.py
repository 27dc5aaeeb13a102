"""ew_lsrk45_step_host: the LSRK45 step on host vectors (the reference
integrator's storage) equals the device step bit for bit, whether the host
array is stepped in place (each call's copy in chained to the previous
call's copy out, chunk by chunk), ping-ponged between two arrays, or not
pinned, and whichever chunk schedule the mesh allows (curved cells: the
whole step between the copies; axis-aligned: the first and last stage by
chunks, or all five stages as a wavefront over the chunks);
ew_wait_host_copies orders the context stream after the copies."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ew_torch():
    import torch
    from exwave_gb300 import build
    build.build()
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    import exwave_gb300 as ew
    return ew, torch


def _device_steps(op, dt, u0, n, torch):
    a = torch.from_numpy(u0.copy()).cuda()
    b = torch.zeros_like(a)
    for _ in range(n):
        op.lsrk45_step(dt, a, b)
        a, b = b, a
    op.synchronize()
    return a.cpu().numpy()


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed_ff"])
# small meshes (neighbours several chunks apart: first and last stage by
# chunks) and meshes whose chunks hold more than one layer of cells (every
# neighbour in the same or the next chunk: all stages as a wavefront)
@pytest.mark.parametrize("dim,k,n,f", [(3, 3, 5, 0.0), (2, 5, 7, 0.05), (3, 2, 3, 0.0), (3, 2, 16, 0.0),
                                       (2, 3, 20, 0.0)])
def test_host_step_equals_device_step(ew_torch, precision, dim, k, n, f):
    ew, torch = ew_torch
    m = ew.hypercube(dim, n, 0, f, boundary_ids=[1, 2, 3, 1] if dim == 2 else [1, 2, 3, 1, 2, 3])
    rng = np.random.default_rng(dim * 10 + k)
    m.speed = rng.uniform(1.0, 3.0, m.n_cells)
    m.density = rng.uniform(1.0, 2.0, m.n_cells)
    op = ew.WaveEquationOperation(m, k, precision=precision)
    u0 = rng.standard_normal(op.n_dofs)
    dt = ew.time_step_size(m, 0.2 / k ** 1.5)
    steps = 4
    ref = _device_steps(op, dt, u0, steps, torch)
    # on a side stream, stepped in place in pinned memory
    s = torch.cuda.Stream()
    op.set_stream(s)
    host = torch.from_numpy(u0.copy()).pin_memory()
    for _ in range(steps):
        op.lsrk45_step_host(dt, host, host)
    op.synchronize()
    assert np.array_equal(host.numpy(), ref)
    # ping-pong between two pinned arrays; the stream fence then a stream sync
    ha = torch.from_numpy(u0.copy()).pin_memory()
    hb = torch.zeros_like(ha).pin_memory()
    for _ in range(steps):
        op.lsrk45_step_host(dt, ha, hb)
        ha, hb = hb, ha
    op.wait_host_copies()
    s.synchronize()
    assert np.array_equal(ha.numpy(), ref)
    # pageable host memory: the same values
    hp = torch.from_numpy(u0.copy())
    for _ in range(steps):
        op.lsrk45_step_host(dt, hp, hp)
    op.synchronize()
    assert np.array_equal(hp.numpy(), ref)
    op.close()


def test_host_step_rejects_device_tensors(ew_torch):
    ew, torch = ew_torch
    op = ew.WaveEquationOperation(ew.hypercube(2, 3, 0, 0.0), 2, precision="mixed")
    d = torch.zeros(op.n_dofs, dtype=torch.float64, device="cuda")
    with pytest.raises(ValueError):
        op.lsrk45_step_host(1e-3, d, d)
    op.close()
