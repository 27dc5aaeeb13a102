"""Serving loop: requests arriving while others run are admitted as memory
frees up, every request completes, and each request's receiver trace is
the same as when it runs alone."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_continuous_batching_matches_alone():
    from exwave_gb300 import build
    build.build()
    from exwave_gb300 import serve
    from exwave_gb300.batch import Batch
    reqs = serve.draw_requests(12, rate=200.0, seed=42, degrees=(2, 4), cells=(3, 5),
                               end_time=(0.02, 0.06), n_receivers=3)
    # budget for about three resident solves: forces queueing and admission
    # while others are on the device
    probe = Batch(precision="mixed", hbm_budget_bytes=1 << 30)
    sizes = [probe.solve_bytes(r.make_solve()) for r in reqs]
    probe.close()
    srv = serve.Server(precision="mixed", hbm_budget_bytes=int(3.2 * max(sizes)), steps_per_tick=2)
    stats = srv.run(reqs)
    assert stats["completed"] == len(reqs)
    assert stats["peak_active"] >= 2
    assert stats["latency_p99_s"] >= stats["latency_p50_s"] > 0
    for r in reqs:
        alone = Batch(precision="mixed", hbm_budget_bytes=1 << 30)
        sid = alone.add(r.make_solve())
        alone.step(r.n_steps)
        alone.synchronize()
        ref = alone.receivers(sid)
        got = np.concatenate(r.trace, axis=0)
        assert got.shape == ref.shape
        assert np.array_equal(got, ref), r.rid
        alone.close()
