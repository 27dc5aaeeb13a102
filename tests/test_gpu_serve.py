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


def _serve(precision, reqs, **kw):
    from exwave_gb300 import serve
    srv = serve.Server(precision=precision, hbm_budget_bytes=2 << 30, steps_per_tick=3, **kw)
    stats = srv.run(reqs)
    srv.batch.close()
    return stats, {r.rid: np.concatenate(r.trace, axis=0) for r in reqs if r.trace}


def test_receiver_traces_against_fp64():
    """The serving configuration's criterion: the same seeded requests served
    in FP64, mixed and compensated precision; each solve's receiver trace
    against its FP64 trace, relative to the FP64 trace's largest value.  The
    compensated operator stays within 1e-10; the mixed one (FP32 operator)
    is recorded against the 1e-6 target and held to 1e-4."""
    from exwave_gb300 import build, serve
    build.build()
    mk = lambda: serve.draw_requests(6, rate=500.0, seed=5, degrees=(3, 4), cells=(3, 4),
                                     end_time=(0.05, 0.1), n_receivers=4)
    s64, t64 = _serve("fp64", mk())
    sff, tff = _serve("mixed_ff", mk())
    smx, tmx = _serve("mixed", mk())
    assert s64["completed"] == sff["completed"] == smx["completed"] == 6
    err = {}
    for name, tr in (("mixed_ff", tff), ("mixed", tmx)):
        err[name] = max(np.abs(tr[i] - t64[i]).max() / np.abs(t64[i]).max() for i in t64)
    print("receiver traces vs FP64: compensated %.3e, mixed %.3e" % (err["mixed_ff"], err["mixed"]))
    assert err["mixed_ff"] < 1e-10
    assert err["mixed"] < 1e-4


def test_diverging_solve_is_evicted():
    """A solve stepped with an unstable time step (ten times the CFL bound)
    is marked diverged by the device once a receiver sample passes the
    blow-up limit; the server evicts it and the stable solve next to it
    completes with the same trace as alone."""
    from exwave_gb300 import build, serve
    from exwave_gb300.batch import Batch
    build.build()
    reqs = serve.draw_requests(2, rate=0.0, seed=9, degrees=(3, 3), cells=(4, 4),
                               end_time=(0.6, 0.6), n_receivers=4)
    bad = reqs[1]
    solve = bad.make_solve()
    solve.dt *= 10.0
    bad.n_steps = solve.n_steps = max(1, int(np.ceil(bad.end_time / solve.dt)))
    stats, traces = _serve("mixed", reqs, blowup_limit=1e3)
    assert stats["completed"] == 1 and stats["failed"] == 1
    assert "diverged" in bad.rejected
    alone = Batch(precision="mixed", hbm_budget_bytes=1 << 30)
    sid = alone.add(reqs[0].make_solve())
    alone.step(reqs[0].n_steps)
    alone.synchronize()
    assert np.array_equal(traces[0], alone.receivers(sid))
    alone.close()
