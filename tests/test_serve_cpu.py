"""The serving loop's host logic (exwave_gb300.serve.Server.run) on the CPU,
with a fake batch in place of the device runtime: FIFO admission under an
HBM budget (waiting while a solve does not fit), retirement at the end
time, receiver samples read once each, latency statistics, requests that
fail admission for a reason of their own rejected while the others are
served, and solves the device reports diverged evicted."""
import numpy as np
import pytest

from exwave_gb300 import _lib, serve


class FakeBatch:
    """Host stand-in of batch.Batch: a solve costs its DoF count in bytes."""

    def __init__(self, budget):
        self.budget, self.used, self.peak = budget, 0, 0
        self.solves, self.next_id, self.admit_order = {}, 0, []
        self.fail_code = None
        self.fail_cells = None     # only solves of this many cells fail
        self.diverge_after = {}    # solve index -> steps after which it diverges

    def add(self, solve):
        if self.fail_code is not None and (self.fail_cells is None or
                                           solve.mesh.n_cells == self.fail_cells):
            raise _lib.EwError(self.fail_code, "injected")
        cost = solve.mesh.n_cells * 4 * (solve.degree + 1) ** 3
        if self.used + cost > self.budget:
            raise _lib.EwError(-4, "over budget")
        sid = self.next_id
        self.next_id += 1
        self.solves[sid] = [solve, 0, cost]
        self.used += cost
        self.peak = max(self.peak, self.used)
        self.admit_order.append(sid)
        return sid

    def remove(self, sid):
        self.used -= self.solves.pop(sid)[2]

    def steps_left(self):
        left = [s.n_steps - d for s, d, _ in self.solves.values() if s.n_steps > d]
        return min(left) if left else 0

    def step(self, n):
        for v in self.solves.values():
            v[1] = min(v[0].n_steps, v[1] + n)

    def synchronize(self):
        pass

    def diverged(self):
        return [sid for sid, (s, d, _) in self.solves.items()
                if sid in self.diverge_after and d >= self.diverge_after[sid]]

    def info(self, sid):
        s, d, _ = self.solves[sid]
        return d, s.n_steps

    def receivers(self, sid, first, count):
        s = self.solves[sid][0]
        return np.arange(first, first + count, dtype=float)[:, None] * np.ones(len(s.receivers))


def _server(budget, steps_per_tick=3):
    srv = serve.Server.__new__(serve.Server)
    srv.batch = FakeBatch(budget)
    srv.steps_per_tick = steps_per_tick
    srv.prepare_threads = 2
    return srv


def test_fifo_admission_under_budget_and_statistics():
    reqs = serve.draw_requests(12, rate=0.0, seed=3, cells=(2, 4), end_time=(0.02, 0.06))
    largest = max(r.dofs() for r in reqs)
    srv = _server(budget=2 * largest)
    stats = srv.run(reqs)
    fb = srv.batch
    assert stats["completed"] == stats["offered"] == 12
    assert stats["backlog_at_end"] == 0 and stats["active_at_end"] == 0
    # admitted in arrival (request id) order, never above the budget
    assert fb.next_id == 12 and fb.peak <= fb.budget
    admitted = sorted(reqs, key=lambda r: r.admitted)
    assert [r.rid for r in admitted] == sorted(r.rid for r in reqs)
    for r in reqs:
        # every step's receiver sample read exactly once, in order
        tr = np.concatenate(r.trace)
        assert tr.shape == (r.n_steps, len(r.receivers))
        assert np.array_equal(tr[:, 0], np.arange(r.n_steps))
        assert r.arrival <= r.admitted <= r.finished
    lat = np.array([r.finished - r.arrival for r in reqs])
    assert stats["latency_p50_s"] == pytest.approx(np.percentile(lat, 50))
    assert stats["latency_p99_s"] == pytest.approx(np.percentile(lat, 99))
    assert stats["peak_active"] >= 1 and stats["ticks"] >= 1


def test_admission_failure_rejects_that_request_only():
    """An admission error of the request's own (not memory) rejects it, with
    the error kept, and the server serves the others."""
    reqs = serve.draw_requests(4, rate=0.0, seed=4, cells=(2, 2), end_time=(0.02, 0.03))
    reqs[1].cells = 3
    srv = _server(budget=1 << 40)
    srv.batch.fail_code = -1
    srv.batch.fail_cells = 27
    stats = srv.run(reqs)
    assert stats["failed"] == 1 and stats["completed"] == 3
    assert "injected" in reqs[1].rejected and reqs[1].finished is None
    assert stats["failures"] == {1: reqs[1].rejected}


def test_diverged_solve_is_evicted():
    """A solve the device marks diverged leaves the batch with an error
    status; the others complete."""
    reqs = serve.draw_requests(3, rate=0.0, seed=8, cells=(2, 2), end_time=(0.05, 0.05))
    srv = _server(budget=1 << 40, steps_per_tick=2)
    srv.batch.diverge_after = {1: 2}
    stats = srv.run(reqs)
    assert stats["completed"] == 2 and stats["failed"] == 1
    assert "diverged" in reqs[1].rejected
    assert 1 not in srv.batch.solves


def test_time_limit_reports_the_backlog():
    # the first request occupies the arena for longer than the time limit;
    # the others wait behind it until the limit ends the run
    reqs = serve.draw_requests(3, rate=0.0, seed=5, cells=(3, 3), end_time=(0.02, 0.02))
    for r in reqs[1:]:
        r.cells = 2
    srv = _server(budget=reqs[0].dofs())
    fb = srv.batch
    fb.step = lambda n: None  # no progress: the first solve never ends
    stats = srv.run(reqs, time_limit=0.05)
    assert stats["completed"] == 0 and stats["backlog_at_end"] == 2
    assert stats["active_at_end"] == 1 and stats["rejected"] == 0
    assert stats["latency_p50_s"] is None


def test_request_larger_than_the_arena_is_rejected():
    """A request that does not fit even into the empty arena is rejected
    (counted, not retried forever) and the others are served; without a time
    limit the run ends."""
    import threading
    reqs = serve.draw_requests(5, rate=0.0, seed=6, cells=(2, 3), end_time=(0.02, 0.05))
    reqs[2].cells = 9
    budget = max(r.dofs() for i, r in enumerate(reqs) if i != 2)
    srv = _server(budget=budget)
    result = {}
    t = threading.Thread(target=lambda: result.update(srv.run(reqs)), daemon=True)
    t.start()
    t.join(timeout=30)
    assert not t.is_alive(), "the serving loop did not end"
    assert result["rejected"] == 1 and result["completed"] == 4
    assert reqs[2].rejected and reqs[2].finished is None
    assert all(r.finished is not None for i, r in enumerate(reqs) if i != 2)


def test_nothing_fits_ends_without_time_limit():
    import threading
    reqs = serve.draw_requests(3, rate=0.0, seed=5, cells=(3, 3), end_time=(0.02, 0.02))
    srv = _server(budget=1)
    result = {}
    t = threading.Thread(target=lambda: result.update(srv.run(reqs)), daemon=True)
    t.start()
    t.join(timeout=30)
    assert not t.is_alive(), "the serving loop did not end"
    assert result["completed"] == 0 and result["rejected"] == 3
