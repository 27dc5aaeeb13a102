"""Serving loop with continuous batching.

Requests (a solve: degree, mesh, material, source, receivers, end time)
arrive over time; they wait in a FIFO queue until the device arena can hold
them (admission by HBM budget), then join the resident batch.  Every tick
advances all admitted solves by a few LSRK45 steps in one batched launch
sequence, streams the new receiver samples to the host and retires the
solves that reached their end time.  Solves that arrive while others run
are admitted as soon as memory frees up, so their work overlaps on the
device.  Latency = completion time - arrival time.
"""
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from . import mesh as mesh_mod
from .batch import Batch, Solve


@dataclass
class Request:
    rid: int
    arrival: float
    degree: int
    cells: int
    speed: float
    density: float
    f0: float
    source_pos: tuple
    receivers: np.ndarray
    end_time: float
    dt: float = 0.0
    n_steps: int = 0
    admitted: float = None
    finished: float = None
    trace: list = field(default_factory=list)
    samples_read: int = 0
    rejected: str = None
    solve: object = None

    def make_solve(self):
        """The request's Solve (mesh and tables), built once and kept."""
        if self.solve is None:
            m = mesh_mod.hypercube(3, self.cells, speed=self.speed, density=self.density)
            h = 1.0 / self.cells
            self.dt = 0.25 * h / (self.speed * self.degree ** 1.5)
            self.n_steps = max(1, int(np.ceil(self.end_time / self.dt - 1e-12)))
            self.solve = Solve(m, self.degree, self.dt, self.n_steps,
                               source=(list(self.source_pos), self.f0, 1.0 / self.f0, 1.0),
                               receivers=self.receivers)
        return self.solve

    def dofs(self):
        return self.cells ** 3 * 4 * (self.degree + 1) ** 3


def draw_requests(n, rate, seed, degrees=(3, 7), cells=(8, 32), speed=(1.0, 4.0),
                  density=(1.0, 3.0), f0=(2.0, 8.0), end_time=(0.2, 2.0), n_receivers=8):
    """Seeded request stream: Poisson arrivals at `rate` per second and the
    per-instance distribution of the batched configuration (degree uniform in
    {3..7}, n^3 cells with n uniform in [8, 32], c ~ U[1,4], rho ~ U[1,3],
    Ricker source f0 ~ U[2,8] at an interior point, 8 receivers)."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, n)) if rate > 0 else np.zeros(n)
    reqs = []
    for i in range(n):
        reqs.append(Request(
            rid=i, arrival=float(t[i]),
            degree=int(rng.integers(degrees[0], degrees[1] + 1)),
            cells=int(rng.integers(cells[0], cells[1] + 1)),
            speed=float(rng.uniform(*speed)), density=float(rng.uniform(*density)),
            f0=float(rng.uniform(*f0)),
            source_pos=tuple(rng.uniform(0.2, 0.8, 3)),
            receivers=rng.uniform(0.1, 0.9, (n_receivers, 3)),
            end_time=float(rng.uniform(*end_time))))
    return reqs


class Server:
    """Continuous-batching request loop over one Batch.

    Every tick advances all resident solves by `steps_per_tick` LSRK45 steps
    (the batch allows overrun: a solve that reaches its end inside a tick
    computes the tick's remaining steps without recording them, instead of
    cutting the tick short for everyone).  While the device runs a tick, a
    worker thread builds the meshes and tables of the requests that wait
    for admission.  After each tick the loop evicts the solves the device
    marked diverged (a receiver sample that is not finite or exceeds
    `blowup_limit`), reads the new receiver samples and retires the solves
    that reached their end.  A request whose admission fails for another
    reason than memory (an error of its own) is rejected, with the error
    kept on the request, and the loop goes on."""

    def __init__(self, precision="mixed", hbm_budget_bytes=150 << 30, steps_per_tick=4,
                 max_solves=4096, device=0, blowup_limit=1e8, prepare_threads=2):
        self.batch = Batch(precision=precision, hbm_budget_bytes=hbm_budget_bytes,
                           max_solves=max_solves, device=device, allow_overrun=True,
                           blowup_limit=blowup_limit)
        self.steps_per_tick = steps_per_tick
        self.prepare_threads = prepare_threads

    def run(self, requests, time_limit=None, log=None):
        """Serve `requests` in real time; returns a statistics dict."""
        import concurrent.futures as cf
        b = self.batch
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        queue = deque()
        active = {}
        done, rejected, failed = [], [], []
        prep = {}
        pool = cf.ThreadPoolExecutor(max_workers=max(1, self.prepare_threads)) \
            if self.prepare_threads > 0 else None
        t0 = time.perf_counter()
        dof_updates = 0
        ticks = 0
        peak_active = 0
        prep_wait = 0.0

        def prepared(r):
            # the request's Solve: from the worker thread if it was started there
            f = prep.pop(r.rid, None)
            return f.result() if f is not None else r.make_solve()

        def reject(r, err, into):
            r.rejected = err
            r.solve = None
            into.append(r)

        try:
            while pending or queue or active:
                now = time.perf_counter() - t0
                if time_limit is not None and now >= time_limit:
                    break
                while pending and pending[0].arrival <= now:
                    r = pending.popleft()
                    queue.append(r)
                    if pool is not None:
                        prep[r.rid] = pool.submit(r.make_solve)
                while queue:
                    r = queue[0]
                    tw = time.perf_counter()
                    try:
                        solve = prepared(r)
                    except Exception as e:  # a request that cannot even be built
                        reject(queue.popleft(), "preparation failed: %s" % e, failed)
                        continue
                    prep_wait += time.perf_counter() - tw
                    try:
                        sid = b.add(solve)
                    except _lib.EwError as e:
                        if e.code in (-4, -6) and active:   # over the HBM budget / slot limit: wait
                            break
                        if e.code in (-4, -6):
                            # does not fit even with no solve resident: it never will
                            reject(queue.popleft(), str(e), rejected)
                        else:
                            # an error of this request (invalid mesh, source, ...)
                            reject(queue.popleft(), str(e), failed)
                        continue
                    r.admitted = time.perf_counter() - t0
                    active[sid] = r
                    queue.popleft()
                peak_active = max(peak_active, len(active))
                if not active:
                    if pending:
                        time.sleep(max(0.0, min(0.01, pending[0].arrival - now)))
                    continue
                k = self.steps_per_tick
                b.step(k)
                # the device runs the tick; the worker threads build waiting requests
                for r in queue:
                    if pool is not None and r.rid not in prep and r.solve is None:
                        prep[r.rid] = pool.submit(r.make_solve)
                for sid in b.diverged():
                    r = active.pop(sid, None)
                    if r is not None:
                        r.finished = time.perf_counter() - t0
                        b.remove(sid)
                        reject(r, "diverged: a receiver sample is not finite or exceeds the "
                                  "blow-up limit", failed)
                b.synchronize()
                ticks += 1
                dof_updates += 5 * k * sum(r.dofs() for r in active.values())
                for sid in list(active):
                    r = active[sid]
                    steps, total = b.info(sid)
                    if steps > r.samples_read:
                        r.trace.append(b.receivers(sid, r.samples_read, steps - r.samples_read))
                        r.samples_read = steps
                    if steps >= total:
                        r.finished = time.perf_counter() - t0
                        r.solve = None  # the host copy of the mesh is no longer needed
                        b.remove(sid)
                        del active[sid]
                        done.append(r)
                        if log:
                            log(r)
        finally:
            if pool is not None:
                pool.shutdown(wait=True, cancel_futures=True)
        wall = time.perf_counter() - t0
        lat = np.array([r.finished - r.arrival for r in done]) if done else np.array([])
        wait = np.array([r.admitted - r.arrival for r in done]) if done else np.array([])
        return {
            "completed": len(done), "offered": len(requests), "rejected": len(rejected),
            "failed": len(failed), "wall_s": wall,
            "solves_per_s": len(done) / wall if wall > 0 else 0.0,
            "latency_p50_s": float(np.percentile(lat, 50)) if len(lat) else None,
            "latency_p99_s": float(np.percentile(lat, 99)) if len(lat) else None,
            "admission_wait_p50_s": float(np.percentile(wait, 50)) if len(wait) else None,
            # arrived but not yet admitted / not yet arrived when the run stopped
            "backlog_at_end": len(queue), "not_arrived_at_end": len(pending),
            "active_at_end": len(active),
            "peak_active": peak_active, "ticks": ticks,
            "host_wait_for_preparation_s": prep_wait,
            "dof_updates_per_s": dof_updates / wall if wall > 0 else 0.0,
            "failures": {r.rid: r.rejected for r in failed},
        }
