"""Benchmark of the DG wave-operator hot path (one JSON line on rank 0).

Workload (default): 3-D vibrating membrane on [0,1]^3, 64^3 affine hexes,
FE_DGQ degree 5 (216 Gauss points x 4 fields per cell = 226,492,416 DoFs),
modes (1,1,1) amplitude 1 and (2,1,3) amplitude 0.5, c = rho = 1, hard walls,
LSRK4(5) with dt = 0.25 h / k^1.5.  One "step" = one LSRK45 time step
(five fused operator + stage-update launches) over the whole mesh.

metric: DoF-updates/s = n_dofs x 5 stages / s (whole job, all ranks).
 - value: device time with the state resident in HBM (CUDA events around
   exactly K steps after W warm-up steps; the state, 1.8 GB, is larger than
   L2, so no flush is needed).
 - fp64: the same workload on the plain FP64 operator; errors: L2 errors of
   both paths against the analytic solution after the timed steps.
 - e2e: the same step through the public C ABI with the state in pinned host
   memory: host->device copy, step, device->host copy, every step.
 - roofline: achieved HBM bandwidth of the stage kernel = algorithmic bytes
   per step (112 B/DoF mixed, 144 B/DoF FP64) / device time per step.
 - cpu_baseline: the CPU restatement for axis-aligned cells (line form, FP64,
   OpenMP, all host threads) on the same 64^3 workload, whole steps for about
   8 s.

--impl reference: the CPU implementation of the path on the host cores
(the reference itself cannot be built: it needs deal.II, p4est and MPI), on
the same metric and the same 64^3 workload; rank 0 only.
Multi-GPU (torchrun): independent replicas, one solve per rank (the path
does not shard), max time over ranks.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

STAGES = 5
# what each precision stores and computes in
DTYPES = {
    "mixed": "f32-operator/f32-stage-input/float-pair-state-in-multi-step-calls/f64-state-at-call-boundary",
    "mixed_ff": "ff-operator(~44-bit)/float-pair-stage-input/float-pair-state-in-multi-step-calls/f64-state-at-call-boundary",
    "fp64": "f64",
}
# algorithmic bytes per DoF and LSRK45 step: each vector once per stage at
# its stored precision (mixed: FP32 stage inputs; compensated: float pairs)
BYTES_PER_DOF_STEP = {"mixed": 112.0, "mixed_ff": 144.0, "fp64": 144.0}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cells", type=int, default=64)
    ap.add_argument("--degree", type=int, default=5)
    ap.add_argument("--precision", default="auto", choices=["auto", "mixed", "mixed_ff", "fp64"],
                    help="auto (membrane3d): time all three and report the fastest at matched L2 "
                         "error; mixed: FP32 operator; mixed_ff: compensated (float-float) operator")
    ap.add_argument("--cells-per-block", type=int, default=0,
                    help="cells per thread block of the operator kernel (0: tuned value)")
    ap.add_argument("--nb-staging", type=int, default=0,
                    help="line kernel's neighbour layout: 0 tuned, 1 per-thread lines, 2 bulk arrays")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 comparison run")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default="membrane3d",
                    choices=["membrane3d", "membrane2d", "ader3d", "batch", "serve", "sweep"],
                    help="membrane3d (default headline), membrane2d (2-D 16^2 k=4 to T=1), ader3d "
                         "(curved two-layer ADER), batch (512 independent solves), serve "
                         "(continuous batching), sweep (degrees)")
    ap.add_argument("--solves", type=int, default=512)
    ap.add_argument("--rates", default="0.5,2,50", help="serve: offered Poisson rates (solves/s)")
    ap.add_argument("--trace-sample", type=int, default=6,
                    help="serve: completed solves replayed on the FP64 path per run")
    ap.add_argument("--time-limit", type=float, default=60.0)
    ap.add_argument("--degrees", default="3,7", help="batch: degree range (inclusive)")
    ap.add_argument("--sizes", default="8,32", help="batch: cells per direction range (inclusive)")
    ap.add_argument("--sweep-degrees", default="2,12", help="sweep: degree range (inclusive)")
    ap.add_argument("--quick", action="store_true",
                    help="ader3d: timing only, without the run to T=0.5 on the three paths")
    return ap.parse_args()


def dist_info():
    from exwave_gb300.replicas import dist_info as di
    return di()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    def __init__(self, index):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = sorted(float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit())
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if s[3 + i].lower() == "active"})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.samples)}


def build_problem(cells, degree):
    import exwave_gb300 as ew
    m = ew.hypercube(3, cells, 0, 0.0, boundary_ids=2)
    dt = ew.time_step_size(m, 0.25 / degree ** 1.5)
    return m, dt


MODES = ([1.0, 0.5], [[1, 1, 1], [2, 1, 3]])


def time_steps(op, dt, steps, warmup, torch, barrier):
    """Device time of exactly `steps` LSRK45 steps after `warmup` steps."""
    u = op.project_membrane(*MODES, 0.0)
    v = torch.zeros_like(u)
    stream = torch.cuda.current_stream()
    op.set_stream(stream)
    # the public multi-step call (the reference's time loop over
    # perform_time_step): warm-up steps, then exactly `steps` timed steps
    op.lsrk45_steps(dt, warmup, u, v)
    u, v = v, u
    torch.cuda.synchronize()
    barrier()
    l0 = op.kernel_launches()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    op.lsrk45_steps(dt, steps, u, v)
    u, v = v, u
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier()
    ms = ev0.elapsed_time(ev1)
    launches = op.kernel_launches() - l0
    op.synchronize()  # raises if a kernel raised its device error flag
    t_end = (warmup + steps) * dt
    errs = op.l2_errors(u, *MODES, t_end)
    return ms, launches, errs, u


def e2e_steps(op, dt, steps, warmup, torch):
    """Same step through the public API with the state in pinned host
    memory, the reference integrator's storage: every step copies the whole
    state host -> device, runs the LSRK45 step and copies the new state
    device -> host (ew_lsrk45_step_host; the copies run in chunks, and one
    step's copy back overlaps the next step's copy in)."""
    n = op.n_dofs
    host = torch.empty(n, dtype=torch.float64, pin_memory=True)
    host.copy_(op.project_membrane(*MODES, 0.0).cpu())
    stream = torch.cuda.current_stream()
    op.set_stream(stream)
    for _ in range(warmup):
        op.lsrk45_step_host(dt, host, host)
    op.synchronize()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(steps):
        op.lsrk45_step_host(dt, host, host)
    # the end event after the last step's copy to the host
    op.wait_host_copies()
    ev1.record(stream)
    torch.cuda.synchronize()
    op.synchronize()
    return ev0.elapsed_time(ev1), n * 8, n * 8


def cpu_problem(cells, degree):
    """The headline workload on the CPU: the oracle's mesh and initial field,
    stepped by the CPU baseline for axis-aligned cells (oracle/ew_cpu_cart.cpp:
    the same operator and LSRK45 step in line form, FP64, OpenMP over all
    host threads)."""
    import numpy as np
    from oracle import oracle
    oracle.build()
    prob = oracle.Problem.hypercube(3, degree, cells, 0, 0.0, 2)
    n = prob.n_cells
    cpu = oracle.CartCPU(3, degree, prob.vertices(), prob.neighbors(), np.ones(n), np.ones(n))
    dt = prob.time_step(0.25 / degree ** 1.5)
    u = prob.project_modes(*MODES)
    return oracle, prob, cpu, dt, u


def cpu_sample(degree, cells=64, min_seconds=8.0):
    """The CPU baseline on the headline workload itself (64^3 cells), timed
    over whole steps until at least min_seconds have passed."""
    import numpy as np
    oracle, prob, cpu, dt, u = cpu_problem(cells, degree)
    v = np.zeros_like(u)
    cpu.lsrk45_step(dt, u, v)  # warm-up (first touch of the pages)
    u, v = v, u
    steps = 0
    t0 = time.perf_counter()
    while True:
        cpu.lsrk45_step(dt, u, v)
        u, v = v, u
        steps += 1
        el = time.perf_counter() - t0
        if el >= min_seconds:
            break
    rate = prob.n_dofs * STAGES * steps / el
    return {"value": rate, "unit": "DoF-updates/s", "cores": oracle.num_threads(), "kind": "port",
            "sample": "3-D k=%d, %d^3 affine cells (%d DoFs, the headline workload), %d LSRK45 "
                      "steps of the CPU restatement for axis-aligned cells (line form, FP64, "
                      "OpenMP)" % (degree, cells, prob.n_dofs, steps)}


def traffic_from_profiles(precision, n_dofs):
    """DRAM bytes per stage launch (average over the five stages of a
    steady-state step) from the committed ncu summary, scaled to this
    workload's DoF count (traffic grows in proportion to the cells)."""
    path = os.path.join(ROOT, "profiles", "stage_kernel_traffic.json")
    try:
        with open(path) as f:
            d = json.load(f)
        e = d[precision]
        return e["dram_bytes_per_dof_launch"] * n_dofs
    except (OSError, KeyError, ValueError):
        return None


def run_reference(args):
    ws, rank, _ = dist_info()
    if rank != 0:
        return
    import numpy as np
    oracle, prob, cpu, dt, u = cpu_problem(args.cells, args.degree)
    v = np.zeros_like(u)
    for _ in range(args.warmup):
        cpu.lsrk45_step(dt, u, v)
        u, v = v, u
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cpu.lsrk45_step(dt, u, v)
        u, v = v, u
    el = time.perf_counter() - t0
    value = prob.n_dofs * STAGES * args.steps / el
    sample = ("3-D k=%d, %d^3 affine cells (%d DoFs), %d timed steps after %d warm-up steps; "
              "the reference (deal.II MatrixFree) cannot be built on this image: its arithmetic "
              "restated for axis-aligned cells in line form (FP64, OpenMP over all host threads) "
              "is timed" % (args.degree, args.cells, prob.n_dofs, args.steps, args.warmup))
    line = {
        "impl": "reference", "metric": "DoF-updates/s", "value": value, "unit": "DoF-updates/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": el / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "3-D vibrating membrane, %d^3 affine hexes, FE_DGQ(%d), LSRK45"
                               % (args.cells, args.degree), "precision": "fp64",
                   "n_dofs": prob.n_dofs},
        "cpu_baseline": {"value": value, "unit": "DoF-updates/s", "cores": oracle.num_threads(),
                         "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "DoF-updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def ader3d(args, torch):
    """ADER of order k+1, 3-D k=4, 40^3 hexes on the curved mesh x_i += 0.03
    prod_d sin(2 pi x_d), two layers split at z = 0.5 (c=1, rho=1 below; c=3,
    rho=2 above), Gaussian pulse (width 0.05) at a seeded point of the lower
    layer, p = 0 on the top face, rigid walls elsewhere; CFL 0.15.  (CFL
    0.2, the value of the reference's 3-D ADER test, is unstable on this
    curved mesh from 24^3 cells on: the oracle, the reference algorithm on
    the CPU, grows exactly like the GPU path from a random state.)"""
    import numpy as np
    import exwave_gb300 as ew
    k, n = 4, (args.cells if args.cells != 64 else 40)
    m = ew.hypercube(3, n, 0, 0.03, transform="sine_all", boundary_ids=[1, 1, 1, 1, 1, 2])
    ew.layered_materials(m, 0.5, below=(1.0, 1.0), above=(3.0, 2.0))
    rng = np.random.default_rng(2024)
    x0 = [rng.uniform(0.2, 0.8), rng.uniform(0.2, 0.8), rng.uniform(0.15, 0.35)]
    cfl = 0.15
    dt = ew.time_step_size(m, cfl / k ** 1.5)
    out = {}
    states = {}
    for prec in ("mixed", "fp64", "mixed_ff"):
        op = ew.WaveEquationOperation(m, k, precision=prec)
        u = op.project_gaussian(x0, 0.05)
        v = torch.zeros_like(u)
        steps = args.steps if prec == "mixed" else max(2, args.steps // 4)
        for _ in range(args.warmup):
            op.ader_step(dt, u, v)
            u, v = v, u
        stream = torch.cuda.current_stream()
        op.set_stream(stream)
        l0 = op.kernel_launches()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(steps):
            op.ader_step(dt, u, v)
            u, v = v, u
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        out[prec] = {"value": op.n_dofs * steps / (ms / 1e3), "ms_per_step": ms / steps,
                     "gpu_launches": op.kernel_launches() - l0}
        op.synchronize()
        states[prec] = (op, u, steps)
    if args.quick:
        return {"metric": "DoF-updates/s (ADER: 1 per DoF and step)", "value": out["mixed"]["value"],
                "unit": "DoF-updates/s", "ms_per_step": out["mixed"]["ms_per_step"],
                "fp64": out["fp64"], "compensated": out["mixed_ff"],
                "gpu_launches": out["mixed"]["gpu_launches"],
                "config": {"workload": "ADER k=4 3-D %d^3 curved two-layer Gaussian pulse" % n,
                           "dt": dt, "cfl": cfl, "x0": x0}}
    # the configuration's run to T = 0.5 on both paths, with 8 seeded
    # receivers sampled every step: final-state and receiver-trace errors of
    # the mixed path against FP64
    rec = np.random.default_rng(2025).uniform(0.1, 0.9, (8, 3))
    t_end = 0.5
    n_steps = int(np.ceil(t_end / dt - 1e-12))
    finals, traces, run_ms = {}, {}, {}
    for prec in ("mixed", "fp64", "mixed_ff"):
        op = ew.WaveEquationOperation(m, k, precision=prec)
        stream = torch.cuda.current_stream()
        op.set_stream(stream)
        op.set_receivers(rec)
        u = op.project_gaussian(x0, 0.05)
        v = torch.zeros_like(u)
        trace = torch.zeros(n_steps + 1, 8 * 4, dtype=torch.float64, device="cuda")
        op.sample_receivers(u, trace[0])
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for s in range(n_steps):
            op.ader_step(dt, u, v)
            u, v = v, u
            op.sample_receivers(u, trace[s + 1])
        e1.record(stream)
        op.synchronize()
        run_ms[prec] = e0.elapsed_time(e1)
        finals[prec] = (op, u)
        traces[prec] = trace.view(n_steps + 1, 8, 4)[:, :, 3].cpu().numpy()
    op64, u64 = finals["fp64"]
    diff = op64.l2_difference(finals["mixed"][1], u64)
    ref = op64.l2_difference(u64, torch.zeros_like(u64))
    tr_err = float(np.abs(traces["mixed"] - traces["fp64"]).max() / np.abs(traces["fp64"]).max())
    diff_ff = op64.l2_difference(finals["mixed_ff"][1], u64)
    tr_err_ff = float(np.abs(traces["mixed_ff"] - traces["fp64"]).max() / np.abs(traces["fp64"]).max())
    return {"metric": "DoF-updates/s (ADER: 1 per DoF and step)", "value": out["mixed"]["value"],
            "unit": "DoF-updates/s", "ms_per_step": out["mixed"]["ms_per_step"],
            "fp64": out["fp64"], "compensated": out["mixed_ff"],
            "gpu_launches": out["mixed"]["gpu_launches"],
            "run_to_T": {"t_end": n_steps * dt, "steps": n_steps, "mixed_ms": run_ms["mixed"],
                         "fp64_ms": run_ms["fp64"], "compensated_ms": run_ms["mixed_ff"],
                         "compensated_vs_fp64_rel_l2_p": diff_ff[0] / ref[0],
                         "compensated_receiver_trace_rel_err_p": tr_err_ff,
                         "mixed_vs_fp64_rel_l2_p": diff[0] / ref[0],
                         "mixed_vs_fp64_rel_l2_u": diff[1] / max(ref[1], 1e-300),
                         "receiver_trace_rel_err_p": tr_err, "receivers": rec.tolist()},
            "config": {"workload": "ADER k=4 3-D 40^3 curved two-layer Gaussian pulse",
                       "n_dofs": op64.n_dofs, "dt": dt, "cfl": cfl, "x0": x0}}


def membrane2d(args, torch):
    """2-D vibrating membrane, 16^2 affine quads, FE_DGQ(4), modes (1,1) +
    0.5 (2,3), p = 0 on the boundary, LSRK45 with dt = 2^-9, 512 steps to
    T = 1, FP64, mixed and compensated: time of the whole run (one
    ew_lsrk45_steps call) and L2 errors against the analytic solution."""
    import exwave_gb300 as ew
    amps, kvecs = [1.0, 0.5], [[1, 1], [2, 3]]
    m = ew.hypercube(2, 16, 0, 0.0, boundary_ids=2)
    dt = ew.time_step_size(m, 0.25 / 4 ** 1.5)
    steps = int(round(1.0 / dt))
    out, states = {}, {}
    for prec in ("mixed", "fp64", "mixed_ff"):
        op = ew.WaveEquationOperation(m, 4, precision=prec)
        stream = torch.cuda.current_stream()
        op.set_stream(stream)
        u0 = op.project_membrane(amps, kvecs, 0.0)
        u, v = u0.clone(), torch.zeros_like(u0)
        op.lsrk45_steps(dt, args.warmup, u, v)  # warm-up (discarded)
        u, v = u0.clone(), torch.zeros_like(u0)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        op.lsrk45_steps(dt, steps, u, v)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        err = op.l2_errors(v, amps, kvecs, steps * dt)
        out[prec] = {"value": op.n_dofs * STAGES * steps / (ms / 1e3), "ms_total": ms,
                     "l2_p": err[0], "l2_u": err[1], "norm_p": err[2]}
        states[prec] = (op, v)
    op64, v64 = states["fp64"]
    diff = op64.l2_difference(states["mixed"][1], v64)
    diffc = op64.l2_difference(states["mixed_ff"][1], v64)
    return {"metric": "DoF-updates/s", "value": out["mixed"]["value"], "unit": "DoF-updates/s",
            "mixed": out["mixed"], "fp64": out["fp64"], "compensated": out["mixed_ff"],
            "error_ratio_p": out["mixed"]["l2_p"] / out["fp64"]["l2_p"],
            "error_ratio_u": out["mixed"]["l2_u"] / out["fp64"]["l2_u"],
            "compensated_error_ratio_p": out["mixed_ff"]["l2_p"] / out["fp64"]["l2_p"],
            "compensated_error_ratio_u": out["mixed_ff"]["l2_u"] / out["fp64"]["l2_u"],
            "mixed_vs_fp64_l2": {"p": diff[0], "u": diff[1]},
            "compensated_vs_fp64_l2": {"p": diffc[0], "u": diffc[1]},
            "config": {"workload": "2-D vibrating membrane, 16^2 affine quads, FE_DGQ(4), LSRK45, "
                                   "512 steps to T=1", "n_dofs": op64.n_dofs, "dt": dt,
                       "steps": steps, "note": "launch-bound at this size (19,200 DoFs)"}}


def batch_workload(args, torch):
    """Batch of independent 3-D solves drawn from a seed (degree uniform in
    {3..7}, n^3 cells n in [8,32], c ~ U[1,4], rho ~ U[1,3], Ricker source
    f0 ~ U[2,8], 8 receivers), all resident; K batch steps timed (every solve
    advances one LSRK45 step per batch step); compared with running a sample
    of the same solves one after another."""
    import numpy as np
    from exwave_gb300 import serve
    from exwave_gb300.batch import Batch
    dg = tuple(int(x) for x in args.degrees.split(","))
    sz = tuple(int(x) for x in args.sizes.split(","))
    reqs = serve.draw_requests(args.solves, rate=0.0, seed=7, end_time=(1.0, 1.0), degrees=dg, cells=sz)
    solves = [r.make_solve() for r in reqs]
    free, total = torch.cuda.mem_get_info()
    b = Batch(precision=args.precision, hbm_budget_bytes=int(free * 0.85), max_solves=len(solves) + 8)
    for s in solves:
        b.add(s)
    dofs = sum(r.dofs() for r in reqs)
    stream = torch.cuda.Stream()  # a real stream: the batch replays its graphs on it
    b.set_stream(stream)
    b.step(args.warmup)
    b.synchronize()
    l0 = b.kernel_launches()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    b.step(args.steps)
    e1.record(stream)
    b.synchronize()
    ms = e0.elapsed_time(e1)
    batched = dofs * 5 * args.steps / (ms / 1e3)
    launches = b.kernel_launches() - l0
    b.close()
    # sequential: a seeded sample of the same solves, each alone
    rng = np.random.default_rng(1)
    idx = rng.choice(len(solves), size=min(16, len(solves)), replace=False)
    seq_t, seq_d = 0.0, 0
    for i in idx:
        one = Batch(precision=args.precision, hbm_budget_bytes=4 << 30, max_solves=2)
        one.add(solves[i])
        one.set_stream(stream)
        one.step(1)
        one.synchronize()
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        one.step(args.steps)
        f1.record(stream)
        one.synchronize()
        seq_t += f0.elapsed_time(f1) / 1e3
        seq_d += reqs[i].dofs() * 5 * args.steps
        one.close()
    sequential = seq_d / seq_t
    with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
        peak = float(json.load(f)["hbm_gbs"])
    # algorithmic bytes of a step (each vector once per stage at its stored
    # precision) over the step time, all groups together
    achieved = BYTES_PER_DOF_STEP[args.precision] * dofs / (ms / args.steps / 1e3) / 1e9
    return {"metric": "DoF-updates/s (aggregate)", "value": batched, "unit": "DoF-updates/s",
            "ms_per_step": ms / args.steps, "gpu_launches": int(launches),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": "measured",
                         "kernel": "stage_cart_kernel (one launch per degree group and stage)"},
            "sequential_value": sequential, "batched_over_sequential": batched / sequential,
            "config": {"workload": "batch of %d 3-D solves (k %d..%d, n %d..%d, Ricker, 8 receivers)"
                                   % ((len(solves),) + dg + sz), "total_dofs": dofs, "precision": args.precision,
                       "sequential_sample": len(idx)}}


def serve_workload(args, torch):
    """Serving (continuous batching) at each offered Poisson rate of --rates,
    for the FP32-operator and the compensated precision (or the one given by
    --precision): solves/s, latency p50 / p99 and the backlog over a run of
    --time-limit seconds per rate.  Then the configuration's accuracy
    criterion: the --trace-sample cheapest completed solves of each run are
    replayed alone on the FP64 path, and their receiver traces compared
    (largest difference over the FP64 trace's largest value)."""
    import numpy as np
    from exwave_gb300 import serve
    from exwave_gb300.batch import Batch
    rates = [float(x) for x in args.rates.split(",")]
    precs = ["mixed", "mixed_ff"] if args.precision == "auto" else [args.precision]
    n_req = args.solves if args.solves != 512 else 20000
    runs = []
    for prec in precs:
        for rate in rates:
            reqs = serve.draw_requests(n_req, rate=rate, seed=11)
            srv = serve.Server(precision=prec, hbm_budget_bytes=150 << 30, steps_per_tick=4)
            stats = srv.run(reqs, time_limit=args.time_limit)
            srv.batch.close()
            done = [r for r in reqs if r.finished is not None and r.rejected is None]
            sample = sorted(done, key=lambda r: r.dofs() * r.n_steps)[:args.trace_sample]
            errs = []
            if sample:
                ref = Batch(precision="fp64", hbm_budget_bytes=16 << 30, allow_overrun=True)
                ids = [ref.add(r.make_solve()) for r in sample]
                ref.step(max(r.n_steps for r in sample))
                ref.synchronize()
                for r, sid in zip(sample, ids):
                    t64 = ref.receivers(sid)
                    got = np.concatenate(r.trace, axis=0)
                    errs.append(float(np.abs(got - t64).max() / max(np.abs(t64).max(), 1e-300)))
                ref.close()
            stats.pop("failures", None)
            runs.append({"precision": prec, "offered_rate_per_s": rate, "stats": stats,
                         "trace_rel_err_vs_fp64": max(errs) if errs else None,
                         "trace_rel_err_vs_fp64_median": float(np.median(errs)) if errs else None,
                         "trace_sample": len(errs),
                         "meets_1e-6": bool(errs and max(errs) <= 1e-6)})
    head = runs[0]
    return {"metric": "solves/s", "value": head["stats"]["solves_per_s"], "unit": "solves/s",
            "latency_p50_s": head["stats"]["latency_p50_s"],
            "latency_p99_s": head["stats"]["latency_p99_s"], "runs": runs,
            "config": {"workload": "serving, Poisson arrivals, T ~ U[0.2,2], 150 GB budget, "
                                   "%d requests per run, %g s per rate" % (n_req, args.time_limit),
                       "rates_per_s": rates, "precisions": precs}}


def sweep_workload(args, torch):
    import exwave_gb300 as ew
    rows = []
    degs = ((2, 128), (3, 96), (4, 77), (5, 64), (6, 55), (7, 48), (8, 42), (9, 38), (10, 35),
            (11, 32), (12, 29))
    lo, hi = (int(x) for x in args.sweep_degrees.split(","))
    for k, n in degs:
        if not lo <= k <= hi:
            continue
        m, dt = build_problem(n, k)
        row = {"degree": k, "cells": n}
        for prec in ("mixed", "fp64", "mixed_ff"):
            op = ew.WaveEquationOperation(m, k, precision=prec)
            steps = args.steps if prec == "mixed" else max(2, args.steps // 4)
            ms, _, errs, _ = time_steps(op, dt, steps, min(args.warmup, 3), torch, lambda: None)
            row[prec] = {"value": op.n_dofs * STAGES * steps / (ms / 1e3),
                         "ms_per_step": ms / steps, "l2_p": errs[0],
                         "gbs": BYTES_PER_DOF_STEP[prec] * op.n_dofs / (ms / steps / 1e3) / 1e9}
            row["n_dofs"] = op.n_dofs
            op.close()
        row["compensated_over_fp64"] = row["mixed_ff"]["value"] / row["fp64"]["value"]
        rows.append(row)
    return {"metric": "DoF-updates/s per degree", "rows": rows,
            "config": {"workload": "3-D membrane degree sweep at ~226M DoFs (the line kernel up "
                                   "to k = 7, the generic kernel with several points per thread "
                                   "from k = 8)"}}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.workload != "membrane3d":
        if args.precision == "auto" and args.workload != "serve":
            # batches: the FP32 operator (the configuration's mixed precision);
            # serving compares the precisions itself
            args.precision = "mixed"
        import torch
        if dist_info()[1] != 0:
            return  # the other workloads are single-GPU cases: rank 0 runs them
        from exwave_gb300 import build
        build.build()
        fn = {"ader3d": ader3d, "batch": batch_workload, "serve": serve_workload,
              "sweep": sweep_workload, "membrane2d": membrane2d}[args.workload]
        with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
            res = fn(args, torch)
        res["clocks"] = clk.summary()
        res["n_gpus"] = 1
        print(json.dumps(res), flush=True)
        return
    import torch
    from exwave_gb300.replicas import Replicas
    rep = Replicas("nccl")
    ws, rank, local = rep.world_size, rep.rank, rep.local_rank
    barrier = rep.barrier
    import exwave_gb300 as ew
    from exwave_gb300 import build
    build.build()
    import numpy as np
    with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
        peaks = json.load(f)
    peak, peak_kind = float(peaks["hbm_gbs"]), "measured"
    m, dt = build_problem(args.cells, args.degree)
    # Every precision runs the same W + K steps (the same final time), so
    # their L2 errors against the analytic solution compare directly; the
    # headline is the fastest precision whose errors are within 1.1x the
    # FP64 path's (the metric's "at equal L2 error").
    order = [args.precision] if args.precision != "auto" else ["mixed", "mixed_ff", "fp64"]
    if args.precision != "auto" and not args.no_fp64 and "fp64" not in order:
        order.append("fp64")
    runs, ops = {}, {}
    with ClockSampler(local) as clk:
        for prec in order:
            o = ew.WaveEquationOperation(m, args.degree, precision=prec, device=local,
                                         cells_per_block=args.cells_per_block,
                                         nb_staging=args.nb_staging)
            ms, launches, errs, _ = time_steps(o, dt, args.steps, args.warmup, torch, barrier)
            ms = rep.max(ms)  # the slowest replica times the whole job
            n = o.n_dofs
            runs[prec] = {"ms": ms, "launches": int(launches), "errs": errs,
                          "value": n * STAGES * args.steps * ws / (ms / 1e3)}
            if prec == args.precision or args.precision == "auto":
                ops[prec] = o
            else:
                o.close()
    e64 = runs["fp64"]["errs"] if "fp64" in runs else None

    def ratio(prec):
        if e64 is None:
            return None, None
        e = runs[prec]["errs"]
        return (float(e[0] / e64[0]) if e64[0] > 0 else None,
                float(e[1] / e64[1]) if e64[1] > 0 else None)

    def matched(prec):
        rp, ru = ratio(prec)
        return bool(rp is not None and ru is not None and rp <= 1.1 and ru <= 1.1)

    if args.precision == "auto":
        ok = [p for p in order if matched(p)]
        head = min(ok, key=lambda p: runs[p]["ms"])
    else:
        head = args.precision
    for p in list(ops):
        if p != head:
            ops.pop(p).close()
    op = ops[head]
    n = op.n_dofs
    ms = runs[head]["ms"]
    ms_step = ms / args.steps
    value = runs[head]["value"]
    # per launch of stage_cart_kernel: average algorithmic bytes of the five
    # stages over the average launch duration (five launches per step)
    alg_bytes = BYTES_PER_DOF_STEP[head] * n / STAGES
    achieved = alg_bytes / (ms_step / STAGES / 1e3) / 1e9
    traffic = traffic_from_profiles(head, n)
    errs = runs[head]["errs"]
    rp, ru = ratio(head)
    result = {
        "metric": "DoF-updates/s", "value": value, "unit": "DoF-updates/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": DTYPES[head],
        "data": "synthetic",
        "config": {"workload": "3-D vibrating membrane, %d^3 affine hexes, FE_DGQ(%d), "
                               "LSRK45, %s" % (args.cells, args.degree, head),
                   "n_dofs": n, "dt": dt, "parallelism": "replicas x%d" % ws,
                   "precision": head,
                   "selection": "fastest precision with L2 errors (p and u, after the same "
                                "W + K steps) within 1.1x the FP64 path's"
                                if args.precision == "auto" else "forced by --precision",
                   "l2": "inputs larger than L2 (state %.2f GB)" % (n * 8 / 1e9)},
        "gpu_launches": runs[head]["launches"],
        "api": "ew_lsrk45_steps (%d steps in one call)" % args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind,
                     "traffic": traffic, "alg_bytes_per_launch": alg_bytes,
                     "launches_per_step": STAGES, "kernel": "stage_cart_kernel"},
        "errors": {"l2_p": errs[0], "l2_u": errs[1], "norm_p": errs[2],
                   "error_ratio_p_vs_fp64": rp, "error_ratio_u_vs_fp64": ru,
                   "matched_l2_error": matched(head) if e64 is not None else None},
        "precisions": {p: {"value": r["value"], "ms_per_step": r["ms"] / args.steps,
                           "dtype": DTYPES[p],
                           "hbm_frac": BYTES_PER_DOF_STEP[p] * n / (r["ms"] / args.steps / 1e3)
                           / 1e9 / peak,
                           "errors": {"l2_p": r["errs"][0], "l2_u": r["errs"][1]},
                           "error_ratio_p_vs_fp64": ratio(p)[0],
                           "error_ratio_u_vs_fp64": ratio(p)[1],
                           "matched_l2_error": matched(p) if e64 is not None else None,
                           "speedup_over_fp64": r["value"] / runs["fp64"]["value"]
                           if "fp64" in runs else None}
                       for p, r in runs.items()},
        "clocks": clk.summary(),
    }
    if not args.no_e2e:
        barrier()
        ms_e, h2d, d2h = e2e_steps(op, dt, args.steps, args.warmup, torch)
        ms_e = rep.max(ms_e)
        result["e2e"] = {"value": n * STAGES * args.steps * ws / (ms_e / 1e3),
                         "unit": "DoF-updates/s", "h2d_bytes_per_step": h2d,
                         "d2h_bytes_per_step": d2h, "ms_per_step": ms_e / args.steps}
    if rank == 0 and not args.no_cpu:
        try:
            result["cpu_baseline"] = cpu_sample(args.degree)
        except Exception as exc:  # the baseline must not hide the GPU result
            result["cpu_baseline"] = {"value": None, "error": str(exc)}
    if rank == 0:
        print(json.dumps(result), flush=True)
    rep.close()


if __name__ == "__main__":
    main()
