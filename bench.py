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
 - cpu_baseline: the CPU restatement (oracle, OpenMP, all host threads) on a
   bounded sample (16^3 cells, same degree).

--impl reference: the CPU implementation of the path on the host cores
(the reference itself cannot be built: it needs deal.II, p4est and MPI), on
the same metric; rank 0 only.
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
BYTES_PER_DOF_STEP = {"mixed": 112.0, "fp64": 144.0}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cells", type=int, default=64)
    ap.add_argument("--degree", type=int, default=5)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 comparison run")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    return ap.parse_args()


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


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
    for _ in range(warmup):
        op.lsrk45_step(dt, u, v)
        u, v = v, u
    torch.cuda.synchronize()
    barrier()
    stream = torch.cuda.current_stream()
    op.set_stream(stream)
    l0 = op.kernel_launches()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(steps):
        op.lsrk45_step(dt, u, v)
        u, v = v, u
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier()
    ms = ev0.elapsed_time(ev1)
    launches = op.kernel_launches() - l0
    t_end = (warmup + steps) * dt
    errs = op.l2_errors(u, *MODES, t_end)
    return ms, launches, errs, u


def e2e_steps(op, dt, steps, warmup, torch):
    """Same step through the public API with the state in pinned host
    memory: H2D copy, LSRK45 step, D2H copy, each step."""
    n = op.n_dofs
    host = torch.empty(n, dtype=torch.float64, pin_memory=True)
    host.copy_(op.project_membrane(*MODES, 0.0).cpu())
    d_in = torch.empty(n, dtype=torch.float64, device="cuda")
    d_out = torch.empty_like(d_in)
    stream = torch.cuda.current_stream()
    op.set_stream(stream)

    def one():
        d_in.copy_(host, non_blocking=True)
        op.lsrk45_step(dt, d_in, d_out)
        host.copy_(d_out, non_blocking=True)

    for _ in range(warmup):
        one()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(steps):
        one()
    ev1.record(stream)
    torch.cuda.synchronize()
    return ev0.elapsed_time(ev1), n * 8, n * 8


def cpu_sample(degree, min_seconds=8.0):
    """The CPU restatement (oracle) on a bounded sample of the workload."""
    import numpy as np
    from oracle import oracle
    oracle.build()
    cells = 16
    prob = oracle.Problem.hypercube(3, degree, cells, 0, 0.0, 2)
    dt = prob.time_step(0.25 / degree ** 1.5)
    u = prob.project_modes(*MODES)
    v = np.zeros_like(u)
    prob.lsrk45_step(dt, u, v)  # warm-up
    steps = 0
    t0 = time.perf_counter()
    while True:
        prob.lsrk45_step(dt, v, u)
        u, v = v, u
        steps += 1
        el = time.perf_counter() - t0
        if el >= min_seconds:
            break
    rate = prob.n_dofs * STAGES * steps / el
    return {"value": rate, "unit": "DoF-updates/s", "cores": oracle.num_threads(), "kind": "port",
            "sample": "3-D k=%d, %d^3 affine cells (%d DoFs), %d LSRK45 steps, OpenMP"
                      % (degree, cells, prob.n_dofs, steps)}


def traffic_from_profiles(precision, n_dofs):
    """DRAM bytes per stage launch from the committed ncu summary, scaled to
    this workload's DoF count (traffic grows in proportion to the cells)."""
    path = os.path.join(ROOT, "profiles", "stage_kernel_traffic.json")
    try:
        with open(path) as f:
            d = json.load(f)
        e = d[precision]
        return e["dram_bytes_per_dof_stage"] * n_dofs
    except (OSError, KeyError, ValueError):
        return None


def run_reference(args):
    ws, rank, _ = dist_info()
    if rank != 0:
        return
    import numpy as np
    from oracle import oracle
    oracle.build()
    cells = 16
    prob = oracle.Problem.hypercube(3, args.degree, cells, 0, 0.0, 2)
    dt = prob.time_step(0.25 / args.degree ** 1.5)
    u = prob.project_modes(*MODES)
    v = np.zeros_like(u)
    for _ in range(args.warmup):
        prob.lsrk45_step(dt, u, v)
        u, v = v, u
    t0 = time.perf_counter()
    for _ in range(args.steps):
        prob.lsrk45_step(dt, u, v)
        u, v = v, u
    el = time.perf_counter() - t0
    value = prob.n_dofs * STAGES * args.steps / el
    sample = ("3-D k=%d, %d^3 affine cells (%d DoFs) per step; the reference (deal.II "
              "MatrixFree) cannot be built on this image, the CPU restatement of its arithmetic "
              "is timed" % (args.degree, cells, prob.n_dofs))
    line = {
        "impl": "reference", "metric": "DoF-updates/s", "value": value, "unit": "DoF-updates/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": el / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "3-D membrane, FE_DGQ(%d) hexes, LSRK45 (sampled at %d^3 cells)"
                               % (args.degree, cells), "precision": "fp64"},
        "cpu_baseline": {"value": value, "unit": "DoF-updates/s", "cores": oracle.num_threads(),
                         "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "DoF-updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    import torch
    ws, rank, local = dist_info()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")

        def barrier():
            dist.barrier()
    else:
        def barrier():
            pass
    import exwave_gb300 as ew
    from exwave_gb300 import build
    build.build()
    import numpy as np
    with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
        peaks = json.load(f)
    peak, peak_kind = float(peaks["hbm_gbs"]), "measured"
    m, dt = build_problem(args.cells, args.degree)
    op = ew.WaveEquationOperation(m, args.degree, precision=args.precision, device=local)
    n = op.n_dofs
    with ClockSampler(local) as clk:
        ms, launches, errs, _ = time_steps(op, dt, args.steps, args.warmup, torch, barrier)
    t = torch.tensor([ms], dtype=torch.float64, device="cuda")
    if ws > 1:
        import torch.distributed as dist
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms = float(t.item())
    ms_step = ms / args.steps
    value = n * STAGES * args.steps * ws / (ms / 1e3)
    alg_bytes = BYTES_PER_DOF_STEP[args.precision] * n
    achieved = alg_bytes / (ms_step / 1e3) / 1e9
    traffic = traffic_from_profiles(args.precision, n)
    result = {
        "metric": "DoF-updates/s", "value": value, "unit": "DoF-updates/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32-operator/f64-state" if args.precision == "mixed" else "f64",
        "data": "synthetic",
        "config": {"workload": "3-D vibrating membrane, %d^3 affine hexes, FE_DGQ(%d), "
                               "LSRK45, %s" % (args.cells, args.degree, args.precision),
                   "n_dofs": n, "dt": dt, "parallelism": "replicas x%d" % ws,
                   "l2": "inputs larger than L2 (state %.2f GB)" % (n * 8 / 1e9)},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind,
                     "traffic": traffic, "alg_bytes_per_step": alg_bytes,
                     "kernel": "stage_kernel (5 launches per step)"},
        "errors": {"l2_p": errs[0], "l2_u": errs[1], "norm_p": errs[2]},
        "clocks": clk.summary(),
    }
    if not args.no_fp64 and args.precision == "mixed":
        op64 = ew.WaveEquationOperation(m, args.degree, precision="fp64", device=local)
        ms64, _, errs64, _ = time_steps(op64, dt, max(2, args.steps // 4), 1, torch, barrier)
        st64 = max(2, args.steps // 4)
        v64 = n * STAGES * st64 * ws / (ms64 / 1e3)
        result["fp64"] = {"value": v64, "ms_per_step": ms64 / st64,
                          "errors": {"l2_p": errs64[0], "l2_u": errs64[1]},
                          "speedup_mixed_over_fp64": value / v64,
                          "error_ratio_p": errs[0] / errs64[0] if errs64[0] > 0 else None}
        op64.close()
        del op64
    if not args.no_e2e:
        ms_e, h2d, d2h = e2e_steps(op, dt, args.steps, args.warmup, torch)
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
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
