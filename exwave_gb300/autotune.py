"""Autotuner of the line kernel's launch shape and shared-memory layout.

For every (dimension, degree, precision: FP64, FP32 operator, compensated)
it builds a Cartesian membrane problem of about `target_dofs` DoFs and times
LSRK45 steps over two knobs: the cells per thread block (threads per block =
cells x lines of the kernel, one thread per (cell, direction, line), at most
512) and, in 3-D where both are built, the shared-memory layout of the
neighbour data (per-thread copies of each thread's neighbour lines, or bulk
copies of the neighbours' whole field arrays).  It keeps the fastest pair.
The threads per cell are fixed by the kernel's design (one per line), so
they are not a knob.  The table is written to
exwave_gb300/tuning/tuning.json and loaded by the library at import
(``ew_tune_set``, ``ew_tune_set_staging``), where ew_create and the batch
runtime use it.

Usage on the GPU: python -m exwave_gb300.autotune [--target-dofs 4e7]
"""
import argparse
import json
import os

import numpy as np

from . import _lib
from . import mesh as mesh_mod
from .operator import WaveEquationOperation

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE = os.path.join(HERE, "tuning", "tuning.json")


def lines_per_cell(dim, degree):
    return dim * (degree + 1) ** (dim - 1)


def candidates(dim, degree):
    lim = max(1, 512 // lines_per_cell(dim, degree))
    c = sorted({1, 2, 3, 4, 5, 6, 8, 10, 12, 16, 24, 32, lim} & set(range(1, lim + 1)))
    return c


def stagings(dim, degree, precision):
    """Neighbour layouts built for this case: 1 per-thread lines, 2 bulk arrays."""
    np_ = degree + 1
    bulk = dim == 3 and (np_ >= 6 or (np_ == 4 and precision == "mixed"))
    return [1, 2] if bulk else [1]


def time_case(dim, degree, precision, cells, cb, steps, torch, staging=0):
    m = mesh_mod.hypercube(dim, cells)
    dt = mesh_mod.time_step_size(m, 0.25 / degree ** 1.5)
    op = WaveEquationOperation(m, degree, precision=precision, cells_per_block=cb,
                               nb_staging=staging)
    u = op.project_membrane([1.0], [[1] * dim])
    v = torch.zeros_like(u)
    stream = torch.cuda.current_stream()
    op.set_stream(stream)
    op.lsrk45_steps(dt, 1, u, v)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    op.lsrk45_steps(dt, steps, v, u)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    n = op.n_dofs
    op.close()
    return n * 5 * steps / (ms / 1e3)


def run(dims=(2, 3), degrees=range(1, 8), precisions=("mixed", "mixed_ff", "fp64"), target_dofs=4e7,
        steps=4, log=print):
    import torch
    entries = []
    for dim in dims:
        for k in degrees:
            dofs_per_cell = (dim + 1) * (k + 1) ** dim
            cells = max(4, int(round((target_dofs / dofs_per_cell) ** (1.0 / dim))))
            for prec in precisions:
                best = None
                res = {}
                for st in stagings(dim, k, prec):
                    for cb in candidates(dim, k):
                        rate = time_case(dim, k, prec, cells, cb, steps if prec == "mixed" else 2,
                                         torch, staging=st)
                        res[(cb, st)] = rate
                        if best is None or rate > res[best]:
                            best = (cb, st)
                entries.append({"dim": dim, "degree": k, "precision": prec,
                                "cells_per_block": best[0], "nb_staging": best[1], "cells": cells,
                                "rates": {"%d/%d" % c: r for c, r in res.items()}})
                if log:
                    log("dim %d k %d %s: best cb %d staging %d (%.3g DoF-updates/s)"
                        % (dim, k, prec, best[0], best[1], res[best]))
    return entries


def save(entries, gpu_name, merge=False):
    """Write the table; with merge, entries of other (dim, degree, precision)
    already in the table are kept."""
    os.makedirs(os.path.dirname(TABLE), exist_ok=True)
    if merge and os.path.exists(TABLE):
        with open(TABLE) as f:
            old = json.load(f).get("entries", [])
        key = lambda e: (e["dim"], e["degree"], e["precision"])
        new_keys = {key(e) for e in entries}
        entries = [e for e in old if key(e) not in new_keys] + entries
        entries.sort(key=lambda e: (e["dim"], e["degree"], e["precision"]))
    with open(TABLE, "w") as f:
        json.dump({"gpu": gpu_name, "entries": entries}, f, indent=1)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--target-dofs", type=float, default=4e7)
    ap.add_argument("--dims", default="2,3")
    ap.add_argument("--precisions", default="mixed,mixed_ff,fp64")
    ap.add_argument("--degrees", default="1,7", help="degree range (inclusive)")
    ap.add_argument("--merge", action="store_true", help="keep the table's other entries")
    args = ap.parse_args()
    import torch
    _lib.load()
    lo, hi = (int(x) for x in args.degrees.split(","))
    entries = run(dims=[int(d) for d in args.dims.split(",")], degrees=range(lo, hi + 1),
                  precisions=args.precisions.split(","), target_dofs=args.target_dofs)
    save(entries, torch.cuda.get_device_name(0), merge=args.merge)
    print("wrote", TABLE)


if __name__ == "__main__":
    main()
