"""Extract the reference's regression goldens into a small JSON fixture.

Reads the ExWave reference's own test inputs and expected outputs
(``tests/*.prm`` and ``tests/*.output`` of kronbichler/exwave) as text and
writes ``reference_runs.json`` next to this script: for every test, the
parameters that matter for the hot path and the printed time-step size and
per-tick error lines ("error p", "error p post", "error v", "solution mag p",
explicit_wave.cc:509-519 of the reference).

Usage (only where the reference checkout is available):
    python tests/golden/make_golden.py /path/to/exwave
"""
import json
import os
import re
import sys

KEYS = {
    "dimension": int,
    "fe_degree": int,
    "n_initial_intervals": int,
    "n_refinements": int,
    "grid_transform_factor": float,
    "time_integrator": str,
    "cfl_number": float,
    "max_time_steps": int,
    "final_time": float,
    "output_every_time": float,
    "use_ader_post": lambda s: s.strip() == "true",
    "spectral_evaluation": lambda s: s.strip() == "true",
    "membrane_modes": int,
    "boundary_id": int,
}

LINE = re.compile(
    r"Time:\s*([0-9.]+)\s*,\s*error p:\s*([0-9.eE+-]+)\s*,\s*error p post:\s*([0-9.eE+-]+)"
    r"\s*,\s*error v:\s*([0-9.eE+-]+)\s*,\s*solution mag p:\s*([0-9.eE+-]+)")
STEP = re.compile(r"write output for time step (\d+) at time ([0-9.]+)")


def parse_prm(text):
    params = {"boundary_id": 2, "spectral_evaluation": True, "use_ader_post": False}
    for line in text.splitlines():
        line = line.split("#", 1)[0].strip()
        m = re.match(r"set\s+(\w+)\s*=\s*(.+)", line)
        if m and m.group(1) in KEYS:
            params[m.group(1)] = KEYS[m.group(1)](m.group(2).strip())
    return params


def parse_output(text):
    rows = []
    for line in text.splitlines():
        m = LINE.search(line)
        if m:
            rows.append({"time": m.group(1), "error_p": m.group(2), "error_p_post": m.group(3),
                         "error_v": m.group(4), "solution_mag_p": m.group(5)})
            continue
        m = STEP.search(line)
        if m and rows:
            rows[-1]["step"] = int(m.group(1))
    dts = re.findall(r"^\s+Time step size:\s*([0-9.eE+-]+)", text, re.M)
    rounded = re.findall(r"^Time step size:\s*([0-9.eE+-]+)", text, re.M)
    return rows, (dts[-1] if dts else None), (rounded[0] if rounded else None)


def main(ref_root):
    tdir = os.path.join(ref_root, "tests")
    runs = {}
    for name in sorted(os.listdir(tdir)):
        if not name.endswith(".prm"):
            continue
        base = name[:-4]
        with open(os.path.join(tdir, name)) as f:
            params = parse_prm(f.read())
        out_path = os.path.join(tdir, base + ".output")
        if not os.path.exists(out_path):
            continue
        with open(out_path) as f:
            rows, dt, dt_rounded = parse_output(f.read())
        runs[base] = {"params": params, "time_step": dt, "time_step_rounded": dt_rounded,
                      "rows": rows}
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "reference_runs.json"), "w") as f:
        json.dump(runs, f, indent=1, sort_keys=True)
    print("wrote", len(runs), "runs")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
