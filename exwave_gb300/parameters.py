"""Reader for the reference's parameter files (deal.II ParameterHandler
syntax, the entries of parameters.cc:36-100) -- the subset the hot path uses.
Defaults are the reference's declared defaults."""
import re

DEFAULTS = {
    "dimension": 2, "boundary_id": 2, "grid_transform_factor": 0.1, "fe_degree": 2,
    "n_initial_intervals": 5, "n_refinements": 0, "n_adaptive_refinements": 0,
    "adaptive_refinement_interval": 0, "time_integrator": "ADER", "cfl_number": 0.1,
    "max_time_steps": 0, "final_time": 1.0, "output_every_time": 0.1, "write_vtu_output": False,
    "cfl_stability_analysis": False, "use_ader_post": False, "spectral_evaluation": True,
    "max_n_clusters": 10, "max_diff_clusters": 7, "initital_cases": 1, "membrane_modes": 2,
    "output_parameters": True,
}
INTEGRATORS = ("ExplEuler", "clRK4", "LSRK45R2", "LSRK33R2", "LSRK45R3", "LSRK59R2", "SSPRK",
               "ADER", "ADERLTS", "ADERADCONFULL")


def _convert(key, text):
    ref = DEFAULTS[key]
    if isinstance(ref, bool):
        if text not in ("true", "false"):
            raise ValueError("%s expects true/false, got %r" % (key, text))
        return text == "true"
    if isinstance(ref, int):
        return int(text)
    if isinstance(ref, float):
        return float(text)
    return text


def parse_prm(text):
    """Parse parameter-file text; unknown keys raise like ParameterHandler."""
    p = dict(DEFAULTS)
    for raw in text.splitlines():
        line = raw.split("#", 1)[0].strip()
        if not line or line.startswith("subsection") or line == "end":
            continue
        m = re.match(r"set\s+(\w+)\s*=\s*(.*)$", line)
        if not m:
            raise ValueError("cannot parse line: %r" % raw)
        key, val = m.group(1), m.group(2).strip()
        if key not in DEFAULTS:
            raise ValueError("unknown parameter %r" % key)
        p[key] = _convert(key, val)
    if p["time_integrator"] not in INTEGRATORS:
        raise ValueError("unknown time integrator " + p["time_integrator"])
    # the Courant number is scaled by k^1.5 (parameters.cc:195)
    p["cfl_scaled"] = p["cfl_number"] / p["fe_degree"] ** 1.5
    return p


def read_prm(path):
    with open(path) as f:
        return parse_prm(f.read())
