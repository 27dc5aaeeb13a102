"""The CPU oracle reproduces the reference's own regression outputs.

Golden data: ``tests/golden/reference_runs.json``, extracted by
``tests/golden/make_golden.py`` from the reference's ``tests/*.prm`` and
``tests/*.output``.  Every printed "error p", "error v" and "solution mag p"
value (4 digits after the point in scientific notation,
explicit_wave.cc:509-519) and every output step number must match exactly.
The post-processed pressure's "error p post" (compute_post_pressure,
wave_equation_operations.cc:784-848) is compared to one unit of the last
printed digit.
ADERLTS (local time stepping) is out of scope.
"""
import json
import math
import os

import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_runs.json")
with open(GOLDEN) as f:
    RUNS = json.load(f)

IN_SCOPE = [n for n, r in sorted(RUNS.items()) if r["params"]["time_integrator"] != "ADERLTS"]


@pytest.mark.parametrize("name", IN_SCOPE)
def test_golden_error_lines(oracle_mod, name):
    run = RUNS[name]
    p = run["params"]
    prob = oracle_mod.Problem.hypercube(p["dimension"], p["fe_degree"], p["n_initial_intervals"],
                                        p["n_refinements"], p["grid_transform_factor"],
                                        p["boundary_id"])
    prob.set_ader_post(p["use_ader_post"])
    rows, dt = prob.run_reference(p["time_integrator"], p["cfl_number"], p["final_time"],
                                  p["output_every_time"], p["membrane_modes"],
                                  p["max_time_steps"])
    # printed with the default 6 significant digits (explicit_wave.cc:701)
    assert "%g" % dt == run["time_step"]
    assert len(rows) == len(run["rows"])
    for mine, ref in zip(rows, run["rows"]):
        assert "%.2f" % mine[0] == ref["time"]
        assert int(mine[1]) == ref.get("step", 0)
        assert "%.4e" % mine[2] == ref["error_p"], (name, ref["time"])
        assert "%.4e" % mine[3] == ref["error_v"], (name, ref["time"])
        assert "%.4e" % mine[4] == ref["solution_mag_p"], (name, ref["time"])
        # p* is solved in another basis than the reference's FE_DGQ(k+1)
        # (the same function up to round-off): one unit of the last printed
        # digit, for values near a rounding tie
        post = float(ref["error_p_post"])
        ulp = 10.0 ** (math.floor(math.log10(post)) - 4)
        assert abs(mine[5] - post) <= ulp, (name, ref["time"], mine[5], post)
