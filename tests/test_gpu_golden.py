"""The GPU FP64 path replays the reference's regression runs: every printed
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


@pytest.mark.parametrize("name", NAMES)
def test_gpu_replays_golden(name):
    from exwave_gb300 import build, driver
    build.build()
    run = RUNS[name]
    p = dict(run["params"])
    p["cfl_scaled"] = p["cfl_number"] / p["fe_degree"] ** 1.5
    rows, dt = driver.run(p, precision="fp64")
    assert "%g" % dt == run["time_step"]
    assert len(rows) == len(run["rows"])
    for mine, ref in zip(rows, run["rows"]):
        assert "%.2f" % mine[0] == ref["time"]
        assert mine[1] == ref.get("step", 0)
        assert "%.4e" % mine[2] == ref["error_p"], (name, ref["time"])
        assert "%.4e" % mine[3] == ref["error_v"], (name, ref["time"])
        assert "%.4e" % mine[4] == ref["solution_mag_p"], (name, ref["time"])
        # p* is solved in another basis than the reference's FE_DGQ(k+1):
        # one unit of the last printed digit, for values near a rounding tie
        post = float(ref["error_p_post"])
        ulp = 10.0 ** (math.floor(math.log10(post)) - 4)
        assert abs(mine[5] - post) <= ulp, (name, ref["time"], mine[5], post)
