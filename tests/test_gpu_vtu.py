"""The driver's VTU output (write_vtu_output, output_results in
explicit_wave.cc:336-406) from a GPU run: one file per output time with the
reference's name, the solution plus its error equal to the exact membrane
pressure at the patch points to the discretisation error."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_driver_writes_vtu(tmp_path):
    from exwave_gb300 import build, driver, parameters, vtu
    build.build()
    p = parameters.parse_prm("""
subsection General
  set dimension = 2
  set fe_degree = 4
  set n_initial_intervals = 8
  set grid_transform_factor = 0.0
  set time_integrator = LSRK45R2
  set cfl_number = 0.2
  set final_time = 0.2
  set output_every_time = 0.1
  set membrane_modes = 2
  set write_vtu_output = true
end
""")
    rows, dt = driver.run(p, precision="fp64", output_dir=str(tmp_path))
    names = sorted({vtu.output_name(4, "Runge-Kutta", 1, 0, int(r[0] / 0.1)) for r in rows})
    assert sorted(os.listdir(tmp_path)) == names
    arr, npts, ncells = vtu.read_vtu(str(tmp_path / names[-1]))
    assert npts == 64 * 25 and ncells == 64 * 16
    x = arr["Points"]
    t = rows[-1][0]
    w = 2 * np.sqrt(2) * np.pi
    exact = np.cos(w * t) * np.sin(2 * np.pi * x[:, 0]) * np.sin(2 * np.pi * x[:, 1])
    total = arr["solution_pressure"][:, 0] + arr["error_pressure"][:, 0]
    assert np.abs(total - exact).max() < 1e-4
    assert 0 < np.abs(arr["error_pressure"]).max() < 1e-4
