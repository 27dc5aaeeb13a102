"""Time loop of one solve on the GPU, mirroring WaveEquationProblem::run
(explicit_wave.cc:549-813): mesh, time step, initial field, integrator,
output of L2 errors at every tick and, with ``write_vtu_output``, a VTU file
of the solution and its error (output_results, explicit_wave.cc:336-406)."""
import os

from . import mesh as mesh_mod
from . import vtu
from .operator import WaveEquationOperation, reference_mode
from .time_integrators import (SSPRK, AderAdconFull, ArbitraryHighOrderDG, ClassRK4, ExplicitEuler,
                               LowStorageRK33Reg2, LowStorageRK45Reg2, LowStorageRK45Reg3,
                               LowStorageRK59Reg2)
from .utilities import TimeControl

# the integrators of parameters.cc:58 except ADERLTS (local time stepping)
SUPPORTED = {"ExplEuler": ExplicitEuler, "clRK4": ClassRK4, "LSRK45R2": LowStorageRK45Reg2,
             "LSRK33R2": LowStorageRK33Reg2, "LSRK45R3": LowStorageRK45Reg3,
             "LSRK59R2": LowStorageRK59Reg2, "SSPRK": SSPRK, "ADER": ArbitraryHighOrderDG,
             "ADERADCONFULL": AderAdconFull}


# Name() of the reference's operators (wave_equation_operations.cc:105-167)
OPERATOR_NAMES = {"ADER": "ADER", "ADERADCONFULL": "ADERADCONFULL"}


def run(params, precision="fp64", on_output=None, output_dir="output"):
    """Run the parameter set; returns rows (time, step, err p, err u, |p|,
    err p post) and the time step used.  ``params`` as returned by
    parameters.parse_prm; VTU files go to ``output_dir``."""
    import torch
    integ = params["time_integrator"]
    if integ not in SUPPORTED:
        raise NotImplementedError("time integrator %s is not built" % integ)
    if params.get("n_adaptive_refinements", 0):
        raise NotImplementedError("adaptive mesh refinement is not built")
    dim, k = params["dimension"], params["fe_degree"]
    m = mesh_mod.hypercube(dim, params["n_initial_intervals"], params["n_refinements"],
                           params["grid_transform_factor"], "reference", params["boundary_id"])
    op = WaveEquationOperation(m, k, precision=precision,
                               use_ader_post=params["use_ader_post"] and integ == "ADER",
                               spectral_evaluation=params.get("spectral_evaluation", True))
    amps, kv = reference_mode(dim, params["membrane_modes"])
    tc = TimeControl()
    dt0 = mesh_mod.time_step_size(m, params["cfl_scaled"])
    tc.setup(params["final_time"], params["output_every_time"], dt0,
             params.get("max_time_steps", 0))
    tc.set_time_step(dt0)  # make_dofs resets the unrounded step (explicit_wave.cc:222)
    sol = op.project_membrane(amps, kv, 0.0)
    tmp = torch.zeros_like(sol)
    integrator = SUPPORTED[integ]()
    rows = []

    def output():
        e = op.l2_errors(sol, amps, kv, tc.time)
        post = op.l2_error_post(sol, amps, kv, tc.time)
        rows.append((tc.time, tc.time_step_number, e[0], e[1], e[2], post))
        if params.get("write_vtu_output"):
            name = vtu.output_name(k, OPERATOR_NAMES.get(integ, "Runge-Kutta"),
                                   params.get("initital_cases", 1), params["n_refinements"],
                                   int(tc.time / tc.tick_size))
            vtu.write_vtu(os.path.join(output_dir, name), m, k, sol,
                          exact=op.project_membrane(amps, kv, tc.time))
        if on_output:
            on_output(rows[-1])

    output()
    while not tc.done():
        tc.advance_time_step()
        tmp, sol = sol, tmp
        integrator.perform_time_step(tmp, sol, tc.time_step, op)
        if tc.at_tick():
            output()
    op.synchronize()
    return rows, tc.time_step
