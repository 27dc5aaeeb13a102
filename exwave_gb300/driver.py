"""Time loop of one solve on the GPU, mirroring WaveEquationProblem::run
(explicit_wave.cc:549-813): mesh, time step, initial field, integrator,
output of L2 errors at every tick."""
from . import mesh as mesh_mod
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


def run(params, precision="fp64", on_output=None):
    """Run the parameter set; returns rows (time, step, err p, err u, |p|,
    err p post) and the time step used.  ``params`` as returned by parameters.parse_prm."""
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
                               use_ader_post=params["use_ader_post"] and integ == "ADER")
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
