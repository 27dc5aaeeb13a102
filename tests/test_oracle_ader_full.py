"""ADER without spectral evaluation in the oracle (parameters.cc:76;
wave_equation_operations.cc:1013, 1037, 1086-1090, 1205-1233).  The
reference has no regression output for it, so the restatement is checked by
its defining properties: up to degree 3 the Cauchy-Kovalevskaya recursion
never reaches a degree reduction, so both evaluations are the same
computation; from degree 4 on they differ, by much less than the
discretisation error, and both stay as accurate against the analytic
membrane solution."""
import numpy as np
import pytest


def _run(oracle_mod, dim, k, spectral, steps, n=3):
    P = oracle_mod.Problem.hypercube(dim, k, n, 0, 0.1, 2)
    P.set_spectral(spectral)
    u = P.project_reference(2)
    v = np.zeros_like(u)
    dt = P.time_step(0.2 / k ** 1.5)
    for _ in range(steps):
        P.ader_step(dt, u, v)
        u, v = v, u
    return P, u, dt


@pytest.mark.parametrize("k", [1, 2, 3])
def test_same_as_spectral_below_degree_4(oracle_mod, k):
    _, a, _ = _run(oracle_mod, 2, k, True, 3)
    _, b, _ = _run(oracle_mod, 2, k, False, 3)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("dim,k", [(2, 4), (2, 6), (3, 5)])
def test_differs_within_the_discretisation_error(oracle_mod, dim, k):
    steps = 10
    Pa, a, dt = _run(oracle_mod, dim, k, True, steps, n=2 if dim == 3 else 3)
    Pb, b, _ = _run(oracle_mod, dim, k, False, steps, n=2 if dim == 3 else 3)
    diff = np.abs(a - b).max() / np.abs(a).max()
    assert 0.0 < diff < 1e-3
    ea = np.zeros(3)
    eb = np.zeros(3)
    oracle_mod.lib().ewo_errors_reference(Pa.h, oracle_mod._dp(a), 2, steps * dt, oracle_mod._dp(ea))
    oracle_mod.lib().ewo_errors_reference(Pb.h, oracle_mod._dp(b), 2, steps * dt, oracle_mod._dp(eb))
    assert eb[0] < 3.0 * ea[0] and ea[0] < 3.0 * eb[0], (ea, eb)
