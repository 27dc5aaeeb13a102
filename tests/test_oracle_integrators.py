"""The oracle's restatements of the reference's composed integrators
(time_integrators.cc:24-31, 66-102, 200-478, 726-795) have no golden output
in the reference's tests; their coefficient tables are checked by the order
of accuracy: on the linear system du/dt = M^-1 A u the local error of one
step against exp(dt M^-1 A) u (a 60-term Taylor series) falls by 2^(p+1)
when dt is halved."""
import numpy as np
import pytest

from oracle import oracle as O

ORDERS = {"ExplEuler": 1, "LSRK33R2": 3, "LSRK45R2": 4, "LSRK45R3": 4, "LSRK59R2": 5,
          "SSPRK": 4, "clRK4": 4}


@pytest.fixture(scope="module")
def problem():
    P = O.Problem.hypercube(2, 3, 3, 0, 0.0, 2)
    u0 = np.zeros(P.n_dofs)
    O.lib().ewo_project_reference(P.h, 2, 0.0, O._dp(u0))
    dt = O.lib().ewo_time_step(P.h, 0.2 / 3 ** 1.5)
    return P, u0, dt


def _exp_step(P, u, dt, terms=60):
    out = u.copy()
    t = u.copy()
    for j in range(1, terms):
        t = P.apply(t) * (dt / j)
        out += t
    return out


@pytest.mark.parametrize("name", sorted(ORDERS))
def test_integrator_order(problem, name):
    P, u0, dt0 = problem
    errs = []
    for dt in (dt0 / 2, dt0 / 4):
        a = u0.copy()
        b = np.zeros_like(u0)
        P.step(name, dt, a, b)
        errs.append(np.linalg.norm(b - _exp_step(P, u0, dt)) / np.linalg.norm(u0))
    ratio = errs[0] / errs[1]
    expected = 2.0 ** (ORDERS[name] + 1)
    assert 0.85 * expected < ratio < 1.3 * expected, (name, errs, ratio)


def test_run_reference_accepts_all_integrators():
    P = O.Problem.hypercube(2, 2, 2, 0, 0.0, 2)
    for name in ("ExplEuler", "LSRK33R2", "LSRK45R3", "LSRK59R2", "SSPRK"):
        rows, dt = P.run_reference(name, 0.1, 0.05, 0.05, 2)
        assert rows.shape[0] >= 2 and np.all(np.isfinite(rows))
