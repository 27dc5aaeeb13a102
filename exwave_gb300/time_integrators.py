"""Explicit integrators over the GPU operator, mirroring the reference's
``ExplicitIntegrator<VectorType,Operator>::perform_time_step(vec_n, vec_np,
time_step, op)`` (time_integrators.h:25-39)."""


class ExplicitIntegrator:
    def perform_time_step(self, vec_n, vec_np, time_step, op):
        raise NotImplementedError


class LowStorageRK45Reg2(ExplicitIntegrator):
    """Kennedy-Carpenter 5-stage, 2-register RK (time_integrators.cc:235-283),
    fused: five launches of operator + stage update.  vec_n is clobbered."""

    def perform_time_step(self, vec_n, vec_np, time_step, op):
        op.lsrk45_step(time_step, vec_n, vec_np)


class ArbitraryHighOrderDG(ExplicitIntegrator):
    """ADER step (time_integrators.cc:37-50): vec_np = vec_n - apply_ader(vec_n),
    as the Cauchy-Kovalevskaya kernel plus the fused second step."""

    def perform_time_step(self, vec_n, vec_np, time_step, op):
        op.ader_step(time_step, vec_n, vec_np)


class AderAdconFull(ExplicitIntegrator):
    """The ADER step with the operator of WaveEquationOperationADERADCONFULL
    (wave_equation_operations.cc:689-735): the Taylor series of the time
    integral from k+1 applications of the full DG operator."""

    def perform_time_step(self, vec_n, vec_np, time_step, op):
        op.aderadconfull_step(time_step, vec_n, vec_np)


class ClassRK4(ExplicitIntegrator):
    """Classical RK4 (time_integrators.cc:66-102) composed from apply and
    vector updates."""

    def __init__(self):
        self.t1 = None
        self.t2 = None

    def perform_time_step(self, vec_n, vec_np, time_step, op):
        if self.t1 is None or self.t1.numel() != vec_n.numel():
            self.t1 = vec_n.new_zeros(vec_n.numel())
            self.t2 = vec_n.new_zeros(vec_n.numel())
        t1, t2 = self.t1, self.t2
        op.apply(vec_n, t1)
        vec_np.copy_(vec_n).add_(t1, alpha=time_step / 6.0)
        t2.copy_(vec_n).add_(t1, alpha=0.5 * time_step)
        op.apply(t2, t1)
        vec_np.add_(t1, alpha=time_step / 3.0)
        t2.copy_(vec_n).add_(t1, alpha=0.5 * time_step)
        op.apply(t2, t1)
        vec_np.add_(t1, alpha=time_step / 3.0)
        t2.copy_(vec_n).add_(t1, alpha=time_step)
        op.apply(t2, t1)
        vec_np.add_(t1, alpha=time_step / 6.0)
