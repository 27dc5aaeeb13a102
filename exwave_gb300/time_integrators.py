"""Explicit integrators over the GPU operator, mirroring the reference's
``ExplicitIntegrator<VectorType,Operator>::perform_time_step(vec_n, vec_np,
time_step, op)`` (time_integrators.h:25-39).  As in the reference, vec_n may
be used as a register (its content afterwards is unspecified) and the new
state is left in vec_np.  Vector operations run on the device through
``op.vec_update`` (y = alpha y + (beta x + gamma z))."""


class ExplicitIntegrator:
    def perform_time_step(self, vec_n, vec_np, time_step, op):
        raise NotImplementedError


def _scratch(holder, name, like, count):
    """Integrator-owned scratch vectors, (re)allocated lazily like the
    reference's vec_tmp1 (time_integrators.cc:254-257)."""
    vs = getattr(holder, name, None)
    if vs is None or vs[0].numel() != like.numel():
        vs = [like.new_zeros(like.numel()) for _ in range(count)]
        setattr(holder, name, vs)
    return vs


class ExplicitEuler(ExplicitIntegrator):
    """vec_np = vec_n + dt M^-1 A(vec_n) (time_integrators.cc:24-31)."""

    def perform_time_step(self, vec_n, vec_np, time_step, op):
        op.apply(vec_n, vec_np)
        op.vec_update(time_step, vec_np, 1.0, vec_n)


class LowStorageRK45Reg2(ExplicitIntegrator):
    """Kennedy-Carpenter 5-stage, 2-register RK (time_integrators.cc:235-283),
    fused: five launches of operator + stage update.  vec_n is clobbered."""

    def perform_time_step(self, vec_n, vec_np, time_step, op):
        op.lsrk45_step(time_step, vec_n, vec_np)


class LowStorageRK33Reg2(ExplicitIntegrator):
    """3-stage, 2-register RK (time_integrators.cc:200-233), fused stages."""

    def perform_time_step(self, vec_n, vec_np, time_step, op):
        op.lsrk_step("LSRK33R2", time_step, vec_n, vec_np)


class LowStorageRK59Reg2(ExplicitIntegrator):
    """9-stage, 2-register RK of order 5 (time_integrators.cc:286-364), fused stages."""

    def perform_time_step(self, vec_n, vec_np, time_step, op):
        op.lsrk_step("LSRK59R2", time_step, vec_n, vec_np)


class LowStorageRK45Reg3(ExplicitIntegrator):
    """5-stage, 3-register RK (time_integrators.cc:366-427): the reference's
    sequence of operator applications and vector operations."""

    A21 = 2365592473904. / 8146167614645.
    A32 = 4278267785271. / 6823155464066.
    A43 = 2789585899612. / 8986505720531.
    A54 = 15310836689591. / 24358012670437.
    A31 = -722262345248. / 10870640012513.
    A42 = 1365858020701. / 8494387045469.
    A53 = 3819021186. / 2763618202291.
    B1 = 846876320697. / 6523801458457.
    B2 = 3032295699695. / 12397907741132.
    B3 = 612618101729. / 6534652265123.
    B4 = 1155491934595. / 2954287928812.
    B5 = 707644755468. / 5028292464395.

    def perform_time_step(self, vec_n, vec_np, time_step, op):
        t1, t2 = _scratch(self, "_tmp", vec_n, 2)
        dt = time_step
        u = op.vec_update
        op.apply(vec_n, vec_np)
        u(1.0, vec_n, self.A21 * dt, vec_np)
        u(0.0, t1, 1.0, vec_n)
        u(1.0, t1, (self.B1 - self.A21) * dt, vec_np)
        op.apply(vec_n, t2)
        u(1.0, t1, self.A32 * dt, t2, (self.A31 - self.B1) * dt, vec_np)
        u((self.B1 - self.A31) * dt, vec_np, 1.0, t1)
        u(1.0, vec_np, (self.B2 - self.A32) * dt, t2)
        op.apply(t1, vec_n)
        u(1.0, vec_np, self.A43 * dt, vec_n, (self.A42 - self.B2) * dt, t2)
        u((self.B2 - self.A42) * dt, t2, 1.0, vec_np)
        u(1.0, t2, (self.B3 - self.A43) * dt, vec_n)
        op.apply(vec_np, t1)
        u(1.0, t2, self.A54 * dt, t1, (self.A53 - self.B3) * dt, vec_n)
        u(0.0, vec_np, 1.0, t2)
        u(1.0, vec_np, (self.B3 - self.A53) * dt, vec_n, (self.B4 - self.A54) * dt, t1)
        op.apply(t2, t1)
        u(1.0, vec_np, self.B5 * dt, t1)


class SSPRK(ExplicitIntegrator):
    """Strong-stability-preserving RK of order 4 with 8 stages, the scheme the
    reference instantiates (SSPRK(4,8), explicit_wave.cc:758;
    time_integrators.cc:440-478): u_s = sum_{l<s} A[s-1][l] u_l +
    dt B[s-1][l] M^-1 A(u_l), u_0 = vec_n, vec_np = u_8.  The nonzero
    coefficients of initialize_coeffs (time_integrators.cc:726-795), per row
    as (l, A, B)."""

    ROWS = (
        ((0, 1., 0.282318339066479),),
        ((0, 0.538569155333175, 0.), (1, 0.461430844666825, 0.130270389660380)),
        ((0, 0.004485387460763, 0.003963092203460), (2, 0.995514612539237, 0.281052031928487)),
        ((0, 0.164495299288580, 0.000038019518678), (1, 0.016875060685979, 0.004764139104512),
         (3, 0.818629640025440, 0.231114160282572)),
        ((0, 0.426933682982668, 0.000019921336144), (1, 0.157047028197878, 0.044337256156151),
         (2, 0.023164224070770, 0.006539685265423), (4, 0.392855064748685, 0.110910189373703)),
        ((0, 0.082083400476958, 0.000000034006679), (1, 0.000000039091042, 0.000000011036118),
         (2, 0.033974171137350, 0.009591531566657), (3, 0.005505195713107, 0.001554217709960),
         (5, 0.878437193581543, 0.247998929466160)),
        ((0, 0.006736365648625, 0.013159891155054), (1, 0.010581829625529, 0.002987444564164),
         (2, 0.009353386191951, 0.002640632454359), (3, 0.101886062556838, 0.028764303955070),
         (4, 0.000023428364930, 0.000006614257074), (6, 0.871418927612128, 0.246017544274548)),
        ((0, 0.071115287415749, 0.000000010647874), (1, 0.018677648343953, 0.005273042658132),
         (2, 0.007902408660034, 0.002230994887525), (3, 0.319384027162348, 0.090167968072837),
         (4, 0.007121989995845, 0.002010668386475), (5, 0.001631615692736, 0.000460635032368),
         (7, 0.574167022729334, 0.162097880203691)),
    )

    def perform_time_step(self, vec_n, vec_np, time_step, op):
        s = len(self.ROWS)
        vs = _scratch(self, "_tmp", vec_n, 2 * s - 1)
        u = [vec_n] + vs[:s - 1] + [vec_np]  # u_0 .. u_8
        k = vs[s - 1:]                       # M^-1 A(u_l), l = 0 .. 7
        for st in range(1, s + 1):
            op.apply(u[st - 1], k[st - 1])
            first = True
            for l, a, b in self.ROWS[st - 1]:
                op.vec_update(0.0 if first else 1.0, u[st], a, u[l], b * time_step, k[l])
                first = False


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
    device vector updates."""

    def perform_time_step(self, vec_n, vec_np, time_step, op):
        t1, t2 = _scratch(self, "_tmp", vec_n, 2)
        u = op.vec_update
        op.apply(vec_n, t1)
        u(0.0, vec_np, 1.0, vec_n, time_step / 6.0, t1)
        u(0.0, t2, 1.0, vec_n, 0.5 * time_step, t1)
        op.apply(t2, t1)
        u(1.0, vec_np, time_step / 3.0, t1)
        u(0.0, t2, 1.0, vec_n, 0.5 * time_step, t1)
        op.apply(t2, t1)
        u(1.0, vec_np, time_step / 3.0, t1)
        u(0.0, t2, 1.0, vec_n, time_step, t1)
        op.apply(t2, t1)
        u(1.0, vec_np, time_step / 6.0, t1)
