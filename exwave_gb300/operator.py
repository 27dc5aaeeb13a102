"""WaveEquationOperation on the GPU: the host-side mirror of the reference's
``WaveEquationOperationBase<dim>`` (wave_equation_operations.h:56-98) over
the C ABI.  Vectors are FP64 CUDA tensors in the canonical layout
[cell][field][Gauss point] (fields u_0..u_{d-1}, p).
"""
import ctypes

import numpy as np

from . import _lib

PRECISIONS = {"fp64": _lib.EW_PREC_FP64, "mixed": _lib.EW_PREC_MIXED,
              "mixed_ff": _lib.EW_PREC_MIXED_FF}


def _ptr(t):
    if t is None:
        return None
    if not (t.is_cuda and t.is_contiguous()):
        raise ValueError("expected a contiguous CUDA tensor")
    return ctypes.c_void_p(t.data_ptr())


def _modes(amps, kvecs):
    amps = np.ascontiguousarray(amps, dtype=np.float64)
    kv = np.zeros((len(amps), 3), dtype=np.int32)
    kv[:, :len(kvecs[0])] = np.asarray(kvecs, dtype=np.int32)
    return amps, kv


class WaveEquationOperation:
    """Operator of one solve: ``apply`` (RK), ``apply_ader`` (ADER), the
    fused integrator steps, initial fields and L2 errors.

    precision: "fp64" (the reference's arithmetic), "mixed" (FP32 operator,
    FP64 state) or "mixed_ff" (compensated: float-float operator on
    float-pair data, equal to the FP64 path to about 1e-14; every mesh and
    integrator, ADER included)."""

    def __init__(self, mesh, degree, precision="fp64", use_ader_post=False, cells_per_block=0,
                 device=0, spectral_evaluation=True, nb_staging=0):
        import torch
        self.torch = torch
        self.L = _lib.load()
        self.mesh = mesh
        self.dim = mesh.dim
        self.degree = degree
        self.precision = precision
        self.use_ader_post = bool(use_ader_post)
        self.device = device
        self._keep = [np.ascontiguousarray(mesh.vertices, np.float64),
                      np.ascontiguousarray(mesh.neighbors, np.int32),
                      np.ascontiguousarray(mesh.speed, np.float64),
                      np.ascontiguousarray(mesh.density, np.float64)]
        md = _lib.MeshDesc()
        md.dim = mesh.dim
        md.degree = degree
        md.n_cells = mesh.n_cells
        md.vertices = self._keep[0].ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        md.neighbors = self._keep[1].ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
        md.speed = self._keep[2].ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        md.density = self._keep[3].ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        op = _lib.Options()
        op.precision = PRECISIONS[precision]
        op.use_ader_post = int(self.use_ader_post)
        op.spectral_evaluation = int(bool(spectral_evaluation))
        op.cells_per_block = cells_per_block
        op.nb_staging = nb_staging
        op.device = device
        h = ctypes.c_void_p()
        _lib.check(self.L.ew_create(ctypes.byref(md), ctypes.byref(op), ctypes.byref(h)))
        self.ctx = h
        self.n_dofs = self.L.ew_n_dofs(h)
        self.n_cells = mesh.n_cells
        self.points = (degree + 1) ** mesh.dim

    def Name(self):
        return "ADER" if self.use_ader_post else "Runge-Kutta"

    def close(self):
        if getattr(self, "ctx", None):
            self.L.ew_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, rc):
        _lib.check(rc, self.ctx)

    def set_stream(self, stream):
        self._chk(self.L.ew_set_stream(self.ctx, ctypes.c_void_p(stream.cuda_stream)))

    def new_vector(self):
        return self.torch.zeros(self.n_dofs, dtype=self.torch.float64,
                                device="cuda:%d" % self.device)

    # -- reference interface -------------------------------------------
    def apply(self, src, dst):
        self._chk(self.L.ew_apply(self.ctx, _ptr(src), _ptr(dst)))

    def apply_ader(self, src, dst, dt):
        self._chk(self.L.ew_apply_ader(self.ctx, dt, _ptr(src), _ptr(dst)))

    def rk_update(self, f1, f2, is_last, v1, v2, v3):
        self._chk(self.L.ew_rk_update(self.ctx, f1, f2, int(is_last), _ptr(v1), _ptr(v2), _ptr(v3)))

    def lsrk45_step(self, dt, vec_n, vec_np):
        self._chk(self.L.ew_lsrk45_step(self.ctx, dt, _ptr(vec_n), _ptr(vec_np)))

    def lsrk45_step_host(self, dt, host_n, host_np):
        """One LSRK45 step on host (CPU) float64 tensors, pinned for
        asynchronous copies; host_n and host_np may be the same tensor.  The
        copies overlap with those of the previous call when its output is
        this call's input.  host_np is complete after synchronize(), or on
        the context stream after wait_host_copies()."""
        for t in (host_n, host_np):
            if t.is_cuda or not t.is_contiguous() or t.dtype != self.torch.float64 or t.numel() != self.n_dofs:
                raise ValueError("expected contiguous float64 host tensors of n_dofs entries")
        self._chk(self.L.ew_lsrk45_step_host(self.ctx, dt, ctypes.c_void_p(host_n.data_ptr()),
                                             ctypes.c_void_p(host_np.data_ptr())))

    def wait_host_copies(self):
        """Orders the context stream after the last host step's copies to the host."""
        self._chk(self.L.ew_wait_host_copies(self.ctx))

    LSRK_SCHEMES = {"LSRK33R2": 0, "LSRK45R2": 1, "LSRK59R2": 2}

    def lsrk_step(self, scheme, dt, vec_n, vec_np):
        """One step of a low-storage 2-register scheme (LSRK33R2, LSRK45R2, LSRK59R2)."""
        self._chk(self.L.ew_lsrk_step(self.ctx, self.LSRK_SCHEMES[scheme], dt, _ptr(vec_n),
                                      _ptr(vec_np)))

    def vec_update(self, alpha, y, beta=0.0, x=None, gamma=0.0, z=None):
        """y = alpha*y + (beta*x + gamma*z) on the device (x or z None: term dropped)."""
        self._chk(self.L.ew_vec_update(self.ctx, alpha, _ptr(y), beta,
                                       None if x is None else _ptr(x), gamma,
                                       None if z is None else _ptr(z)))

    def lsrk45_steps(self, dt, n_steps, vec_n, vec_np):
        """n_steps LSRK45 steps in one call (vec_n in, clobbered; vec_np out)."""
        self._chk(self.L.ew_lsrk45_steps(self.ctx, dt, int(n_steps), _ptr(vec_n), _ptr(vec_np)))

    def set_receivers(self, points):
        """Locate receiver points (array n x dim) once."""
        p = np.ascontiguousarray(np.asarray(points, dtype=np.float64).reshape(-1, self.dim))
        self._chk(self.L.ew_set_receivers(self.ctx, p.shape[0], p.ctypes.data))
        self.n_receivers = p.shape[0]

    def sample_receivers(self, state, out=None):
        """Fields at the receivers: a (n, dim + 1) device tensor (or a view of
        `out`, e.g. one row of a preallocated trace)."""
        if out is None:
            out = self.torch.zeros(self.n_receivers * (self.dim + 1), dtype=self.torch.float64,
                                   device="cuda:%d" % self.device)
        self._chk(self.L.ew_sample_receivers(self.ctx, _ptr(state), _ptr(out)))
        return out.view(self.n_receivers, self.dim + 1)

    def aderadconfull_step(self, dt, vec_n, vec_np):
        self._chk(self.L.ew_aderadconfull_step(self.ctx, dt, _ptr(vec_n), _ptr(vec_np)))

    def ader_step(self, dt, vec_n, vec_np):
        self._chk(self.L.ew_ader_step(self.ctx, dt, _ptr(vec_n), _ptr(vec_np)))

    def quadrature_points(self):
        out = self.torch.zeros(self.n_cells * self.points * self.dim, dtype=self.torch.float64,
                               device="cuda:%d" % self.device)
        self._chk(self.L.ew_quadrature_points(self.ctx, _ptr(out)))
        return out.view(self.n_cells, self.points, self.dim)

    def project_membrane(self, amps, kvecs, t=0.0, out=None):
        a, kv = _modes(amps, kvecs)
        out = self.new_vector() if out is None else out
        self._chk(self.L.ew_project_membrane(self.ctx, len(a), a.ctypes.data, kv.ctypes.data, t,
                                             _ptr(out)))
        return out

    def project_gaussian(self, x0, width, amp=1.0, out=None):
        c = np.zeros(3)
        c[:len(x0)] = x0
        out = self.new_vector() if out is None else out
        self._chk(self.L.ew_project_gaussian(self.ctx, c.ctypes.data, width, amp, _ptr(out)))
        return out

    def l2_errors(self, u, amps, kvecs, t):
        a, kv = _modes(amps, kvecs)
        out = np.zeros(3)
        self._chk(self.L.ew_l2_errors_membrane(self.ctx, _ptr(u), len(a), a.ctypes.data,
                                               kv.ctypes.data, t, out.ctypes.data))
        return out

    def l2_error_post(self, u, amps, kvecs, t):
        """L2 error of the post-processed pressure of degree k+1 (compute_post_pressure,
        wave_equation_operations.cc:784-848; explicit_wave.cc:476-484)."""
        a, kv = _modes(amps, kvecs)
        out = np.zeros(1)
        self._chk(self.L.ew_l2_error_post_membrane(self.ctx, _ptr(u), len(a), a.ctypes.data,
                                                   kv.ctypes.data, t, out.ctypes.data))
        return float(out[0])

    def l2_difference(self, a, b):
        out = np.zeros(2)
        self._chk(self.L.ew_l2_difference(self.ctx, _ptr(a), _ptr(b), out.ctypes.data))
        return out

    def synchronize(self):
        self._chk(self.L.ew_synchronize(self.ctx))

    def kernel_launches(self):
        return self.L.ew_kernel_launches(self.ctx)


def reference_mode(dim, m):
    """The reference's single membrane mode (input_parameters.h:95-128): wave
    number m in every direction, unit amplitude."""
    return [1.0], [[m] * dim]
