"""ctypes wrapper of the CPU oracle (test infrastructure only).

The oracle restates the reference's hot-path arithmetic in plain FP64 C++
(``ew_oracle.cpp``).  Only the test-suite, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` import this module; the product package never
does.  ``build()`` compiles the shared library with the Makefile next to it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libew_oracle.so")

INTEGRATORS = {"LSRK45R2": 0, "clRK4": 1, "ADER": 2, "ADERADCONFULL": 3, "ExplEuler": 4,
               "LSRK33R2": 5, "LSRK45R3": 6, "LSRK59R2": 7, "SSPRK": 8}
# one step of each integrator: the oracle's entry point
STEP_FUNCS = {"LSRK45R2": "ewo_lsrk45_step", "clRK4": "ewo_clrk4_step", "ADER": "ewo_ader_step",
              "ADERADCONFULL": "ewo_aderadconfull_step", "ExplEuler": "ewo_expleuler_step",
              "LSRK33R2": "ewo_lsrk33_step", "LSRK45R3": "ewo_lsrk45r3_step",
              "LSRK59R2": "ewo_lsrk59_step", "SSPRK": "ewo_ssprk_step"}

_lib = None


def build(quiet=True):
    """Compile the oracle library (idempotent)."""
    out = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        i32p = ctypes.POINTER(ctypes.c_int32)
        L.ewo_create.restype = P
        L.ewo_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int64, dp, i32p, dp, dp]
        L.ewo_create_hypercube.restype = P
        L.ewo_create_hypercube.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_double, ctypes.c_int]
        L.ewo_destroy.argtypes = [P]
        L.ewo_n_cells.restype = ctypes.c_int64
        L.ewo_n_cells.argtypes = [P]
        L.ewo_n_dofs.restype = ctypes.c_int64
        L.ewo_n_dofs.argtypes = [P]
        L.ewo_vertices.restype = dp
        L.ewo_vertices.argtypes = [P]
        L.ewo_neighbors.restype = i32p
        L.ewo_neighbors.argtypes = [P]
        L.ewo_set_ader_post.argtypes = [P, ctypes.c_int]
        L.ewo_set_spectral.argtypes = [P, ctypes.c_int]
        L.ewo_time_step.restype = ctypes.c_double
        L.ewo_time_step.argtypes = [P, ctypes.c_double]
        L.ewo_quadrature_points.argtypes = [P, dp]
        L.ewo_project_reference.argtypes = [P, ctypes.c_int, ctypes.c_double, dp]
        L.ewo_project_modes.argtypes = [P, ctypes.c_int, dp, ip, ctypes.c_double, dp]
        L.ewo_project_gaussian.argtypes = [P, dp, ctypes.c_double, ctypes.c_double, dp]
        L.ewo_apply.argtypes = [P, dp, dp, ctypes.c_double]
        L.ewo_rk_update.argtypes = [ctypes.c_int64, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                    dp, dp, dp]
        for name in tuple(STEP_FUNCS.values()) + ("ewo_ader_taylor", "ewo_apply_ader"):
            getattr(L, name).argtypes = [P, ctypes.c_double, dp, dp]
        L.ewo_errors_reference.argtypes = [P, dp, ctypes.c_int, ctypes.c_double, dp]
        L.ewo_errors_modes.argtypes = [P, dp, ctypes.c_int, dp, ip, ctypes.c_double, dp]
        L.ewo_run_reference.restype = ctypes.c_int
        L.ewo_run_reference.argtypes = [P, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_int, ctypes.c_int, dp,
                                        ctypes.c_int, dp]
        L.ewo_post_error_reference.restype = ctypes.c_double
        L.ewo_post_error_reference.argtypes = [P, dp, ctypes.c_int, ctypes.c_double]
        L.ewo_point_values.restype = ctypes.c_int
        L.ewo_point_values.argtypes = [P, dp, ctypes.c_int, dp, dp]
        L.ewo_lsrk45_step_source.restype = ctypes.c_int
        L.ewo_lsrk45_step_source.argtypes = [P, ctypes.c_double, ctypes.c_double, dp, dp, dp,
                                             ctypes.c_double, ctypes.c_double, ctypes.c_double]
        L.ewo_last_error.restype = ctypes.c_char_p
        L.ewo_num_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Problem:
    """An oracle operator over one mesh: the CPU restatement of
    WaveEquationOperation<dim,k> plus its integrators."""

    def __init__(self, handle, dim, degree):
        if not handle:
            raise RuntimeError(lib().ewo_last_error().decode())
        self.h = handle
        self.dim = dim
        self.degree = degree
        self.n_cells = lib().ewo_n_cells(handle)
        self.n_dofs = lib().ewo_n_dofs(handle)

    @classmethod
    def hypercube(cls, dim, degree, n_intervals, n_refinements=0, transform=0.0, boundary_id=2):
        h = lib().ewo_create_hypercube(dim, degree, n_intervals, n_refinements, transform,
                                       boundary_id)
        return cls(h, dim, degree)

    @classmethod
    def from_mesh(cls, dim, degree, vertices, neighbors, speed, density):
        vertices = np.ascontiguousarray(vertices, dtype=np.float64)
        neighbors = np.ascontiguousarray(neighbors, dtype=np.int32)
        speed = np.ascontiguousarray(speed, dtype=np.float64)
        density = np.ascontiguousarray(density, dtype=np.float64)
        n_cells = speed.shape[0]
        h = lib().ewo_create(dim, degree, n_cells, _dp(vertices),
                             neighbors.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                             _dp(speed), _dp(density))
        return cls(h, dim, degree)

    def __del__(self):
        if getattr(self, "h", None):
            lib().ewo_destroy(self.h)
            self.h = None

    def vertices(self):
        nv = (1 << self.dim) * self.dim
        p = lib().ewo_vertices(self.h)
        return np.ctypeslib.as_array(p, shape=(self.n_cells * nv,)).copy().reshape(
            self.n_cells, 1 << self.dim, self.dim)

    def neighbors(self):
        p = lib().ewo_neighbors(self.h)
        return np.ctypeslib.as_array(p, shape=(self.n_cells * 2 * self.dim,)).copy().reshape(
            self.n_cells, 2 * self.dim)

    def set_ader_post(self, on):
        lib().ewo_set_ader_post(self.h, int(bool(on)))

    def set_spectral(self, on):
        """ADER with (the default) or without spectral evaluation."""
        lib().ewo_set_spectral(self.h, int(bool(on)))

    def time_step(self, cfl_scaled):
        return lib().ewo_time_step(self.h, cfl_scaled)

    def zeros(self):
        return np.zeros(self.n_dofs, dtype=np.float64)

    def project_reference(self, modes, t=0.0):
        u = self.zeros()
        lib().ewo_project_reference(self.h, modes, t, _dp(u))
        return u

    def project_modes(self, amps, kvecs, t=0.0):
        amps = np.ascontiguousarray(amps, dtype=np.float64)
        kv = np.zeros((len(amps), 3), dtype=np.int32)
        kv[:, :len(kvecs[0])] = np.asarray(kvecs)
        u = self.zeros()
        lib().ewo_project_modes(self.h, len(amps), _dp(amps),
                                kv.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), t, _dp(u))
        return u

    def quadrature_points(self):
        """Physical coordinates of every Gauss point, (n_cells, N, dim)."""
        xyz = np.zeros(self.n_dofs // (self.dim + 1) * self.dim)
        lib().ewo_quadrature_points(self.h, _dp(xyz))
        return xyz.reshape(-1, (self.degree + 1) ** self.dim, self.dim)

    def project_gaussian(self, x0, width, amp=1.0):
        c = np.zeros(3)
        c[:len(x0)] = x0
        u = self.zeros()
        lib().ewo_project_gaussian(self.h, _dp(c), width, amp, _dp(u))
        return u

    def apply(self, src, boundary_fac=1.0):
        src = np.ascontiguousarray(src, dtype=np.float64)
        dst = self.zeros()
        lib().ewo_apply(self.h, _dp(src), _dp(dst), boundary_fac)
        return dst

    def lsrk45_step(self, dt, vec_n, vec_np):
        lib().ewo_lsrk45_step(self.h, dt, _dp(vec_n), _dp(vec_np))

    def clrk4_step(self, dt, vec_n, vec_np):
        lib().ewo_clrk4_step(self.h, dt, _dp(vec_n), _dp(vec_np))

    def step(self, integrator, dt, vec_n, vec_np):
        """One perform_time_step of the named integrator (vec_n may be clobbered)."""
        getattr(lib(), STEP_FUNCS[integrator])(self.h, dt, _dp(vec_n), _dp(vec_np))

    def ader_step(self, dt, vec_n, vec_np):
        lib().ewo_ader_step(self.h, dt, _dp(vec_n), _dp(vec_np))

    def aderadconfull_step(self, dt, vec_n, vec_np):
        lib().ewo_aderadconfull_step(self.h, dt, _dp(vec_n), _dp(vec_np))

    def ader_taylor(self, dt, src):
        src = np.ascontiguousarray(src, dtype=np.float64)
        T = self.zeros()
        lib().ewo_ader_taylor(self.h, dt, _dp(src), _dp(T))
        return T

    def apply_ader(self, dt, src):
        src = np.ascontiguousarray(src, dtype=np.float64)
        dst = self.zeros()
        lib().ewo_apply_ader(self.h, dt, _dp(src), _dp(dst))
        return dst

    def errors_reference(self, u, modes, t):
        out = np.zeros(3)
        lib().ewo_errors_reference(self.h, _dp(np.ascontiguousarray(u)), modes, t, _dp(out))
        return out

    def post_error_reference(self, u, modes, t):
        return lib().ewo_post_error_reference(self.h, _dp(np.ascontiguousarray(u)), modes, t)

    def errors_modes(self, u, amps, kvecs, t):
        amps = np.ascontiguousarray(amps, dtype=np.float64)
        kv = np.zeros((len(amps), 3), dtype=np.int32)
        kv[:, :len(kvecs[0])] = np.asarray(kvecs)
        out = np.zeros(3)
        lib().ewo_errors_modes(self.h, _dp(np.ascontiguousarray(u)), len(amps), _dp(amps),
                               kv.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), t, _dp(out))
        return out

    def point_values(self, u, points):
        pts = np.ascontiguousarray(points, dtype=np.float64)
        out = np.zeros(pts.shape[0])
        if lib().ewo_point_values(self.h, _dp(np.ascontiguousarray(u)), pts.shape[0], _dp(pts),
                                  _dp(out)) != 0:
            raise RuntimeError(lib().ewo_last_error().decode())
        return out

    def lsrk45_step_source(self, dt, t, vec_n, vec_np, xs, amp, f0, delay):
        x = np.zeros(3)
        x[:len(xs)] = xs
        if lib().ewo_lsrk45_step_source(self.h, dt, t, _dp(vec_n), _dp(vec_np), _dp(x), amp, f0,
                                        delay) != 0:
            raise RuntimeError(lib().ewo_last_error().decode())

    def run_reference(self, integrator, cfl, final_time, tick, modes, max_time_steps=1000000):
        rows = np.zeros((4096, 6))  # time, step, err p, err v, |p|, err p post
        dt = np.zeros(1)
        nr = lib().ewo_run_reference(self.h, INTEGRATORS[integrator], cfl, final_time, tick, modes,
                                     max_time_steps, _dp(rows), rows.shape[0], _dp(dt))
        if nr < 0:
            raise RuntimeError(lib().ewo_last_error().decode())
        return rows[:nr].copy(), float(dt[0])


def gauss_data(np_):
    """1-D Gauss-Legendre data on [0, 1]: points, weights, the derivative
    matrix D[i, j] = l_j'(x_i) of the Lagrange basis on the points, and the
    traces l_j(0), l_j(1)."""
    x, w = np.polynomial.legendre.leggauss(np_)
    x, w = 0.5 * (x + 1.0), 0.5 * w
    D = np.zeros((np_, np_))
    L0, L1 = np.ones(np_), np.ones(np_)
    for j in range(np_):
        others = [m for m in range(np_) if m != j]
        den = np.prod([x[j] - x[m] for m in others])
        L0[j] = np.prod([0.0 - x[m] for m in others]) / den
        L1[j] = np.prod([1.0 - x[m] for m in others]) / den
        for i in range(np_):
            s = 0.0
            for a in others:
                s += np.prod([x[i] - x[m] for m in others if m != a])
            D[i, j] = s / den
    return x, w, D, L0, L1


class CartCPU:
    """CPU baseline for axis-aligned meshes (``ew_cpu_cart.cpp``): the same
    operator and LSRK45 step as the oracle in the line form, OpenMP over
    cells; timed by ``bench.py``'s CPU legs and checked against ``Problem``
    by the tests."""

    def __init__(self, dim, degree, vertices, neighbors, speed, density):
        L = lib()
        P = ctypes.c_void_p
        dp = ctypes.POINTER(ctypes.c_double)
        L.ewc_create.restype = P
        L.ewc_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int64, dp,
                                 ctypes.POINTER(ctypes.c_int32), dp, dp, dp, dp, dp, dp]
        L.ewc_destroy.argtypes = [P]
        L.ewc_apply.argtypes = [P, dp, dp]
        L.ewc_lsrk45_step.argtypes = [P, ctypes.c_double, dp, dp, dp]
        np_ = degree + 1
        _, w, D, L0, L1 = gauss_data(np_)
        self.keep = [np.ascontiguousarray(a, dtype=np.float64) for a in (vertices, speed, density)]
        self.keep.append(np.ascontiguousarray(neighbors, dtype=np.int32))
        self.keep += [np.ascontiguousarray(a, dtype=np.float64) for a in (w, D, L0, L1)]
        v, sp, de, nb, w_, D_, L0_, L1_ = self.keep
        self.n_cells = sp.shape[0]
        self.n_dofs = self.n_cells * (dim + 1) * np_ ** dim
        self.h = L.ewc_create(dim, np_, self.n_cells, _dp(v),
                              nb.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), _dp(sp), _dp(de),
                              _dp(w_), _dp(D_), _dp(L0_), _dp(L1_))
        if not self.h:
            raise RuntimeError("CartCPU: not an axis-aligned mesh or unsupported degree")
        self.tmp = np.zeros(self.n_dofs)

    def __del__(self):
        if getattr(self, "h", None):
            lib().ewc_destroy(self.h)
            self.h = None

    def apply(self, src):
        dst = np.zeros_like(src)
        lib().ewc_apply(self.h, _dp(src), _dp(dst))
        return dst

    def lsrk45_step(self, dt, vec_n, vec_np):
        lib().ewc_lsrk45_step(self.h, dt, _dp(vec_n), _dp(vec_np), _dp(self.tmp))


def num_threads():
    return lib().ewo_num_threads()
