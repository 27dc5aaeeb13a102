"""Batched solves: many independent simulations (uneven degree, mesh size,
material, source, receivers) resident on one GPU and stepped together by
persistent per-degree launches (``ew_batch_*`` in the C ABI)."""
import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import _lib


class SourceDesc(ctypes.Structure):
    _fields_ = [("position", ctypes.c_double * 3), ("frequency", ctypes.c_double),
                ("delay", ctypes.c_double), ("amplitude", ctypes.c_double)]


class SolveDesc(ctypes.Structure):
    _fields_ = [("mesh", _lib.MeshDesc), ("dt", ctypes.c_double), ("n_steps", ctypes.c_int64),
                ("n_sources", ctypes.c_int32), ("source", SourceDesc),
                ("n_receivers", ctypes.c_int32), ("receivers", ctypes.c_void_p)]


class BatchOptions(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int32), ("device", ctypes.c_int32),
                ("hbm_budget_bytes", ctypes.c_int64), ("max_solves", ctypes.c_int32),
                ("use_graphs", ctypes.c_int32), ("allow_overrun", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("blowup_limit", ctypes.c_double)]


_SIG = {
    "ew_batch_create": (ctypes.c_int, [ctypes.POINTER(BatchOptions), ctypes.POINTER(ctypes.c_void_p)]),
    "ew_batch_destroy": (None, [ctypes.c_void_p]),
    "ew_batch_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "ew_batch_solve_bytes": (ctypes.c_int64, [ctypes.c_void_p, ctypes.POINTER(SolveDesc)]),
    "ew_batch_bytes_free": (ctypes.c_int64, [ctypes.c_void_p]),
    "ew_batch_add": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(SolveDesc),
                                    ctypes.POINTER(ctypes.c_int32)]),
    "ew_batch_remove": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "ew_batch_set_state": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p]),
    "ew_batch_get_state": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p]),
    "ew_batch_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "ew_batch_info": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32,
                                     ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]),
    "ew_batch_diverged": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32), ctypes.c_int32,
                                         ctypes.POINTER(ctypes.c_int32)]),
    "ew_batch_receivers": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64,
                                          ctypes.c_int64, ctypes.c_void_p]),
    "ew_batch_set_stream": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "ew_batch_synchronize": (ctypes.c_int, [ctypes.c_void_p]),
    "ew_batch_kernel_launches": (ctypes.c_int64, [ctypes.c_void_p]),
}


def _L():
    L = _lib.load()
    if not getattr(L, "_batch_sig", False):
        for name, (res, args) in _SIG.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        L._batch_sig = True
    return L


@dataclass
class Solve:
    """One simulation: mesh, degree, time step, number of steps, optional
    Ricker source (position, f0, delay, amplitude) and receiver points."""
    mesh: object
    degree: int
    dt: float
    n_steps: int
    source: tuple = None            # (position, f0, delay, amplitude)
    receivers: np.ndarray = None    # (n, dim)
    keep: list = field(default_factory=list)

    def desc(self):
        m = self.mesh
        arrs = [np.ascontiguousarray(m.vertices, np.float64), np.ascontiguousarray(m.neighbors, np.int32),
                np.ascontiguousarray(m.speed, np.float64), np.ascontiguousarray(m.density, np.float64)]
        d = SolveDesc()
        d.mesh.dim = m.dim
        d.mesh.degree = self.degree
        d.mesh.n_cells = m.n_cells
        d.mesh.vertices = arrs[0].ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        d.mesh.neighbors = arrs[1].ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
        d.mesh.speed = arrs[2].ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        d.mesh.density = arrs[3].ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        d.dt = self.dt
        d.n_steps = self.n_steps
        if self.source is not None:
            pos, f0, delay, amp = self.source
            d.n_sources = 1
            for i in range(len(pos)):
                d.source.position[i] = pos[i]
            d.source.frequency = f0
            d.source.delay = delay
            d.source.amplitude = amp
        rec = None
        if self.receivers is not None and len(self.receivers):
            rec = np.ascontiguousarray(self.receivers, np.float64)
            d.n_receivers = rec.shape[0]
            d.receivers = rec.ctypes.data
        self.keep = arrs + ([rec] if rec is not None else [])
        return d


class Batch:
    """Device-resident set of solves advanced together."""

    def __init__(self, precision="mixed", hbm_budget_bytes=8 << 30, max_solves=4096,
                 use_graphs=True, device=0, allow_overrun=False, blowup_limit=0.0):
        self.L = _L()
        o = BatchOptions()
        o.precision = {"fp64": _lib.EW_PREC_FP64, "mixed": _lib.EW_PREC_MIXED,
                       "mixed_ff": _lib.EW_PREC_MIXED_FF}[precision]
        o.device = device
        o.hbm_budget_bytes = int(hbm_budget_bytes)
        o.max_solves = max_solves
        o.use_graphs = int(bool(use_graphs))
        o.allow_overrun = int(bool(allow_overrun))
        o.blowup_limit = float(blowup_limit)
        h = ctypes.c_void_p()
        rc = self.L.ew_batch_create(ctypes.byref(o), ctypes.byref(h))
        if rc != 0:
            raise _lib.EwError(rc, "ew_batch_create failed")
        self.h = h
        self.precision = precision
        self.solves = {}

    def _chk(self, rc):
        if rc != 0:
            msg = self.L.ew_batch_last_error(self.h)
            raise _lib.EwError(rc, msg.decode() if msg else "")

    def close(self):
        if getattr(self, "h", None):
            self.L.ew_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def solve_bytes(self, solve):
        return self.L.ew_batch_solve_bytes(self.h, ctypes.byref(solve.desc()))

    def bytes_free(self):
        return self.L.ew_batch_bytes_free(self.h)

    def add(self, solve):
        """Admit a solve; raises EwError (EW_ERR_OOM) when over budget."""
        d = solve.desc()
        sid = ctypes.c_int32()
        self._chk(self.L.ew_batch_add(self.h, ctypes.byref(d), ctypes.byref(sid)))
        self.solves[sid.value] = solve
        return sid.value

    def remove(self, sid):
        self._chk(self.L.ew_batch_remove(self.h, sid))
        self.solves.pop(sid, None)

    def set_state(self, sid, state):
        self._chk(self.L.ew_batch_set_state(self.h, sid, ctypes.c_void_p(state.data_ptr())))

    def get_state(self, sid, out):
        self._chk(self.L.ew_batch_get_state(self.h, sid, ctypes.c_void_p(out.data_ptr())))
        return out

    def step(self, n=1):
        self._chk(self.L.ew_batch_step(self.h, n))

    def info(self, sid):
        a, b = ctypes.c_int64(), ctypes.c_int64()
        self._chk(self.L.ew_batch_info(self.h, sid, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def steps_left(self):
        left = [b - a for a, b in (self.info(s) for s in self.solves)]
        left = [x for x in left if x > 0]
        return min(left) if left else 0

    def diverged(self):
        """Ids of the solves whose receiver samples went non-finite or past
        the blow-up limit (waits for the batch's stream)."""
        cap = max(1, len(self.solves))
        ids = (ctypes.c_int32 * cap)()
        n = ctypes.c_int32()
        self._chk(self.L.ew_batch_diverged(self.h, ids, cap, ctypes.byref(n)))
        return [ids[i] for i in range(n.value)]

    def receivers(self, sid, first=0, count=None):
        done, _ = self.info(sid)
        count = done - first if count is None else count
        s = self.solves[sid]
        nrec = 0 if s.receivers is None else len(s.receivers)
        out = np.zeros((count, max(nrec, 1)))
        self._chk(self.L.ew_batch_receivers(self.h, sid, first, count, out.ctypes.data))
        return out[:, :nrec]

    def set_stream(self, stream):
        self._chk(self.L.ew_batch_set_stream(self.h, ctypes.c_void_p(stream.cuda_stream)))

    def synchronize(self):
        self._chk(self.L.ew_batch_synchronize(self.h))

    def kernel_launches(self):
        return self.L.ew_batch_kernel_launches(self.h)
