"""ctypes binding of libexwave_gb300.so (the C ABI in include/exwave_gb300.h).

The library is built in-tree (``python -m exwave_gb300.build``).  There is
no fallback: if the shared library cannot be loaded, every call raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libexwave_gb300.so")

EW_OK = 0
STATUS = {0: "EW_OK", -1: "EW_ERR_INVALID", -2: "EW_ERR_UNSUPPORTED", -3: "EW_ERR_CUDA",
          -4: "EW_ERR_OOM", -5: "EW_ERR_DEVICE", -6: "EW_ERR_TOO_LARGE"}
EW_PREC_FP64 = 0
EW_PREC_MIXED = 1
EW_PREC_MIXED_FF = 2
EW_MAX_DEGREE = 12

# every entry point declared in include/exwave_gb300.h
EXPORTS = ["ew_create", "ew_destroy", "ew_last_error", "ew_set_stream", "ew_n_dofs", "ew_n_cells",
           "ew_apply", "ew_rk_update", "ew_lsrk45_step", "ew_apply_ader", "ew_ader_step",
           "ew_quadrature_points", "ew_project_membrane", "ew_project_gaussian",
           "ew_l2_errors_membrane", "ew_l2_difference", "ew_hypercube_n_cells",
           "ew_hypercube_mesh", "ew_nodal_to_gauss", "ew_gauss_to_nodal", "ew_synchronize", "ew_kernel_launches",
           "ew_batch_create", "ew_batch_destroy", "ew_batch_last_error", "ew_batch_solve_bytes",
           "ew_batch_bytes_free", "ew_batch_add", "ew_batch_remove", "ew_batch_set_state",
           "ew_batch_get_state", "ew_batch_step", "ew_batch_info", "ew_batch_diverged", "ew_batch_receivers",
           "ew_batch_set_stream", "ew_batch_synchronize", "ew_batch_kernel_launches",
           "ew_tune_set", "ew_tune_get", "ew_tune_set_staging", "ew_tune_get_staging",
           "ew_lsrk45_step_static", "ew_lsrk45_steps",
           "ew_set_receivers", "ew_sample_receivers", "ew_aderadconfull_step",
           "ew_l2_error_post_membrane", "ew_lsrk_step", "ew_vec_update", "ew_check_wait_timeout",
           "ew_lsrk45_step_host", "ew_wait_host_copies"]


class EwError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (STATUS.get(code, "?"), code, msg))
        self.code = code


class MeshDesc(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int32), ("degree", ctypes.c_int32), ("n_cells", ctypes.c_int64),
                ("vertices", ctypes.POINTER(ctypes.c_double)),
                ("neighbors", ctypes.POINTER(ctypes.c_int32)),
                ("speed", ctypes.POINTER(ctypes.c_double)),
                ("density", ctypes.POINTER(ctypes.c_double))]


class Options(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int32), ("use_ader_post", ctypes.c_int32),
                ("spectral_evaluation", ctypes.c_int32), ("cells_per_block", ctypes.c_int32),
                ("device", ctypes.c_int32), ("nb_staging", ctypes.c_int32)]


class HypercubeDesc(ctypes.Structure):
    _fields_ = [("dim", ctypes.c_int32), ("n_intervals", ctypes.c_int32),
                ("n_refinements", ctypes.c_int32), ("transform", ctypes.c_int32),
                ("transform_factor", ctypes.c_double), ("boundary_ids", ctypes.c_int32 * 6)]


_lib = None


def load():
    """Load the shared library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libexwave_gb300.so not built: run python -m exwave_gb300.build "
                           "(or __graft_entry__.build())")
    L = ctypes.CDLL(LIB_PATH)
    vp, dp, i32p = ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p
    d, i32, i64 = ctypes.c_double, ctypes.c_int32, ctypes.c_int64
    sig = {
        "ew_create": (ctypes.c_int, [ctypes.POINTER(MeshDesc), ctypes.POINTER(Options),
                                     ctypes.POINTER(ctypes.c_void_p)]),
        "ew_destroy": (None, [vp]),
        "ew_last_error": (ctypes.c_char_p, [vp]),
        "ew_set_stream": (ctypes.c_int, [vp, vp]),
        "ew_n_dofs": (i64, [vp]),
        "ew_n_cells": (i64, [vp]),
        "ew_apply": (ctypes.c_int, [vp, dp, dp]),
        "ew_rk_update": (ctypes.c_int, [vp, d, d, i32, dp, dp, dp]),
        "ew_lsrk45_step": (ctypes.c_int, [vp, d, dp, dp]),
        "ew_lsrk45_step_static": (ctypes.c_int, [vp, d, dp, dp]),
        "ew_lsrk45_step_host": (ctypes.c_int, [vp, d, vp, vp]),
        "ew_wait_host_copies": (ctypes.c_int, [vp]),
        "ew_lsrk45_steps": (ctypes.c_int, [vp, d, i64, dp, dp]),
        "ew_set_receivers": (ctypes.c_int, [vp, i32, dp]),
        "ew_aderadconfull_step": (ctypes.c_int, [vp, d, dp, dp]),
        "ew_sample_receivers": (ctypes.c_int, [vp, dp, dp]),
        "ew_apply_ader": (ctypes.c_int, [vp, d, dp, dp]),
        "ew_ader_step": (ctypes.c_int, [vp, d, dp, dp]),
        "ew_quadrature_points": (ctypes.c_int, [vp, dp]),
        "ew_project_membrane": (ctypes.c_int, [vp, i32, dp, i32p, d, dp]),
        "ew_project_gaussian": (ctypes.c_int, [vp, dp, d, d, dp]),
        "ew_l2_errors_membrane": (ctypes.c_int, [vp, dp, i32, dp, i32p, d, dp]),
        "ew_l2_error_post_membrane": (ctypes.c_int, [vp, dp, i32, dp, i32p, d, dp]),
        "ew_lsrk_step": (ctypes.c_int, [vp, i32, d, dp, dp]),
        "ew_vec_update": (ctypes.c_int, [vp, d, dp, d, dp, d, dp]),
        "ew_l2_difference": (ctypes.c_int, [vp, dp, dp, dp]),
        "ew_hypercube_n_cells": (i64, [ctypes.POINTER(HypercubeDesc)]),
        "ew_hypercube_mesh": (ctypes.c_int, [ctypes.POINTER(HypercubeDesc), dp, i32p]),
        "ew_nodal_to_gauss": (ctypes.c_int, [i32, i32, i64, i32, dp, dp, dp]),
        "ew_gauss_to_nodal": (ctypes.c_int, [i32, i32, i64, i32, dp, dp, dp]),
        "ew_synchronize": (ctypes.c_int, [vp]),
        "ew_check_wait_timeout": (ctypes.c_int, [vp, ctypes.c_int32]),
        "ew_kernel_launches": (i64, [vp]),
        "ew_tune_set": (ctypes.c_int, [i32, i32, i32, i32]),
        "ew_tune_get": (i32, [i32, i32, i32]),
        "ew_tune_set_staging": (ctypes.c_int, [i32, i32, i32, i32]),
        "ew_tune_get_staging": (i32, [i32, i32, i32]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    _apply_tuning(L)
    return L


def _apply_tuning(L):
    """Load the tuned cells-per-block table of this GPU model, if any."""
    import json
    path = os.path.join(HERE, "tuning", "tuning.json")
    if not os.path.exists(path):
        return
    try:
        with open(path) as f:
            table = json.load(f)
    except (OSError, ValueError):
        return
    for e in table.get("entries", []):
        prec = {"fp64": 0, "mixed": 1, "mixed_ff": 2}[e["precision"]]
        L.ew_tune_set(int(e["dim"]), int(e["degree"]), prec, int(e["cells_per_block"]))
        L.ew_tune_set_staging(int(e["dim"]), int(e["degree"]), prec, int(e.get("nb_staging", 0)))


def check(rc, ctx=None):
    if rc != EW_OK:
        msg = load().ew_last_error(ctx)
        raise EwError(rc, msg.decode() if msg else "")
