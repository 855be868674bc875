"""ctypes binding of ``libsps_gb300.so`` (C ABI in ``include/sps_pdhg.h``).

The library is built in-tree by ``_build.build()``.  Loading fails loudly when
it is missing: there is no CPU fallback on this path.
"""

from __future__ import annotations

import ctypes as C
import os

from . import _build

_i32p = C.POINTER(C.c_int32)
_f64p = C.POINTER(C.c_double)
_f32p = C.POINTER(C.c_float)

ERRORS = {
    -1: "SPS_ERR_INVALID",
    -2: "SPS_ERR_CUDA",
    -3: "SPS_ERR_OOM",
    -4: "SPS_ERR_STATE",
    -5: "SPS_ERR_TIMEOUT",
}
STATUS = {0: "optimal", 1: "iteration_limit", 2: "time_limit", 3: "numeric_error", 4: "stalled",
          5: "infeasible", 6: "unbounded"}
ESCALATE = {"off": 0, "fp64": 1, "stop": 2}
MODES = {"reference": 0, "adaptive": 1}
PRECISIONS = {"fp32": 0, "fp64": 1}
KKT_FORMS = {"lagrangian": 0, "pdlp": 1}


class ProblemDesc(C.Structure):
    _fields_ = [
        ("n", C.c_int32), ("m_ub", C.c_int32), ("m_eq", C.c_int32),
        ("ub_indptr", _i32p), ("ub_indices", _i32p), ("ub_values", _f64p),
        ("eq_indptr", _i32p), ("eq_indices", _i32p), ("eq_values", _f64p),
        ("c", _f64p), ("b_ub", _f64p), ("b_eq", _f64p), ("lb", _f64p), ("ub", _f64p),
    ]


class Options(C.Structure):
    _fields_ = [
        ("mode", C.c_int32), ("precision", C.c_int32), ("max_iters", C.c_int64), ("tol", C.c_double),
        ("check_interval", C.c_int32), ("ruiz_iters", C.c_int32), ("time_limit_s", C.c_double),
        ("graph_mode", C.c_int32), ("device", C.c_int32), ("max_blocks", C.c_int32),
        ("batch_group", C.c_int32), ("escalate", C.c_int32), ("warm_fallback", C.c_int32),
        ("batch_team", C.c_int32), ("batch_team_nnz", C.c_int32), ("batch_handoff_nnz", C.c_int32),
        ("kkt_form", C.c_int32),
    ]


class BatchStats(C.Structure):
    _fields_ = [
        ("setup_ms", C.c_double), ("solve_ms", C.c_double), ("total_iterations", C.c_int64),
        ("optimal", C.c_int32), ("lanes_per_column", C.c_int32), ("blocks", C.c_int32),
        ("escalated", C.c_int32), ("lanes_per_row", C.c_int32), ("team", C.c_int32), ("handed_off", C.c_int32),
        ("reserved", C.c_int32 * 1),
    ]


class Result(C.Structure):
    _fields_ = [
        ("status", C.c_int32), ("restarts", C.c_int32), ("iterations", C.c_int64),
        ("accepted_steps", C.c_int64), ("objective", C.c_double), ("rel_kkt", C.c_double),
        ("rel_primal", C.c_double), ("rel_dual", C.c_double), ("rel_gap", C.c_double),
        ("primal_weight", C.c_double), ("step_size", C.c_double), ("setup_ms", C.c_double),
        ("solve_ms", C.c_double), ("kernel_launches", C.c_int64), ("returned_average", C.c_int32),
        ("escalated", C.c_int32), ("warm_start_used", C.c_int32), ("reserved", C.c_int32),
        ("rel_kkt_lagrangian", C.c_double),
    ]


class DeviceLP(C.Structure):
    """sps_device_lp: every pointer is a device address (integers from the caller's allocator)."""
    _fields_ = [
        ("n", C.c_int32), ("m_ub", C.c_int32), ("m_eq", C.c_int32),
        ("indptr", C.c_void_p), ("indices", C.c_void_p), ("values", C.c_void_p),
        ("c", C.c_void_p), ("rhs", C.c_void_p), ("lb", C.c_void_p), ("ub", C.c_void_p),
    ]


class GnnGraph(C.Structure):
    _fields_ = [
        ("n_var", C.c_int32), ("n_con", C.c_int32),
        ("con_ptr", _i32p), ("con_idx", _i32p), ("con_val", C.POINTER(C.c_float)),
        ("f_var", C.c_int32), ("f_con", C.c_int32), ("con_kind", C.POINTER(C.c_int8)),
    ]


class GnnOptions(C.Structure):
    _fields_ = [
        ("hidden", C.c_int32), ("layers", C.c_int32), ("seed", C.c_uint64),
        ("lr", C.c_float), ("beta1", C.c_float), ("beta2", C.c_float), ("eps", C.c_float),
        ("loss_x", C.c_float), ("loss_y", C.c_float), ("loss_omega", C.c_float),
        ("max_batch", C.c_int32), ("device", C.c_int32), ("lp_features", C.c_int32),
        ("reserved", C.c_int32 * 5),
    ]


_lib = None


def library_path() -> str:
    return _build.LIB


def load() -> C.CDLL:
    """Load the engine library (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} is missing: build it with `python -c \"import __graft_entry__ as g; g.build()\"` "
            "(needs nvcc for sm_103a); the PDHG engine has no CPU fallback")
    lib = C.CDLL(path)
    H = C.c_void_p
    sig = {
        "sps_options_init": (C.c_int, [C.POINTER(Options)]),
        "sps_create": (C.c_int, [C.POINTER(ProblemDesc), C.POINTER(Options), C.POINTER(H)]),
        "sps_set_warm_start": (C.c_int, [H, _f64p, _f64p, C.c_double]),
        "sps_solve": (C.c_int, [H, C.POINTER(Result)]),
        "sps_get_solution": (C.c_int, [H, _f64p, _f64p]),
        "sps_last_error": (C.c_char_p, [H]),
        "sps_destroy": (None, [H]),
        "sps_pin_host": (C.c_int, [C.c_void_p, C.c_uint64]),
        "sps_unpin_host": (C.c_int, [C.c_void_p]),
        "sps_version": (C.c_char_p, []),
        "sps_device_count": (C.c_int, []),
        "sps_time_iteration_kernels": (C.c_int, [H, C.c_int32, _f64p]),
        "sps_time_iteration_kernels_graph": (C.c_int, [H, C.c_int32, _f64p]),
        "sps_time_gather_floor": (C.c_int, [C.c_int64, C.c_int32, C.c_int32, C.c_int32, _f64p]),
        "sps_kkt_noalloc": (C.c_int, [C.POINTER(DeviceLP), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
        "sps_batch_create": (C.c_int, [C.c_int32, C.POINTER(ProblemDesc), C.POINTER(Options), C.POINTER(H)]),
        "sps_batch_solve": (C.c_int, [H, C.POINTER(BatchStats)]),
        "sps_batch_get": (C.c_int, [H, C.c_int32, _f64p, _f64p, C.POINTER(Result)]),
        "sps_batch_set_warm_starts": (C.c_int, [H, _f64p, _f64p, _f64p]),
        "sps_batch_last_error": (C.c_char_p, [H]),
        "sps_batch_destroy": (None, [H]),
        "sps_gnn_options_init": (C.c_int, [C.POINTER(GnnOptions)]),
        "sps_gnn_create": (C.c_int, [C.POINTER(GnnGraph), C.POINTER(GnnOptions), C.POINTER(H)]),
        "sps_gnn_predict": (C.c_int, [H, C.c_int32, _f32p, _f32p, _f32p, _f32p, _f32p]),
        "sps_gnn_loss_grad": (C.c_int, [H, C.c_int32, _f32p, _f32p, _f32p, _f32p, _f32p, _f64p, _f32p]),
        "sps_gnn_train_step": (C.c_int, [H, C.c_int32, _f32p, _f32p, _f32p, _f32p, _f32p, _f64p]),
        "sps_gnn_num_params": (C.c_int64, [H]),
        "sps_gnn_get_params": (C.c_int, [H, _f32p]),
        "sps_gnn_set_params": (C.c_int, [H, _f32p]),
        "sps_gnn_last_error": (C.c_char_p, [H]),
        "sps_gnn_destroy": (None, [H]),
        "sps_batch_set_warm_starts_gnn": (C.c_int, [H, H, _f64p]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def check(rc: int, handle=None) -> None:
    if rc != 0:
        lib = load()
        msg = lib.sps_last_error(handle).decode(errors="replace")
        kind = ERRORS.get(rc, str(rc))
        if rc == -1:
            raise ValueError(f"{kind}: {msg}")
        raise RuntimeError(f"{kind}: {msg}")


def f64p(a):
    return a.ctypes.data_as(_f64p) if a is not None and a.size else None


def f32p(a):
    return a.ctypes.data_as(_f32p) if a is not None and a.size else None


def i32p(a):
    return a.ctypes.data_as(_i32p) if a is not None and a.size else None
