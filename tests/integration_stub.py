"""Struct declarations of the ctypes stub a maintainer adds to the reference
tree to bind the C ABI (``solver/lp/pdhg_gb300.py``, shown in full in the
integration notes).  Kept here as a fixture so that a test can check them
field by field against the package's binding and the header."""

import ctypes as C

i32p, f64p = C.POINTER(C.c_int32), C.POINTER(C.c_double)


class Desc(C.Structure):      # sps_problem_desc
    _fields_ = [("n", C.c_int32), ("m_ub", C.c_int32), ("m_eq", C.c_int32),
                ("ub_indptr", i32p), ("ub_indices", i32p), ("ub_values", f64p),
                ("eq_indptr", i32p), ("eq_indices", i32p), ("eq_values", f64p),
                ("c", f64p), ("b_ub", f64p), ("b_eq", f64p), ("lb", f64p), ("ub", f64p)]


class Opts(C.Structure):      # sps_options
    _fields_ = [("mode", C.c_int32), ("precision", C.c_int32), ("max_iters", C.c_int64),
                ("tol", C.c_double), ("check_interval", C.c_int32), ("ruiz_iters", C.c_int32),
                ("time_limit_s", C.c_double), ("graph_mode", C.c_int32), ("device", C.c_int32),
                ("max_blocks", C.c_int32), ("batch_group", C.c_int32), ("escalate", C.c_int32),
                ("warm_fallback", C.c_int32), ("batch_team", C.c_int32), ("batch_team_nnz", C.c_int32),
                ("batch_handoff_nnz", C.c_int32), ("kkt_form", C.c_int32)]


class Res(C.Structure):       # sps_result
    _fields_ = [("status", C.c_int32), ("restarts", C.c_int32), ("iterations", C.c_int64),
                ("accepted_steps", C.c_int64), ("objective", C.c_double), ("rel_kkt", C.c_double),
                ("rel_primal", C.c_double), ("rel_dual", C.c_double), ("rel_gap", C.c_double),
                ("primal_weight", C.c_double), ("step_size", C.c_double), ("setup_ms", C.c_double),
                ("solve_ms", C.c_double), ("kernel_launches", C.c_int64),
                ("returned_average", C.c_int32), ("escalated", C.c_int32),
                ("warm_start_used", C.c_int32), ("reserved", C.c_int32), ("rel_kkt_lagrangian", C.c_double)]
