"""ctypes wrapper of the oracle's C + OpenMP restatement — TEST INFRASTRUCTURE ONLY.

Same algorithm and results as ``oracle.pdhg_ref.solve`` (checked by
``tests/test_oracle_c.py``); used as the timed CPU baseline with all host threads.
"""

import ctypes as C
import os

import numpy as np

from . import build as _build
from . import pdhg_ref

_lib = None


def _load():
    global _lib
    if _lib is None:
        _build.build()
        lib = C.CDLL(_build.LIB)
        ip, dp = C.POINTER(C.c_int32), C.POINTER(C.c_double)
        lib.oracle_pdhg_ref.restype = C.c_int
        lib.oracle_pdhg_ref.argtypes = [C.c_int, C.c_int, ip, ip, dp, ip, ip, dp, dp, dp, C.c_long,
                                        C.c_double, dp, dp, C.POINTER(C.c_long), C.POINTER(C.c_int)]
        _lib = lib
    return _lib


def threads() -> int:
    return int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))


def solve_std(std: "pdhg_ref.StdForm", max_iters: int, tol: float):
    """Run on a prepared standard form; returns (status, z, w, iters, restarts)."""
    lib = _load()
    A = std.A.tocsr()
    AT = A.T.tocsr()
    m, n = A.shape
    i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
    f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    Ap, Ai, Ax = i32(A.indptr), i32(A.indices), f64(A.data)
    Tp, Ti, Tx = i32(AT.indptr), i32(AT.indices), f64(AT.data)
    b, c = f64(std.b), f64(std.c)
    z, w = np.zeros(n), np.zeros(m)
    it, rs = C.c_long(0), C.c_int(0)
    P = lambda a, t: a.ctypes.data_as(C.POINTER(t))
    st = lib.oracle_pdhg_ref(m, n, P(Ap, C.c_int32), P(Ai, C.c_int32), P(Ax, C.c_double),
                             P(Tp, C.c_int32), P(Ti, C.c_int32), P(Tx, C.c_double), P(b, C.c_double),
                             P(c, C.c_double), int(max_iters), float(tol), P(z, C.c_double),
                             P(w, C.c_double), C.byref(it), C.byref(rs))
    return ("optimal" if st == 0 else "iteration_limit"), z, w, int(it.value), int(rs.value)


def solve(problem, max_iters=pdhg_ref.DEFAULT_MAX_ITERS, tol=pdhg_ref.DEFAULT_TOL):
    std = pdhg_ref.to_standard_form(problem)
    if std.A.shape[0] == 0 or std.A.shape[1] == 0:
        return pdhg_ref.RefResult("optimal", np.zeros(problem.n_vars), 0.0, 0, std=std)
    status, z, w, it, rs = solve_std(std, max_iters, tol)
    x = pdhg_ref.recover_x(problem, std, z)
    obj = float(np.asarray(problem.c, float) @ x)
    if problem.sense == "max":
        obj = -obj
    return pdhg_ref.RefResult(status, x, obj, it, z=z, w=w, restarts=rs, std=std)
