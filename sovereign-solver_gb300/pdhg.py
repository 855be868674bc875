"""Restarted PDHG on the GB300 — host side of the hot path.

Mirrors the reference's entry points for this path with the same names,
argument meaning and error behaviour:

* ``solve_lp_pdhg(problem, max_iters, tol)``         — ``solver/lp/pdhg.py:152-156``
* ``solve_lp_pdhg_gpu(problem, device, max_iters, tol)`` — ``solver/lp/pdhg_gpu.py:315-320``
* ``get_available_device()``                          — ``solver/lp/pdhg_gpu.py:42-67``

Behind them every solve runs in ``libsps_gb300.so`` (hand-written sm_103a
kernels); there is no CPU fallback.  Two rule sets are available:

* ``mode="adaptive"`` (default): box form (bounds projected, no slack rows),
  Ruiz + Pock-Chambolle scaling, adaptive step size and primal weight, KKT-based
  restarts to the average or the current iterate; FP32 iterates and SpMV with
  FP64 checks (``precision="fp32"``) or FP64 throughout.
* ``mode="reference"``: the reference's own rules (standard form with bound rows
  and slacks, fixed diagonal steps τ_j = 0.999/Σ|A_ij|, σ_i = 0.999/Σ|A_ij|,
  θ = 1, ergodic average, KKT of the average every 50 iterations, restart when
  it halves) — ``solver/lp/pdhg.py:62-259``.

The returned ``rel_kkt`` is the relative KKT error of the returned point,
evaluated on the GPU in FP64: for ``adaptive`` the box-form error
max(‖primal residual‖/(1+‖rhs‖), ‖dual residual‖/(1+‖c‖), |gap|/(1+|p|+|d|));
for ``reference`` the reference's own formula (``pdhg.py:184-196``).
"""

from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np
import scipy.sparse as sp

from . import _native as N
from .result import SolveResult

MAX_PDHG_ITERS = 100_000    # solver/config.py:37
PDHG_TOL = 1e-6             # solver/config.py:12


def get_available_device() -> str:
    """'cuda' when a CUDA device is visible to the engine, else 'cpu'.

    'cpu' only describes the machine: the engine itself never runs there.
    """
    try:
        return "cuda" if N.load().sps_device_count() > 0 else "cpu"
    except (OSError, RuntimeError):
        return "cpu"


def _csr(M, n):
    M = sp.csr_matrix(M, dtype=np.float64)
    if M.shape[1] != n:
        raise ValueError(f"matrix has {M.shape[1]} columns, expected {n}")
    return (np.ascontiguousarray(M.indptr, dtype=np.int32),
            np.ascontiguousarray(M.indices, dtype=np.int32),
            np.ascontiguousarray(M.data, dtype=np.float64))


class _Desc:
    """Problem fields as contiguous arrays plus the C descriptor over them."""

    def __init__(self, problem):
        n = int(problem.n_vars)
        self.n = n
        self.m_ub, self.m_eq = int(problem.n_ineq), int(problem.n_eq)
        self.ub = _csr(problem.A_ub, n)
        self.eq = _csr(problem.A_eq, n)
        f = lambda v: np.ascontiguousarray(np.asarray(v, dtype=np.float64).ravel())
        self.c, self.b_ub, self.b_eq = f(problem.c), f(problem.b_ub), f(problem.b_eq)
        self.lb, self.ubd = f(problem.lb), f(problem.ub)
        if self.b_ub.size != self.m_ub or self.b_eq.size != self.m_eq:
            raise ValueError("right-hand side length does not match the constraint rows")
        if self.c.size != n or self.lb.size != n or self.ubd.size != n:
            raise ValueError("c/lb/ub length does not match n_vars")
        d = N.ProblemDesc()
        d.n, d.m_ub, d.m_eq = n, self.m_ub, self.m_eq
        d.ub_indptr, d.ub_indices, d.ub_values = N.i32p(self.ub[0]), N.i32p(self.ub[1]), N.f64p(self.ub[2])
        d.eq_indptr, d.eq_indices, d.eq_values = N.i32p(self.eq[0]), N.i32p(self.eq[1]), N.f64p(self.eq[2])
        d.c, d.b_ub, d.b_eq = N.f64p(self.c), N.f64p(self.b_ub), N.f64p(self.b_eq)
        d.lb, d.ub = N.f64p(self.lb), N.f64p(self.ubd)
        self.desc = d

    def arrays(self):
        return [*self.ub, *self.eq, self.c, self.b_ub, self.b_eq, self.lb, self.ubd]


def make_options(mode="adaptive", precision="fp32", max_iters=MAX_PDHG_ITERS, tol=PDHG_TOL,
                 check_interval=0, ruiz_iters=10, time_limit=0.0, graph_mode=2, device=0,
                 max_blocks=0, escalate="fp64", warm_fallback=True, kkt_form="lagrangian") -> N.Options:
    """Options for ``sps_create``.  ``escalate`` (adaptive FP32): "fp64" continues a
    stalled solve in FP64 from its best point, "stop" ends it with status
    "stalled", "off" keeps iterating in FP32 (a single LP counts as stalled only
    once its best relative KKT error is at most 1e-3 and has not halved for
    max(2048, k/2) attempts since, k the attempt of the last halving).  ``warm_fallback``: start cold when
    a warm start's relative KKT error is above the cold start's.  ``kkt_form``
    (adaptive mode): "lagrangian" puts every finite bound into the dual
    objective; "pdlp" leaves out bounds farther from x_j than |x_j| and counts
    the reduced cost they would absorb as dual residual (PDLP's default)."""
    if mode not in N.MODES:
        raise ValueError(f"Unknown mode {mode!r}. Choose 'adaptive' or 'reference'.")
    if precision not in N.PRECISIONS:
        raise ValueError(f"Unknown precision {precision!r}. Choose 'fp32' or 'fp64'.")
    if escalate not in N.ESCALATE:
        raise ValueError(f"Unknown escalate {escalate!r}. Choose 'fp64', 'stop' or 'off'.")
    if kkt_form not in N.KKT_FORMS:
        raise ValueError(f"Unknown kkt_form {kkt_form!r}. Choose 'lagrangian' or 'pdlp'.")
    o = N.Options()
    N.load().sps_options_init(C.byref(o))
    o.mode, o.precision = N.MODES[mode], N.PRECISIONS[precision]
    o.max_iters, o.tol = int(max_iters), float(tol)
    o.check_interval, o.ruiz_iters = int(check_interval), int(ruiz_iters)
    o.time_limit_s, o.graph_mode, o.device = float(time_limit), int(graph_mode), int(device)
    o.max_blocks = int(max_blocks)
    o.escalate = N.ESCALATE[escalate]
    o.warm_fallback = 1 if warm_fallback else 0
    o.kkt_form = N.KKT_FORMS[kkt_form]
    return o


class PDHGEngine:
    """A problem resident on the GPU, solvable repeatedly (cold or warm).

    Construction uploads the problem and builds the device layout
    (``sps_create``); ``solve()`` runs the iteration on the resident data.
    """

    def __init__(self, problem, **opts):
        self.lib = N.load()
        self.problem = problem
        self.opts = dict(opts)
        self.mode = opts.get("mode", "adaptive")
        self.precision = opts.get("precision", "fp32")
        self._d = _Desc(problem)
        self._o = make_options(**opts)
        h = C.c_void_p()
        N.check(self.lib.sps_create(C.byref(self._d.desc), C.byref(self._o), C.byref(h)), None)
        self.h = h
        self.n, self.m = self._d.n, self._d.m_ub + self._d.m_eq

    def warm_start(self, x0: Optional[np.ndarray] = None, y0: Optional[np.ndarray] = None,
                   omega0: float = 0.0) -> None:
        xa = None if x0 is None else np.ascontiguousarray(x0, dtype=np.float64)
        ya = None if y0 is None else np.ascontiguousarray(y0, dtype=np.float64)
        if xa is not None and xa.size != self.n:
            raise ValueError("x0 length != n_vars")
        if ya is not None and ya.size != self.m:
            raise ValueError("y0 length != number of rows")
        N.check(self.lib.sps_set_warm_start(self.h, N.f64p(xa), N.f64p(ya), float(omega0)), self.h)

    def solve_raw(self) -> N.Result:
        r = N.Result()
        N.check(self.lib.sps_solve(self.h, C.byref(r)), self.h)
        return r

    def solution(self):
        x = np.empty(self.n)
        y = np.empty(self.m)
        N.check(self.lib.sps_get_solution(self.h, N.f64p(x), N.f64p(y)), self.h)
        return x, y

    def solve(self) -> SolveResult:
        r = self.solve_raw()
        x, y = self.solution()
        return to_result(self.problem, r, x, y, self.mode, self.precision)

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.sps_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def to_result(problem, r: N.Result, x, y, mode, precision) -> SolveResult:
    obj = float(r.objective)
    if getattr(problem, "sense", "min") == "max":
        obj = -obj
    status = N.STATUS.get(r.status, str(r.status))
    stats = {
        "mode": mode, "precision": precision, "restarts": int(r.restarts),
        "accepted_steps": int(r.accepted_steps), "rel_primal": float(r.rel_primal),
        "rel_dual": float(r.rel_dual), "rel_gap": float(r.rel_gap),
        "primal_weight": float(r.primal_weight), "step_size": float(r.step_size),
        "setup_ms": float(r.setup_ms), "solve_ms": float(r.solve_ms),
        "kernel_launches": int(r.kernel_launches), "returned_average": bool(r.returned_average),
        "escalated": bool(r.escalated), "warm_start_used": bool(r.warm_start_used),
        "rel_kkt_lagrangian": float(r.rel_kkt_lagrangian),
    }
    msg = f"{mode}/{precision} PDHG on GPU: rel_kkt={r.rel_kkt:.3e}"
    return SolveResult(status, x, obj, int(r.iterations), message=msg, y=y,
                       rel_kkt=float(r.rel_kkt), stats=stats)


def solve_lp_pdhg(problem, max_iters: int = MAX_PDHG_ITERS, tol: float = PDHG_TOL, *,
                  mode: str = "adaptive", precision: str = "fp32", warm_start=None,
                  time_limit: float = 0.0, graph_mode: int = 2, check_interval: int = 0,
                  device: int = 0, escalate: str = "fp64", kkt_form: str = "lagrangian") -> SolveResult:
    """Solve an LP with restarted PDHG on the GPU (``solver/lp/pdhg.py:152``).

    ``warm_start`` = (x0, y0, omega0) starts from a given point (adaptive mode).
    Non-convergence is not an error: status ``"iteration_limit"``.  With FP32
    iterates a solve whose error stops halving continues in FP64 from its best
    point (``escalate="fp64"``; ``stats["escalated"]`` tells).  ``kkt_form`` picks
    the measure ``tol`` applies to (``make_options``).
    """
    with PDHGEngine(problem, mode=mode, precision=precision, max_iters=max_iters, tol=tol,
                    time_limit=time_limit, graph_mode=graph_mode, check_interval=check_interval,
                    device=device, escalate=escalate, kkt_form=kkt_form) as eng:
        if warm_start is not None:
            x0, y0, w0 = (tuple(warm_start) + (None, None, 0.0))[:3]
            eng.warm_start(x0, y0, w0 or 0.0)
        return eng.solve()


def solve_lp_pdhg_gpu(problem, device: str = "auto", max_iters: int = MAX_PDHG_ITERS,
                      tol: float = PDHG_TOL, **kw) -> SolveResult:
    """``solver/lp/pdhg_gpu.py:315`` signature.  ``device`` must be 'auto' or
    'cuda' (or a CUDA ordinal such as 'cuda:1'): there is no CPU/MPS path."""
    if device in ("auto", "cuda"):
        ordinal = 0
    elif isinstance(device, str) and device.startswith("cuda:") and device[5:].isdigit():
        ordinal = int(device[5:])
    else:
        raise ValueError(f"Unknown device: {device!r}. This engine runs on 'auto' or 'cuda' only.")
    return solve_lp_pdhg(problem, max_iters=max_iters, tol=tol, device=ordinal, **kw)
