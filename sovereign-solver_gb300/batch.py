"""Batched restarted PDHG: many independent LPs solved in one persistent launch.

New API surface (the reference solves one LP per call).  Each instance keeps
its own step size, primal weight, restarts and termination; the batch is
packed and scaled on the GPU once (``PDHGBatch``), then solved by one
persistent kernel launch replayed from a CUDA graph (``PDHGBatch.solve``).
Adaptive mode with FP32 iterates and FP64 checks; an instance whose error
stops halving in FP32 is finished in FP64 by the single-LP engine after the
launch, warm-started from its best point (``escalate="fp64"``, the default).
"""

from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import _native as N
from .pdhg import MAX_PDHG_ITERS, _Desc, make_options, to_result
from .result import SolveResult


class PDHGBatch:
    """A batch of problems resident on the GPU.

    ``batch_group`` picks the lanes per column of the column pass (1, 2, 4, 8,
    16, 32); 0 lets the library time the candidates on a sample of the batch.
    The lanes per row of the row pass (4, 8, 16, 32) are always timed.
    ``batch_team``: blocks (a thread-block cluster) per large instance, 1 = one
    block per instance, 0 = 4 (or, in a batch of fewer instances than half the
    resident blocks, the largest of 2, 4, 8 that keeps them all resident);
    ``batch_team_nnz``: nonzeros from which an instance is large (0 = 65 536 in
    such a small batch, else the larger of 65 536 and twice the median).
    ``escalate``: "fp64" (FP64 continuation of stalled instances), "stop"
    (status "stalled") or "off" (FP32 to the iteration limit).
    ``batch_handoff_nnz`` (> 0): once the instance queue is empty and 7/8 of the
    blocks have left, instances with at least this many nonzeros (and 512
    attempts) still running leave the launch and are finished by the single-LP
    engine on the whole GPU; which ones leave depends on timing, so results are
    not bit-identical from run to run.  0 (default) = never.
    ``kkt_form``: the batched solver measures the Lagrangian form only (the
    PDLP form is an option of the single-LP engine).
    """

    def __init__(self, problems: Sequence, tol: float = 1e-4, max_iters: int = MAX_PDHG_ITERS,
                 batch_group: int = 0, time_limit: float = 0.0, check_interval: int = 0,
                 graph_mode: int = 2, device: int = 0, ruiz_iters: int = 10, escalate: str = "fp64",
                 warm_fallback: bool = True, batch_team: int = 0, batch_team_nnz: int = 0,
                 batch_handoff_nnz: int = 0, kkt_form: str = "lagrangian"):
        self.lib = N.load()
        self.problems = list(problems)
        if not self.problems:
            raise ValueError("empty batch")
        self._descs = [_Desc(p) for p in self.problems]
        arr = (N.ProblemDesc * len(self._descs))(*[d.desc for d in self._descs])
        o = make_options(tol=tol, max_iters=max_iters, time_limit=time_limit,
                         check_interval=check_interval, graph_mode=graph_mode, device=device,
                         ruiz_iters=ruiz_iters, escalate=escalate, warm_fallback=warm_fallback,
                         kkt_form=kkt_form)
        o.batch_group = int(batch_group)
        o.batch_team = int(batch_team)
        o.batch_team_nnz = int(batch_team_nnz)
        o.batch_handoff_nnz = int(batch_handoff_nnz)
        h = C.c_void_p()
        N.check(self.lib.sps_batch_create(len(self._descs), arr, C.byref(o), C.byref(h)), None)
        self.h = h
        self.stats = None

    def _check(self, rc):
        if rc != 0:
            msg = self.lib.sps_batch_last_error(self.h).decode(errors="replace")
            raise RuntimeError(f"{N.ERRORS.get(rc, rc)}: {msg}")

    def set_warm_starts(self, starts) -> None:
        """Warm starts for the following solves: one (x0, y0, omega0) per problem (omega0
        <= 0 or None = default), e.g. from ``WarmStartGNN.predict``; None clears them."""
        if starts is None:
            self._check(self.lib.sps_batch_set_warm_starts(self.h, None, None, None))
            return
        starts = list(starts)
        if len(starts) != len(self.problems):
            raise ValueError("one warm start per problem")
        xs, ys, om = [], [], np.empty(len(starts))
        for k, (d, st) in enumerate(zip(self._descs, starts)):
            x0, y0, w0 = (tuple(st) + (None, None, None))[:3]
            xs.append(np.zeros(d.n) if x0 is None else np.asarray(x0, float).ravel())
            ys.append(np.zeros(d.m_ub + d.m_eq) if y0 is None else np.asarray(y0, float).ravel())
            if xs[-1].size != d.n or ys[-1].size != d.m_ub + d.m_eq:
                raise ValueError(f"warm start {k}: wrong length")
            om[k] = -1.0 if w0 is None else float(w0)
        x = np.ascontiguousarray(np.concatenate(xs))
        y = np.ascontiguousarray(np.concatenate(ys))
        self._check(self.lib.sps_batch_set_warm_starts(self.h, N.f64p(x), N.f64p(y), N.f64p(om)))

    def set_warm_starts_gnn(self, net) -> None:
        """Warm starts predicted on the device by ``net`` (a ``WarmStartGNN`` with LP
        features for this batch's constraint pattern) for every problem; nothing
        crosses the host."""
        sc = np.array([net.scales[k] for k in ("c", "b", "x", "y")], dtype=np.float64)
        self._check(self.lib.sps_batch_set_warm_starts_gnn(self.h, net.h, N.f64p(sc)))

    def solve_raw(self) -> N.BatchStats:
        st = N.BatchStats()
        self._check(self.lib.sps_batch_solve(self.h, C.byref(st)))
        self.stats = st
        return st

    def result(self, k: int) -> SolveResult:
        d = self._descs[k]
        x = np.empty(d.n)
        y = np.empty(d.m_ub + d.m_eq)
        r = N.Result()
        self._check(self.lib.sps_batch_get(self.h, int(k), N.f64p(x), N.f64p(y), C.byref(r)))
        return to_result(self.problems[k], r, x, y, "adaptive-batch", "fp32")

    def solve(self) -> list[SolveResult]:
        self.solve_raw()
        return [self.result(k) for k in range(len(self.problems))]

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.sps_batch_destroy(self.h)
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


def solve_lp_pdhg_batch(problems: Sequence, tol: float = 1e-4, max_iters: int = MAX_PDHG_ITERS,
                        **kw) -> list[SolveResult]:
    """Solve every problem of ``problems`` on the GPU in one persistent launch."""
    with PDHGBatch(problems, tol=tol, max_iters=max_iters, **kw) as b:
        return b.solve()
