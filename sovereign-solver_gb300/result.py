"""Solver output type.

Keeps the reference ``SolveResult`` fields and constructor order
(``solver/lp/simplex_dense.py:36-62``: status, x, objective, iterations,
message, basis, gaps) and adds what the GPU engine reports beyond them:

* ``y``        — dual multipliers of the original rows (A_ub rows first, then
                  A_eq rows); sign convention: the Lagrangian is
                  ``cᵀx − yᵀ(Kx − rhs)`` so ``y ≤ 0`` on ≤ rows of a min problem.
* ``rel_kkt``  — max(relative primal residual, relative dual residual,
                  relative gap) of the returned point, computed in FP64 on the GPU.
* ``stats``    — dict: restarts, kernel launches, timings, precision, mode, …
"""

from __future__ import annotations

from typing import Optional

import numpy as np


class SolveResult:
    def __init__(
        self,
        status: str,
        x: Optional[np.ndarray],
        objective: float,
        iterations: int,
        message: str = "",
        basis: Optional[np.ndarray] = None,
        gaps: Optional[list] = None,
        y: Optional[np.ndarray] = None,
        rel_kkt: Optional[float] = None,
        stats: Optional[dict] = None,
    ):
        self.status = status
        self.x = x
        self.objective = objective
        self.iterations = iterations
        self.message = message
        self.basis = basis
        self.gaps = gaps or []
        self.y = y
        self.rel_kkt = rel_kkt
        self.obj_error: Optional[float] = None
        self.stats = stats or {}

    def __repr__(self) -> str:
        obj = f"{self.objective:.6g}" if self.objective is not None else "N/A"
        kkt = f", rel_kkt={self.rel_kkt:.2e}" if self.rel_kkt is not None else ""
        return f"SolveResult(status={self.status!r}, obj={obj}, iters={self.iterations}{kkt})"
