"""``Solver`` facade — the reference's public entry (``solver/solver.py:25-162``)
for the methods this engine provides.

``Solver().set_problem(p).solve(method="pdhg")`` and ``method="pdhg_gpu"``
(``solver.py:113-119``) run the GPU engine.  Other reference methods (simplex,
revised, ipm, milp, qp) are not part of this engine and raise ``ValueError``
like an unknown method does (``solver.py:144-148``).
"""

from __future__ import annotations

from typing import Optional

from .pdhg import solve_lp_pdhg, solve_lp_pdhg_gpu
from .problem import Problem


class Solver:
    def __init__(self) -> None:
        self.problem: Optional[Problem] = None
        self._result = None

    def read_mps(self, path) -> "Solver":
        """Load a problem from an MPS file (``solver/solver.py:41-44``); returns
        self for chaining, without validating, as the reference does."""
        from .mps import read_mps as _read_mps
        self.problem = _read_mps(path)
        return self

    def set_problem(self, problem) -> "Solver":
        problem.validate()
        self.problem = problem
        return self

    def solve(self, method: str = "auto", device: str = "auto", **kw):
        """Solve the loaded problem.  ``method``: 'pdhg', 'pdhg_gpu' or 'auto'
        (= 'pdhg' here).  Extra keywords go to :func:`solve_lp_pdhg`."""
        if self.problem is None:
            raise RuntimeError("No problem loaded. Call set_problem() first.")
        if method == "auto":
            method = "pdhg"
        if method == "pdhg":
            result = solve_lp_pdhg(self.problem, **kw)
        elif method == "pdhg_gpu":
            result = solve_lp_pdhg_gpu(self.problem, device=device, **kw)
        else:
            raise ValueError(f"Unknown method {method!r}. This engine provides: auto, pdhg, pdhg_gpu")
        self._result = result
        return result

    @property
    def result(self):
        return self._result

    def __repr__(self) -> str:
        return f"Solver({self.problem!r})" if self.problem else "Solver(no problem loaded)"
