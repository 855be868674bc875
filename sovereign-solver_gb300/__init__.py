"""GB300-native restarted-PDHG LP engine, a drop-in for the reference's
``Solver(...).solve(method='pdhg')`` path (``solver/solver.py:113-119``).

Public names mirror the reference package exports (``solver/__init__.py:22-38``)
for this path: ``Solver``, ``Problem``, ``SolveResult``, ``solve_lp_pdhg``,
``solve_lp_pdhg_gpu``, ``get_available_device``.
"""

from .problem import Problem
from .result import SolveResult

__version__ = "0.1.0"
__all__ = ["Problem", "SolveResult"]
