"""GB300-native restarted-PDHG LP engine, a drop-in for the reference's
``Solver(...).solve(method='pdhg')`` path (``solver/solver.py:113-119``).

Public names mirror the reference package exports (``solver/__init__.py:22-38``)
for this path: ``Solver``, ``Problem``, ``SolveResult``, ``solve_lp_pdhg``,
``solve_lp_pdhg_gpu``, ``get_available_device``; plus ``PDHGEngine`` (a problem
kept resident on the GPU for repeated / warm-started solves), ``PDHGBatch``
(many LPs in one persistent launch) and ``branching`` (strong branching with
the child LPs solved as one batch, ``solver/milp/branching.py``).
"""

from .problem import Problem
from .result import SolveResult
from .pdhg import PDHGEngine, get_available_device, solve_lp_pdhg, solve_lp_pdhg_gpu
from .solver import Solver
from .batch import PDHGBatch, solve_lp_pdhg_batch
from .mps import read_mps
from . import branching

__version__ = "0.1.0"
__all__ = ["Solver", "Problem", "SolveResult", "PDHGEngine", "solve_lp_pdhg",
           "solve_lp_pdhg_gpu", "get_available_device", "PDHGBatch", "solve_lp_pdhg_batch", "read_mps"]
