"""Strong branching for branch-and-bound with the child LPs solved as one GPU batch.

Drop-in for the reference's strong-branching rules in
``solver/milp/branching.py``:

* ``branch_strong``                  (``:158-210``): the K most fractional
  candidates (K = 20, ``solver/config.py:44``), two children each; the product
  score ``max(eps, gain_down) * max(eps, gain_up)`` picks the variable;
* ``branch_reliability_pseudocost``  (``:215-262``): pseudocost scores for
  reliable candidates, strong branching for the rest;
* ``PseudocostTable``                (``:47-92``): per-variable gain statistics.

The reference evaluates each child with ``_lp_gain`` (``:132-144``), one
sequential simplex solve per child.  Here the 2K children (same constraint
matrix, one tightened bound each) are solved together by ``PDHGBatch``: one
persistent launch, each child warm-started from the parent's point clipped to
its bounds.  A child's gain keeps ``_lp_gain``'s meaning: +inf when the child
is infeasible (PDHG's infeasibility certificate), ``max(0, objective -
parent_obj)`` when it is solved, 0 otherwise (iteration or time limit,
unbounded).  Gains are as exact as the solve tolerance (relative KKT error
``tol``): the objective of a child is within about ``tol`` (relative) of the
simplex value the reference computes.
"""

from __future__ import annotations

import dataclasses
from typing import Dict, Optional, Sequence, Tuple

import numpy as np

from .batch import PDHGBatch
from .problem import Problem
from .result import SolveResult

INTEGER_TOL = 1e-5              # solver/config.py:14
STRONG_BRANCH_CANDIDATES = 20   # solver/config.py:44
RELIABILITY_THRESHOLD = 8       # solver/config.py:46
SCORE_EPS = 1e-6                # branching.py:71, :197, :256


@dataclasses.dataclass
class PseudocostEntry:
    """Gain statistics of one variable (the reference's ``PseudocostEntry``)."""
    up_sum: float = 0.0
    down_sum: float = 0.0
    up_cnt: int = 0
    down_cnt: int = 0

    @property
    def up_score(self) -> float:
        return self.up_sum / max(1, self.up_cnt)

    @property
    def down_score(self) -> float:
        return self.down_sum / max(1, self.down_cnt)

    @property
    def is_reliable(self) -> bool:
        return self.up_cnt >= RELIABILITY_THRESHOLD and self.down_cnt >= RELIABILITY_THRESHOLD

    def score(self, frac: float) -> float:
        return max(SCORE_EPS, self.down_score * frac) * max(SCORE_EPS, self.up_score * (1.0 - frac))


class PseudocostTable:
    """Per-variable ``PseudocostEntry``, created on first access; gains are
    recorded clipped at zero (an infinite gain stays infinite)."""

    def __init__(self, n_vars: int):
        self.n = n_vars
        self._data: Dict[int, PseudocostEntry] = {}

    def __getitem__(self, j: int) -> PseudocostEntry:
        if j not in self._data:
            self._data[j] = PseudocostEntry()
        return self._data[j]

    def update_up(self, j: int, gain: float) -> None:
        self[j].up_sum += max(0.0, gain)
        self[j].up_cnt += 1

    def update_down(self, j: int, gain: float) -> None:
        self[j].down_sum += max(0.0, gain)
        self[j].down_cnt += 1


def fractional_vars(x: np.ndarray, mask: np.ndarray) -> np.ndarray:
    """Integer variables whose value is more than ``INTEGER_TOL`` from an integer."""
    iv = np.flatnonzero(mask)
    return iv[np.abs(x[iv] - np.round(x[iv])) > INTEGER_TOL]


def child_problem(problem, lb_extra: np.ndarray, ub_extra: np.ndarray, j: int, direction: str,
                  x_val: float) -> Problem:
    """LP relaxation of one child: the node's bounds (problem bounds tightened
    by ``lb_extra`` / ``ub_extra``) plus x_j <= floor(x_val) ("down") or
    x_j >= ceil(x_val) ("up")."""
    lb = np.maximum(problem.lb, lb_extra).astype(float)
    ub = np.minimum(problem.ub, ub_extra).astype(float)
    if direction == "down":
        ub[j] = min(ub[j], np.floor(x_val))
    elif direction == "up":
        lb[j] = max(lb[j], np.ceil(x_val))
    else:
        raise ValueError(f"direction must be 'down' or 'up', got {direction!r}")
    return Problem(c=problem.c, A_ub=problem.A_ub, b_ub=problem.b_ub, A_eq=problem.A_eq,
                   b_eq=problem.b_eq, lb=lb, ub=ub, integer_mask=np.zeros(len(problem.c), dtype=bool),
                   sense=getattr(problem, "sense", "min"), name=getattr(problem, "name", ""))


def gain_of(result, parent_obj: float) -> float:
    """``_lp_gain``'s reading of a child solve."""
    if result.status == "infeasible":
        return np.inf
    if result.status == "optimal":
        return max(0.0, float(result.objective) - parent_obj)
    return 0.0


def child_gains(problem, candidates: Sequence[int], x: np.ndarray, lb_extra: np.ndarray,
                ub_extra: np.ndarray, parent_obj: float, *, y: Optional[np.ndarray] = None,
                tol: float = 1e-4, max_iters: int = 100_000, time_limit: float = 0.0,
                device: int = 0, return_results: bool = False):
    """Gains (down, up) of every candidate, all 2K children in one batched solve.

    Children are ordered (down_0, up_0, down_1, up_1, ...).  Each starts from
    the parent's x clipped to its own bounds and the parent's y (zeros when
    not given); a start worse than the cold one is dropped by the solver."""
    cands = [int(j) for j in candidates]
    down = np.zeros(len(cands))
    up = np.zeros(len(cands))
    if not cands:
        return (down, up, []) if return_results else (down, up)
    x = np.asarray(x, dtype=float)
    kids = []
    for j in cands:
        kids.append(child_problem(problem, lb_extra, ub_extra, j, "down", x[j]))
        kids.append(child_problem(problem, lb_extra, ub_extra, j, "up", x[j]))
    m = problem.A_ub.shape[0] + problem.A_eq.shape[0]
    y0 = np.zeros(m) if y is None else np.asarray(y, dtype=float)
    # a child whose bounds cross (a fractional node bound below the floor) is
    # infeasible as it stands: it is not solved
    solve_idx = [q for q, kp in enumerate(kids) if not np.any(kp.lb > kp.ub)]
    res = [SolveResult("infeasible", None, np.nan, 0, message="crossed bounds") for _ in kids]
    if solve_idx:
        starts = [(np.clip(x, kids[q].lb, kids[q].ub), y0, None) for q in solve_idx]
        with PDHGBatch([kids[q] for q in solve_idx], tol=tol, max_iters=max_iters,
                       time_limit=time_limit, device=device) as b:
            b.set_warm_starts(starts)
            for q, r in zip(solve_idx, b.solve()):
                res[q] = r
    for q in range(len(cands)):
        down[q] = gain_of(res[2 * q], parent_obj)
        up[q] = gain_of(res[2 * q + 1], parent_obj)
    return (down, up, res) if return_results else (down, up)


def strong_candidates(x: np.ndarray, mask: np.ndarray, k: int = STRONG_BRANCH_CANDIDATES) -> np.ndarray:
    """The reference's candidate list: fractional variables ranked by distance
    to the nearest integer, farthest first, at most k (the same ``argsort``
    call as ``branching.py:176-181``, so ties fall the same way)."""
    cands = fractional_vars(x, mask)
    if len(cands) == 0:
        return cands
    fracs = np.abs(x[cands] - np.round(x[cands]))
    scores = np.minimum(fracs, 1.0 - fracs)
    top_k = min(k, len(cands))
    return cands[np.argsort(scores)[::-1][:top_k]]


def pick_by_product(cands: Sequence[int], down: np.ndarray, up: np.ndarray) -> Tuple[int, float, float]:
    """First candidate with the largest ``max(eps, down) * max(eps, up)``."""
    best, best_score, bd, bu = int(cands[0]), -np.inf, 0.0, 0.0
    for q, j in enumerate(cands):
        s = max(SCORE_EPS, down[q]) * max(SCORE_EPS, up[q])
        if s > best_score:
            best, best_score, bd, bu = int(j), s, float(down[q]), float(up[q])
    return best, bd, bu


def branch_strong(x: np.ndarray, mask: np.ndarray, problem, lb_extra: np.ndarray, ub_extra: np.ndarray,
                  parent_obj: float, pseudocosts: Optional[PseudocostTable] = None, *,
                  y: Optional[np.ndarray] = None, candidates: int = STRONG_BRANCH_CANDIDATES,
                  tol: float = 1e-4, max_iters: int = 100_000, device: int = 0) -> Tuple[int, float, float]:
    """Strong branching (``branching.py:158-210``): returns (variable, down
    gain, up gain), or (-1, 0, 0) when no integer variable is fractional."""
    x = np.asarray(x, dtype=float)
    top = strong_candidates(x, mask, candidates)
    if len(top) == 0:
        return -1, 0.0, 0.0
    down, up = child_gains(problem, top, x, lb_extra, ub_extra, parent_obj, y=y, tol=tol,
                           max_iters=max_iters, device=device)
    if pseudocosts is not None:
        for q, j in enumerate(top):
            pseudocosts.update_down(int(j), down[q])
            pseudocosts.update_up(int(j), up[q])
    return pick_by_product(top, down, up)


def branch_reliability_pseudocost(x: np.ndarray, mask: np.ndarray, problem, lb_extra: np.ndarray,
                                  ub_extra: np.ndarray, parent_obj: float, pseudocosts: PseudocostTable, *,
                                  y: Optional[np.ndarray] = None, tol: float = 1e-4,
                                  max_iters: int = 100_000, device: int = 0) -> Tuple[int, float, float]:
    """Reliability pseudocost branching (``branching.py:215-262``): reliable
    candidates are scored from their pseudocosts, the unreliable ones by strong
    branching (all their children in one batch); returns (variable, estimated
    down gain, estimated up gain) from the pseudocosts after the update."""
    x = np.asarray(x, dtype=float)
    cands = fractional_vars(x, mask)
    if len(cands) == 0:
        return -1, 0.0, 0.0
    scores: Dict[int, float] = {}
    unreliable = []
    for j in cands:
        pc = pseudocosts[int(j)]
        if pc.is_reliable:
            scores[int(j)] = pc.score(x[j] - np.floor(x[j]))
        else:
            unreliable.append(int(j))
    if unreliable:
        down, up = child_gains(problem, unreliable, x, lb_extra, ub_extra, parent_obj, y=y, tol=tol,
                               max_iters=max_iters, device=device)
        for q, j in enumerate(unreliable):
            pseudocosts.update_down(j, down[q])
            pseudocosts.update_up(j, up[q])
            scores[j] = max(SCORE_EPS, down[q]) * max(SCORE_EPS, up[q])
    best = max(scores, key=scores.get)
    pc = pseudocosts[best]
    frac = x[best] - np.floor(x[best])
    return best, pc.down_score * frac, pc.up_score * (1.0 - frac)


def branch_most_fractional(x: np.ndarray, mask: np.ndarray) -> int:
    """The integer variable farthest from an integer (``branching.py:147-155``), -1 if none."""
    cands = fractional_vars(x, mask)
    if len(cands) == 0:
        return -1
    fracs = np.abs(x[cands] - np.round(x[cands]))
    return int(cands[np.argmax(np.minimum(fracs, 1.0 - fracs))])
