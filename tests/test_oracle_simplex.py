"""The repository's FP64 bounded revised simplex (the objective oracle) against
the reference's own simplex objectives (golden vectors made by running the
reference) and against planted optima (c^T x* = b^T y* exactly)."""

import numpy as np
import pytest
import scipy.sparse as sp

import sovereign_solver_gb300 as sps
import sovereign_solver_gb300.workloads as wl
from fixtures import load_golden, load_problems
from oracle import simplex

GOLD = load_golden()
PROBS = load_problems()
NAMES = [k for k, g in GOLD.items() if g.get("simplex_objective") is not None and k in PROBS]


@pytest.mark.parametrize("name", NAMES)
def test_matches_reference_simplex(name):
    r = simplex.solve(PROBS[name])
    ref = float(GOLD[name]["simplex_objective"])
    assert r.status == "optimal"
    assert abs(r.objective - ref) <= 1e-9 * (1 + abs(ref)), (r.objective, ref)


@pytest.mark.parametrize("seed", [0, 1])
def test_planted_optimum(seed):
    p, info = wl.planted_lp(seed=seed)
    r = simplex.solve(p)
    assert r.status == "optimal"
    assert abs(r.objective - info["obj_star"]) <= 1e-10 * (1 + abs(info["obj_star"]))
    assert np.all(r.x >= p.lb - 1e-9) and np.all(r.x <= p.ub + 1e-9)
    assert np.abs(p.A_eq @ r.x - p.b_eq).max() < 1e-8


def _lp(c, A_ub, b_ub, lb, ub):
    n = len(c)
    return sps.Problem(c=np.asarray(c, float), A_ub=sp.csr_matrix(np.asarray(A_ub, float)),
                       b_ub=np.asarray(b_ub, float), A_eq=sp.csr_matrix((0, n)), b_eq=np.zeros(0),
                       lb=np.asarray(lb, float), ub=np.asarray(ub, float), integer_mask=np.zeros(n, bool))


def test_infeasible_and_unbounded():
    infeasible = _lp([1, 1], [[1, 1], [-1, -1]], [1, -2], [0, 0], [np.inf, np.inf])   # x1+x2 <= 1 and >= 2
    assert simplex.solve(infeasible).status == "infeasible"
    unbounded = _lp([-1, 0], [[1, -1]], [1], [0, 0], [np.inf, np.inf])              # x1 - x2 <= 1, max x1
    assert simplex.solve(unbounded).status == "unbounded"
    free = _lp([1, -1], [[1, 1], [-1, 1]], [4, 2], [-np.inf, -np.inf], [np.inf, 3])  # free and upper-only columns
    r = simplex.solve(free)
    assert r.status == "optimal" and abs(r.objective - (-2.0)) < 1e-12
