"""Strong branching with batched child solves (sovereign_solver_gb300.branching)
against the reference's rules (solver/milp/branching.py:98-262) evaluated with
the repository's FP64 simplex (the oracle) in place of the reference's.

CPU tests: candidate ranking, scores, pseudocosts, child bounds, and the batch
plumbing (with the batch replaced by the oracle simplex).  GPU tests: gains
and chosen variables of the real batched PDHG against the oracle."""

import numpy as np
import pytest
import scipy.sparse as sp

import sovereign_solver_gb300 as sps
import sovereign_solver_gb300.branching as br
from oracle import simplex


def milp(c, A_ub, b_ub, ints, lb=None, ub=None, A_eq=None, b_eq=None):
    n = len(c)
    mask = np.zeros(n, dtype=bool)
    mask[list(ints)] = True
    return sps.Problem(c=np.asarray(c, float), A_ub=sp.csr_matrix(np.asarray(A_ub, float).reshape(-1, n)),
                       b_ub=np.asarray(b_ub, float),
                       A_eq=sp.csr_matrix((0, n)) if A_eq is None else sp.csr_matrix(np.asarray(A_eq, float)),
                       b_eq=np.zeros(0) if b_eq is None else np.asarray(b_eq, float),
                       lb=np.zeros(n) if lb is None else np.asarray(lb, float),
                       ub=np.full(n, np.inf) if ub is None else np.asarray(ub, float), integer_mask=mask)


def relax(p):
    return sps.Problem(c=p.c, A_ub=p.A_ub, b_ub=p.b_ub, A_eq=p.A_eq, b_eq=p.b_eq, lb=p.lb, ub=p.ub,
                       integer_mask=np.zeros(len(p.c), dtype=bool))


def knapsack(seed, n=40, m=4):
    rng = np.random.default_rng(seed)
    W = rng.uniform(1, 10, (m, n))
    cap = 0.4 * W.sum(1)
    v = rng.uniform(1, 10, n)
    return milp(-v, W, cap, range(n), ub=np.ones(n))


def set_cover(seed, m=30, n=60):
    rng = np.random.default_rng(seed)
    A = (rng.random((m, n)) < 0.15).astype(float)
    for i in range(m):
        if not A[i].any():
            A[i, rng.integers(n)] = 1.0
    return milp(rng.uniform(1, 5, n), -A, -np.ones(m), range(n), ub=np.ones(n))


def oracle_gain(child, parent_obj):
    """_lp_gain (branching.py:132-144) with the oracle simplex."""
    r = simplex.solve(child)
    if r.status == "infeasible":
        return np.inf
    if r.status == "optimal":
        return max(0.0, r.objective - parent_obj)
    return 0.0


def oracle_strong(p, x, parent_obj):
    top = br.strong_candidates(x, p.integer_mask)
    down = np.array([oracle_gain(br.child_problem(p, p.lb, p.ub, j, "down", x[j]), parent_obj) for j in top])
    up = np.array([oracle_gain(br.child_problem(p, p.lb, p.ub, j, "up", x[j]), parent_obj) for j in top])
    return top, down, up


# ---------------------------------------------------------------- CPU -------

def test_most_fractional_rules():
    assert br.branch_most_fractional(np.array([1.9, 2.5, 0.1]), np.array([True] * 3)) == 1
    assert br.branch_most_fractional(np.array([1.0, 2.0, 3.0]), np.array([True] * 3)) == -1
    assert br.branch_most_fractional(np.array([1.5, 2.5]), np.array([False, True])) == 1


def test_candidates_match_reference_ranking():
    rng = np.random.default_rng(3)
    for _ in range(20):
        x = np.round(rng.uniform(0, 5, 60) * 4) / 4        # many ties (quarters)
        x[rng.random(60) < 0.3] = np.round(x[rng.random(60) < 0.3].mean())
        mask = rng.random(60) < 0.8
        # branching.py:98-102 and 176-181, written out
        iv = np.where(mask)[0]
        cands = iv[np.abs(x[iv] - np.round(x[iv])) > 1e-5]
        if len(cands) == 0:
            assert len(br.strong_candidates(x, mask)) == 0
            continue
        fr = np.abs(x[cands] - np.round(x[cands]))
        want = cands[np.argsort(np.minimum(fr, 1.0 - fr))[::-1][:min(20, len(cands))]]
        np.testing.assert_array_equal(br.strong_candidates(x, mask), want)


def test_product_score_pick():
    # infinite gains win; the first of equal scores is kept; eps floors zero gains
    assert br.pick_by_product([4, 7, 9], np.array([1.0, np.inf, 2.0]), np.array([1.0, 0.0, 3.0]))[0] == 7
    assert br.pick_by_product([4, 7], np.array([2.0, 2.0]), np.array([3.0, 3.0])) == (4, 2.0, 3.0)
    assert br.pick_by_product([4, 7], np.array([0.0, 1e-3]), np.array([5.0, 1e-3]))[0] == 4


def test_pseudocost_table():
    pc = br.PseudocostTable(3)
    pc.update_up(0, 2.0); pc.update_up(0, 4.0); pc.update_down(0, 1.0); pc.update_down(0, -5.0)
    assert pc[0].up_score == 3.0 and pc[0].down_score == 0.5
    assert pc[0].up_cnt == 2 and pc[0].down_cnt == 2 and not pc[0].is_reliable
    for _ in range(br.RELIABILITY_THRESHOLD):
        pc.update_up(1, 1.0); pc.update_down(1, 1.0)
    assert pc[1].is_reliable
    assert pc[1].score(0.25) == pytest.approx(0.25 * 0.75)
    pc.update_up(2, np.inf)
    assert np.isinf(pc[2].up_score)


def test_child_bounds():
    p = milp([1, 1, 1], [[1, 1, 1]], [5], [0, 1, 2], lb=[0, 0.5, 0], ub=[4, 4, 4])
    lbx, ubx = np.array([1.0, 0.0, 0.0]), np.array([np.inf, 3.0, np.inf])
    d = br.child_problem(p, lbx, ubx, 0, "down", 2.6)
    u = br.child_problem(p, lbx, ubx, 0, "up", 2.6)
    np.testing.assert_array_equal(d.lb, [1, 0.5, 0]); np.testing.assert_array_equal(d.ub, [2, 3, 4])
    np.testing.assert_array_equal(u.lb, [3, 0.5, 0]); np.testing.assert_array_equal(u.ub, [4, 3, 4])
    assert not d.integer_mask.any()
    # a fractional node bound above the floor crosses: x1 in [0.5, ...], x1 <= floor(0.7) = 0
    assert np.any(br.child_problem(p, lbx, ubx, 1, "down", 0.7).lb > br.child_problem(p, lbx, ubx, 1, "down", 0.7).ub)
    with pytest.raises(ValueError):
        br.child_problem(p, lbx, ubx, 0, "sideways", 2.6)


class _OracleBatch:
    """Stands in for PDHGBatch on the CPU: every problem solved by the oracle
    simplex; records what the branching code passed."""
    seen = []

    def __init__(self, problems, **kw):
        self.problems = list(problems)
        self.kw = kw
        _OracleBatch.seen.append(self)

    def set_warm_starts(self, starts):
        self.starts = list(starts)

    def solve(self):
        out = []
        for p in self.problems:
            r = simplex.solve(p)
            out.append(sps.SolveResult(r.status, r.x, r.objective, r.iterations))
        return out

    def __enter__(self):
        return self

    def __exit__(self, *a):
        pass


def test_batch_plumbing_with_oracle(monkeypatch):
    monkeypatch.setattr(br, "PDHGBatch", _OracleBatch)
    _OracleBatch.seen.clear()
    p = knapsack(5)
    lp = simplex.solve(relax(p))
    top, down_o, up_o = oracle_strong(p, lp.x, lp.objective)
    assert len(top) > 0
    down, up = br.child_gains(p, top, lp.x, p.lb, p.ub, lp.objective, tol=1e-6)
    np.testing.assert_allclose(down, down_o, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(up, up_o, rtol=1e-12, atol=1e-12)
    b = _OracleBatch.seen[-1]
    assert len(b.problems) == 2 * len(top) and b.kw["tol"] == 1e-6
    for q, j in enumerate(top):                      # (down_j, up_j) pairs in candidate order
        assert b.problems[2 * q].ub[j] == np.floor(lp.x[j]) and b.problems[2 * q + 1].lb[j] == np.ceil(lp.x[j])
        for k in (2 * q, 2 * q + 1):
            x0, y0, w0 = b.starts[k]
            assert np.all(x0 >= b.problems[k].lb) and np.all(x0 <= b.problems[k].ub)
            assert y0.shape == (p.A_ub.shape[0],) and w0 is None
    j, dg, ug = br.branch_strong(lp.x, p.integer_mask, p, p.lb, p.ub, lp.objective)
    assert (j, dg, ug) == br.pick_by_product(top, down_o, up_o)


def test_crossed_bounds_are_infeasible_without_a_solve(monkeypatch):
    monkeypatch.setattr(br, "PDHGBatch", _OracleBatch)
    _OracleBatch.seen.clear()
    p = milp([1, 1], [[1, 1]], [3], [0, 1], lb=[0.5, 0], ub=[4, 4])
    down, up, res = br.child_gains(p, [0], np.array([0.7, 1.0]), p.lb, p.ub, 0.7, return_results=True)
    assert np.isinf(down[0]) and res[0].status == "infeasible" and res[1].status == "optimal"
    assert len(_OracleBatch.seen[-1].problems) == 1


def test_reliability_uses_pseudocosts_for_reliable(monkeypatch):
    monkeypatch.setattr(br, "PDHGBatch", _OracleBatch)
    _OracleBatch.seen.clear()
    p = knapsack(9)
    lp = simplex.solve(relax(p))
    cands = br.fractional_vars(lp.x, p.integer_mask)
    assert len(cands) >= 2
    pc = br.PseudocostTable(len(p.c))
    rel = int(cands[0])
    for _ in range(br.RELIABILITY_THRESHOLD):
        pc.update_up(rel, 100.0); pc.update_down(rel, 100.0)
    j, dg, ug = br.branch_reliability_pseudocost(lp.x, p.integer_mask, p, p.lb, p.ub, lp.objective, pc)
    assert j in cands
    # only the unreliable candidates were strong-branched, in one batch
    assert len(_OracleBatch.seen) == 1 and len(_OracleBatch.seen[0].problems) == 2 * (len(cands) - 1)
    assert pc[rel].up_cnt == br.RELIABILITY_THRESHOLD


# ---------------------------------------------------------------- GPU -------

def _check_against_oracle(p, tol_gain):
    lp = simplex.solve(relax(p))
    assert lp.status == "optimal"
    top, down_o, up_o = oracle_strong(p, lp.x, lp.objective)
    if len(top) == 0:
        pytest.skip("LP optimum already integral")
    down, up, res = br.child_gains(p, top, lp.x, p.lb, p.ub, lp.objective, tol=1e-6, return_results=True)
    scale = 1.0 + abs(lp.objective)
    for q in range(len(top)):
        for g, go in ((down[q], down_o[q]), (up[q], up_o[q])):
            if np.isinf(go):
                assert np.isinf(g), (top[q], g, go)
            else:
                assert abs(g - go) <= tol_gain * scale, (top[q], g, go)
    j, dg, ug = br.branch_strong(lp.x, p.integer_mask, p, p.lb, p.ub, lp.objective, tol=1e-6)
    s_o = np.maximum(1e-6, down_o) * np.maximum(1e-6, up_o)
    best = np.max(s_o)
    # the chosen variable is one whose oracle score is within the gain tolerance of the best
    q = list(top).index(j)
    assert s_o[q] >= best * (1 - 1e-3) - 1e-9 or np.isinf(best) and np.isinf(s_o[q]), (j, s_o[q], best)
    return res


@pytest.mark.gpu
def test_reference_two_variable_milp():
    # tests/test_branching.py:102-128 of the reference: min 2x0 + x1, x0 + x1 >= 3.5
    p = milp([2.0, 1.0], [[-1.0, -1.0]], [-3.5], [0, 1])
    lp = simplex.solve(relax(p))
    j, dg, ug = br.branch_strong(lp.x, p.integer_mask, p, p.lb.copy(), p.ub.copy(), lp.objective, tol=1e-6)
    assert j in (0, 1) and dg >= 0 and ug >= 0
    assert abs(dg - 0.5) < 1e-4 and abs(ug - 0.5) < 1e-4


@pytest.mark.gpu
def test_infeasible_child_gain_is_infinite():
    # min x0 + 2 x1, x0 + x1 = 1.5, 0 <= x <= 1: down child of x1 (x1 <= 0) needs x0 = 1.5 > 1
    p = milp([1.0, 2.0], np.zeros((0, 2)), [], [0, 1], ub=[1.0, 1.0], A_eq=[[1.0, 1.0]], b_eq=[1.5])
    lp = simplex.solve(relax(p))
    down, up, res = br.child_gains(p, [1], lp.x, p.lb, p.ub, lp.objective, tol=1e-6, return_results=True)
    assert res[0].status == "infeasible" and np.isinf(down[0])
    assert res[1].status == "optimal" and abs(up[0] - 0.5) < 1e-4


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_knapsack_gains_match_oracle(seed):
    _check_against_oracle(knapsack(seed), 1e-4)


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [0, 1])
def test_set_cover_gains_match_oracle(seed):
    _check_against_oracle(set_cover(seed), 1e-4)


@pytest.mark.gpu
def test_reliability_pseudocost_on_gpu():
    p = knapsack(4)
    lp = simplex.solve(relax(p))
    pc = br.PseudocostTable(len(p.c))
    j, dg, ug = br.branch_reliability_pseudocost(lp.x, p.integer_mask, p, p.lb, p.ub, lp.objective, pc,
                                                 tol=1e-6)
    assert j in br.fractional_vars(lp.x, p.integer_mask)
    assert dg >= 0 and ug >= 0
