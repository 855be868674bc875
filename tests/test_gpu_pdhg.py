"""GPU parity: the sm_103a engine (through the C ABI) against the CPU oracle.

Bars
----
* reference mode, FP64: same status and iteration count as the oracle (which
  reproduces the reference bit-for-bit), objective within 1e-9 relative.
* reference mode, FP32: same status; the returned point certifies in the
  reference's own error formula (FP64, CPU) to 2x the tolerance.
* adaptive mode: optimal at tol; the oracle's FP64 box-form relative KKT of the
  returned (x, y) is below 1.5x tol (FP32 iterates) and the objective agrees
  with the planted optimum / the reference simplex to the gap the KKT allows.
"""

import numpy as np
import pytest
import scipy.sparse as sp

import sovereign_solver_gb300 as sps
import sovereign_solver_gb300.workloads as wl
from fixtures import load_golden, load_problems
from oracle import kkt, pdhg_ref

pytestmark = pytest.mark.gpu

GOLD = load_golden()
PROBLEMS = load_problems()
REF_CASES = sorted(GOLD)


@pytest.mark.parametrize("name", REF_CASES)
def test_reference_mode_fp64_matches_oracle(name):
    g = GOLD[name]
    p = PROBLEMS[name]
    r = sps.solve_lp_pdhg(p, max_iters=g["max_iters"], tol=g["tol"], mode="reference", precision="fp64")
    assert r.status == g["status"], (r, g)
    assert r.iterations == g["iterations"], (r.iterations, g["iterations"])
    ref_obj = float(g["objective"])
    assert abs(r.objective - ref_obj) <= 1e-9 * max(1.0, abs(ref_obj)), (r.objective, ref_obj)
    if g["x"] is not None:
        np.testing.assert_allclose(r.x, [float(v) for v in g["x"]], rtol=1e-7, atol=1e-9)


@pytest.mark.parametrize("name", ["afiro", "blending", "t_2var", "t_random46", "mixed_bounds",
                                  "planted200x500_s0", "planted200x500_s2"])
def test_reference_mode_fp32_certifies(name):
    g = GOLD[name]
    p = PROBLEMS[name]
    tol = max(g["tol"], 1e-4)
    r = sps.solve_lp_pdhg(p, max_iters=g["max_iters"], tol=tol, mode="reference", precision="fp32")
    assert r.status == "optimal", r
    assert r.rel_kkt < tol
    # the engine's FP64 on-device error agrees with the oracle's own formula
    o = pdhg_ref.solve(p, max_iters=g["max_iters"], tol=tol)
    assert abs(r.objective - o.objective) <= 50 * tol * (1 + abs(o.objective))


@pytest.mark.parametrize("seed", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_adaptive_planted(seed, precision):
    p, info = wl.planted_lp(seed=seed)
    tol = 1e-4 if precision == "fp32" else 1e-7
    r = sps.solve_lp_pdhg(p, tol=tol, precision=precision)
    assert r.status == "optimal", r
    box = kkt.box_rel_kkt(p, r.x, r.y)
    assert box["err"] < 1.5 * tol, box
    assert abs(box["err"] - r.rel_kkt) < 0.5 * tol + 1e-3 * box["err"]   # device FP64 check agrees
    assert np.all(r.x >= p.lb - 1e-12) and np.all(r.x <= p.ub + 1e-12)
    obj_star = info["obj_star"]
    assert abs(r.objective - obj_star) <= 10 * tol * (1 + abs(obj_star)), (r.objective, obj_star)
    ref = kkt.ref_form_error(p, r.x, r.y)
    assert ref["err"] < 10 * tol, ref


@pytest.mark.parametrize("seed", [0, 1, 2, 3, 4])
def test_adaptive_agrees_with_reference_pdhg(seed):
    """The bar of the drop-in: on the same 200 x 500 planted LP, the adaptive
    FP32 engine's (x, y) mapped into the reference's standard form has a
    relative KKT error below 1e-4 by the reference's own formula
    (``solver/lp/pdhg.py:181-196``, evaluated in FP64 on the CPU), and its
    objective agrees with the reference PDHG's answer at tol 1e-4 to the
    accuracy either tolerance allows."""
    p, _ = wl.planted_lp(seed=seed)
    r = sps.solve_lp_pdhg(p, tol=5e-5)
    assert r.status == "optimal", r
    assert kkt.ref_form_error(p, r.x, r.y)["err"] < 1e-4
    o = pdhg_ref.solve(p, max_iters=100000, tol=1e-4)
    assert o.status == "optimal"
    assert abs(r.objective - o.objective) <= 2e-3 * (1 + abs(o.objective)), (r.objective, o.objective)


@pytest.mark.parametrize("name", ["afiro", "blending", "adlittle", "t_2var", "t_simple_min",
                                  "t_random46", "t_ub_simple", "t_ub_tight", "mixed_bounds"])
def test_adaptive_known_answers(name):
    g = GOLD[name]
    p = PROBLEMS[name]
    r = sps.solve_lp_pdhg(p, tol=1e-4, max_iters=200000)
    assert r.status == "optimal", r
    box = kkt.box_rel_kkt(p, r.x, r.y)
    assert box["err"] < 1.5e-4, box
    s = g.get("simplex_objective")
    if s is not None:
        s = float(s)
        assert abs(r.objective - s) <= 2e-3 * (1 + abs(s)), (r.objective, s)


def test_transportation_small():
    p, _ = wl.transportation_lp(40, 80, seed=3)
    r = sps.solve_lp_pdhg(p, tol=1e-4)
    assert r.status == "optimal"
    assert kkt.box_rel_kkt(p, r.x, r.y)["err"] < 1.5e-4


@pytest.mark.parametrize("graph_mode", [0, 1, 2])
def test_graph_modes_agree_bitwise(graph_mode):
    p, _ = wl.planted_lp(seed=7)
    base = sps.solve_lp_pdhg(p, tol=1e-5, graph_mode=2)
    r = sps.solve_lp_pdhg(p, tol=1e-5, graph_mode=graph_mode)
    assert r.iterations == base.iterations
    np.testing.assert_array_equal(r.x, base.x)
    np.testing.assert_array_equal(r.y, base.y)


@pytest.mark.parametrize("max_blocks", [8, 0])
def test_segmented_rows_deterministic(max_blocks):
    """Rows longer than one 512-nonzero segment, with few blocks so each warp
    handles several segments: results must be bit-identical run to run."""
    p, _ = wl.transportation_lp(120, 1500, seed=4)      # supply rows of 1500 -> 3 segments
    runs = []
    for gm in (2, 0):
        with sps.PDHGEngine(p, tol=1e-4, max_blocks=max_blocks, graph_mode=gm) as eng:
            runs += [eng.solve(), eng.solve()]
    for r in runs[1:]:
        assert r.iterations == runs[0].iterations
        np.testing.assert_array_equal(r.x, runs[0].x)
        np.testing.assert_array_equal(r.y, runs[0].y)
    assert runs[0].status == "optimal"
    assert kkt.box_rel_kkt(p, runs[0].x, runs[0].y)["err"] < 1.5e-4


def test_repeat_solve_is_deterministic_and_warm_start_helps():
    p, info = wl.planted_lp(seed=5)
    with sps.PDHGEngine(p, tol=1e-5) as eng:
        a = eng.solve()
        b = eng.solve()
        assert a.iterations == b.iterations
        np.testing.assert_array_equal(a.x, b.x)
        eng.warm_start(info["x_star"], info["y_star"])
        w = eng.solve()
    assert w.status == "optimal"
    assert w.iterations <= 64 < a.iterations


def test_iteration_limit_and_max_sense():
    p, _ = wl.planted_lp(seed=1)
    r = sps.solve_lp_pdhg(p, tol=1e-12, max_iters=100)
    assert r.status == "iteration_limit" and r.iterations == 100
    q = load_problems()["mixed_bounds"]      # a 'max' problem with c stored negated
    r = sps.solve_lp_pdhg(q, tol=1e-6, max_iters=200000)
    o = float(GOLD["mixed_bounds"]["simplex_objective"])
    assert abs(r.objective - o) <= 1e-3 * (1 + abs(o))


def test_solver_facade_drop_in():
    p = sps.Problem(c=np.array([-3.0, -5.0]), A_ub=sp.csr_matrix(np.array([[1.0, 0], [0, 2], [3, 2]])),
                    b_ub=np.array([4.0, 12, 18]), A_eq=sp.csr_matrix((0, 2)), b_eq=np.zeros(0),
                    lb=np.zeros(2), ub=np.full(2, np.inf), integer_mask=np.zeros(2, bool))
    for method in ("pdhg", "pdhg_gpu"):
        r = sps.Solver().set_problem(p).solve(method=method)
        assert r.status == "optimal"
        assert abs(r.objective + 36.0) < 1e-3
        np.testing.assert_allclose(r.x, [2.0, 6.0], atol=1e-3)


def test_empty_problem():
    r = sps.solve_lp_pdhg(sps.Problem.empty(3), mode="reference")
    assert r.status == "optimal" and r.iterations == 0 and np.all(r.x == 0)


def _lp(c, A_ub, b_ub, lb, ub, A_eq=None, b_eq=None):
    n = len(c)
    return sps.Problem(c=np.asarray(c, float), A_ub=sp.csr_matrix(np.asarray(A_ub, float).reshape(-1, n)),
                       b_ub=np.asarray(b_ub, float),
                       A_eq=sp.csr_matrix((0, n)) if A_eq is None else sp.csr_matrix(np.asarray(A_eq, float)),
                       b_eq=np.zeros(0) if b_eq is None else np.asarray(b_eq, float),
                       lb=np.asarray(lb, float), ub=np.asarray(ub, float), integer_mask=np.zeros(n, bool))


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_infeasible_and_unbounded_detected(precision):
    """Certificates from the change since the last restart (the reference PDHG
    has none and runs to its iteration limit)."""
    inf = np.inf
    infeasible = _lp([1, 1], [[1, 1], [-1, -1]], [1, -2], [0, 0], [inf, inf])       # x1+x2 <= 1 and >= 2
    r = sps.solve_lp_pdhg(infeasible, max_iters=100000, tol=1e-6, precision=precision)
    assert r.status == "infeasible", (r.status, r.iterations)
    infeasible_eq = _lp([1, 2, 0], [[1, 1, 0]], [3], [0, 0, 0], [1, inf, inf],
                        A_eq=[[1, 0, 1], [0, 1, -1]], b_eq=[-1, 2])                    # x1 + x3 = -1 with x >= 0
    r = sps.solve_lp_pdhg(infeasible_eq, max_iters=100000, tol=1e-6, precision=precision)
    assert r.status == "infeasible", (r.status, r.iterations)
    unbounded = _lp([-1, 0], [[1, -1]], [1], [0, 0], [inf, inf])                    # min -x1, x1 - x2 <= 1
    r = sps.solve_lp_pdhg(unbounded, max_iters=100000, tol=1e-6, precision=precision)
    assert r.status == "unbounded", (r.status, r.iterations)
    free_unbounded = _lp([1, -1], [[1, 1]], [4], [-inf, 0], [inf, inf])              # x1 free, min x1 - x2
    r = sps.solve_lp_pdhg(free_unbounded, max_iters=100000, tol=1e-6, precision=precision)
    assert r.status == "unbounded", (r.status, r.iterations)
