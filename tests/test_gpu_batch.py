"""Batched PDHG on the GPU: every instance checked by the CPU oracle in FP64.

The batch mixes planted equality LPs of uneven sizes (the batched workload's
construction at smaller sizes), small transportation LPs (<= rows, unbounded
columns) and the mixed-bounds fixture (free / boxed / one-sided columns).
"""

import numpy as np
import pytest

import sovereign_solver_gb300 as sps
import sovereign_solver_gb300.workloads as wl
from fixtures import load_problems
from oracle import kkt

pytestmark = pytest.mark.gpu

TOL = 1e-4


def _batch():
    probs, stars = [], []
    for k in range(40):
        p, info = wl.batch_planted_lp(k, m_range=(20, 400))
        probs.append(p)
        stars.append(info["obj_star"])
    for s in range(6):
        probs.append(wl.transportation_lp(20 + 5 * s, 40 + 7 * s, seed=s)[0])
        stars.append(None)
    probs.append(load_problems()["mixed_bounds"])
    stars.append(None)
    return probs, stars


@pytest.mark.parametrize("group", [0, 4, 32])
def test_batch_solves_every_instance(group):
    probs, stars = _batch()
    with sps.PDHGBatch(probs, tol=TOL, max_iters=200000, batch_group=group) as b:
        res = b.solve()
        st = b.stats
    assert st.optimal == len(probs)
    assert group == 0 or st.lanes_per_column == group
    for p, r, star in zip(probs, res, stars):
        assert r.status == "optimal", (p.name, r)
        box = kkt.box_rel_kkt(p, r.x, r.y)
        assert box["err"] < 1.5 * TOL, (p.name, box)
        if star is not None:
            assert abs(r.objective - star) <= 20 * TOL * (1 + abs(star)), (p.name, r.objective, star)


def test_batch_matches_single_and_is_deterministic():
    probs, _ = _batch()
    probs = probs[:12]
    with sps.PDHGBatch(probs, tol=TOL, batch_group=8) as b:
        a = b.solve()
        c = b.solve()                    # graph replay
    for r1, r2 in zip(a, c):
        assert r1.iterations == r2.iterations
        np.testing.assert_array_equal(r1.x, r2.x)
    for p, r in zip(probs, a):
        s = sps.solve_lp_pdhg(p, tol=TOL)
        assert abs(s.objective - r.objective) <= 20 * TOL * (1 + abs(s.objective))


def test_batch_iteration_limit():
    probs, _ = _batch()
    res = sps.solve_lp_pdhg_batch(probs[:5], tol=1e-12, max_iters=128)
    for r in res:
        assert r.status == "iteration_limit" and r.iterations == 128


def _large_batch():
    """Planted instances of the batched workload with at least 65 536 nonzeros
    (solved by a cluster of blocks) mixed with small ones (one block each)."""
    probs = []
    for k in range(200):
        p, info = wl.batch_planted_lp(k)
        if p.A_eq.nnz >= 65536 and sum(q.A_eq.nnz >= 65536 for q in probs) < 6:
            probs.append(p)
    probs += [wl.batch_planted_lp(k, m_range=(20, 300))[0] for k in range(10)]
    return probs


@pytest.mark.parametrize("size", [4, 8])
def test_team_solves_large_instances(size):
    probs = _large_batch()
    assert sum(p.A_eq.nnz >= 65536 for p in probs) >= 4
    with sps.PDHGBatch(probs, tol=TOL, batch_team=size) as b:
        team = b.solve()
        assert b.stats.team == size
        again = b.solve()                     # graph replay: same bits
    with sps.PDHGBatch(probs, tol=TOL, batch_team=1) as b:
        solo = b.solve()
        assert b.stats.team == 1
    for p, t, a, s in zip(probs, team, again, solo):
        assert t.status == "optimal" and s.status == "optimal", p.name
        assert kkt.box_rel_kkt(p, t.x, t.y)["err"] < 1.5 * TOL, p.name
        assert t.iterations == a.iterations
        np.testing.assert_array_equal(t.x, a.x)
        assert abs(t.objective - s.objective) <= 50 * TOL * (1 + abs(s.objective))


def test_small_batch_gets_wide_teams():
    """16 instances on 608 resident blocks: every instance of 65 536 nonzeros or
    more is solved by a cluster of 8 blocks by default."""
    probs = _large_batch()
    with sps.PDHGBatch(probs, tol=TOL) as b:
        res = b.solve()
        assert b.stats.team == 8
        assert b.stats.blocks >= 8 * sum(p.A_eq.nnz >= 65536 for p in probs)
    for p, r in zip(probs, res):
        assert r.status == "optimal", p.name
        assert kkt.box_rel_kkt(p, r.x, r.y)["err"] < 1.5 * TOL, p.name


def test_tail_handoff_to_single_engine():
    """60 tiny instances and 4 larger ones, one block each: once the tiny ones are
    done (at least 7/8 of the blocks idle) the larger ones leave the launch at
    their first check after 512 attempts and the single-LP engine finishes them;
    same answers as without hand-off (the default)."""
    probs = [wl.batch_planted_lp(k, m_range=(20, 40))[0] for k in range(60)]
    probs += [wl.batch_planted_lp(100 + k, m_range=(1500, 2000))[0] for k in range(4)]
    with sps.PDHGBatch(probs, tol=TOL, batch_team=1, batch_handoff_nnz=1) as b:
        hand = b.solve()
        n_hand = b.stats.handed_off
    with sps.PDHGBatch(probs, tol=TOL, batch_team=1) as b:
        stay = b.solve()
        assert b.stats.handed_off == 0
    assert n_hand >= 1
    for p, h, s in zip(probs, hand, stay):
        assert h.status == "optimal" and s.status == "optimal", p.name
        assert kkt.box_rel_kkt(p, h.x, h.y)["err"] < 1.5 * TOL, p.name
        assert abs(h.objective - s.objective) <= 50 * TOL * (1 + abs(s.objective)), p.name


def test_batch_edge_cases():
    """An instance with no rows, one with an empty column, beside a normal one."""
    import scipy.sparse as sp
    no_rows = sps.Problem(c=np.array([1.0, -1.0, 0.5]), A_ub=sp.csr_matrix((0, 3)), b_ub=np.zeros(0),
                          A_eq=sp.csr_matrix((0, 3)), b_eq=np.zeros(0), lb=np.zeros(3),
                          ub=np.array([1.0, 2.0, 3.0]), integer_mask=np.zeros(3, bool), name="no_rows")
    A = sp.csr_matrix(np.array([[1.0, 1.0, 0.0], [1.0, -1.0, 0.0]]))
    empty_col = sps.Problem(c=np.array([1.0, 2.0, 3.0]), A_ub=sp.csr_matrix((0, 3)), b_ub=np.zeros(0),
                            A_eq=A, b_eq=np.array([2.0, 0.0]), lb=np.zeros(3), ub=np.full(3, np.inf),
                            integer_mask=np.zeros(3, bool), name="empty_column")
    normal = wl.batch_planted_lp(3, m_range=(50, 200))[0]
    probs = [no_rows, empty_col, normal]
    with sps.PDHGBatch(probs, tol=TOL) as b:
        res = b.solve()
    for p, r in zip(probs, res):
        assert r.status == "optimal", (p.name, r.status)
        assert kkt.box_rel_kkt(p, r.x, r.y)["err"] < 1.5 * TOL, p.name
    np.testing.assert_allclose(res[0].x[:2], [0.0, 2.0], atol=1e-6)
    assert abs(res[0].objective - (-2.0)) < 1e-5
    np.testing.assert_allclose(res[1].x, [1.0, 1.0, 0.0], atol=2e-3)


def test_batch_time_limit():
    """A time limit far below the solve time stops the launch: statuses time_limit, no error."""
    probs = [wl.batch_planted_lp(k)[0] for k in range(64)]
    with sps.PDHGBatch(probs, tol=1e-8, time_limit=0.05, escalate="off") as b:
        res = b.solve()
        assert b.stats.solve_ms < 5000
    assert sum(r.status == "time_limit" for r in res) >= 32


def test_batch_detects_infeasible_and_unbounded():
    import scipy.sparse as sp
    inf = np.inf

    def lp(c, A_ub, b_ub, lb, ub):
        n = len(c)
        return sps.Problem(c=np.asarray(c, float), A_ub=sp.csr_matrix(np.asarray(A_ub, float)),
                           b_ub=np.asarray(b_ub, float), A_eq=sp.csr_matrix((0, n)), b_eq=np.zeros(0),
                           lb=np.asarray(lb, float), ub=np.asarray(ub, float), integer_mask=np.zeros(n, bool))
    probs = [wl.batch_planted_lp(7, m_range=(50, 200))[0],
             lp([1, 1], [[1, 1], [-1, -1]], [1, -2], [0, 0], [inf, inf]),          # infeasible
             lp([-1, 0], [[1, -1]], [1], [0, 0], [inf, inf]),                       # unbounded
             wl.batch_planted_lp(8, m_range=(50, 200))[0]]
    with sps.PDHGBatch(probs, tol=1e-6) as b:
        res = b.solve()
    assert [r.status for r in res] == ["optimal", "infeasible", "unbounded", "optimal"]
