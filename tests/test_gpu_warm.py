"""Warm starts with the cold-start fallback, single-LP and batched.

A warm start at the solution is kept and finishes in a few iterations; a bad
one (far from feasible) is rejected by the fallback, after which the solve is
the cold solve exactly (same iterations, same bits)."""

import numpy as np
import pytest

import sovereign_solver_gb300 as sps
import sovereign_solver_gb300.workloads as wl
from oracle import kkt

pytestmark = pytest.mark.gpu
TOL = 1e-4


def _bad_start(p, scale=1e3):
    rng = np.random.default_rng(0)
    return rng.random(p.n_vars) * scale, -rng.random(p.n_ineq + p.n_eq) * scale, 1.0


def test_single_warm_start_and_fallback():
    p, info = wl.batch_planted_lp(5, m_range=(100, 400))
    with sps.PDHGEngine(p, tol=TOL) as eng:
        cold = eng.solve()
        assert cold.status == "optimal" and not cold.stats["warm_start_used"]
        eng.warm_start(cold.x, cold.y, cold.stats["primal_weight"])
        warm = eng.solve()
        assert warm.status == "optimal" and warm.stats["warm_start_used"]
        assert warm.iterations <= max(64, cold.iterations // 4)
        eng.warm_start(*_bad_start(p))
        fb = eng.solve()
        assert fb.status == "optimal" and not fb.stats["warm_start_used"]
        assert fb.iterations == cold.iterations
        np.testing.assert_array_equal(fb.x, cold.x)
    # without the fallback the bad start is used (and still converges or not; it is judged by KKT)
    with sps.PDHGEngine(p, tol=TOL, warm_fallback=False) as eng:
        eng.warm_start(*_bad_start(p))
        r = eng.solve()
        assert r.stats["warm_start_used"]
        if r.status == "optimal":
            assert kkt.box_rel_kkt(p, r.x, r.y)["err"] < 1.5 * TOL


def test_batch_warm_starts_and_fallback():
    probs = [wl.batch_planted_lp(k, m_range=(50, 400))[0] for k in range(12)]
    with sps.PDHGBatch(probs, tol=TOL) as b:
        cold = b.solve()
        starts = []
        for k, (p, r) in enumerate(zip(probs, cold)):
            starts.append((r.x, r.y, r.stats["primal_weight"]) if k % 2 == 0 else _bad_start(p))
        b.set_warm_starts(starts)
        warm = b.solve()
        b.set_warm_starts(None)
        again = b.solve()
    for k, (p, c, w, a) in enumerate(zip(probs, cold, warm, again)):
        assert w.status == "optimal", k
        assert kkt.box_rel_kkt(p, w.x, w.y)["err"] < 1.5 * TOL
        if k % 2 == 0:
            assert w.stats["warm_start_used"] and w.iterations <= max(64, c.iterations // 4), (k, w.iterations)
        else:
            assert not w.stats["warm_start_used"] and w.iterations == c.iterations, k
            np.testing.assert_array_equal(w.x, c.x)
        assert a.iterations == c.iterations and not a.stats["warm_start_used"]
