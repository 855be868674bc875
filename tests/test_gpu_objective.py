"""Objective error of the GPU engine against the repository's own FP64 revised
simplex (config-0 LPs: 200 x 500 planted, equality rows, 0 <= x <= 2) at the
benchmark tolerance, FP32 iterates."""

import pytest

import sovereign_solver_gb300 as sps
import sovereign_solver_gb300.workloads as wl
from oracle import kkt, simplex

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_objective_error_vs_simplex(seed):
    p, info = wl.planted_lp(seed=seed)
    ref = simplex.solve(p)
    assert ref.status == "optimal"
    r = sps.solve_lp_pdhg(p, tol=1e-4)
    assert r.status == "optimal"
    err = abs(r.objective - ref.objective) / (1 + abs(ref.objective))
    print(f"seed {seed}: objective {r.objective:.9f} vs simplex {ref.objective:.9f}, rel error {err:.2e}")
    # the relative duality gap is below 1e-4 and the residuals are small: the
    # objective is within a few gap units of the optimum
    assert err < 1e-3
    assert kkt.box_rel_kkt(p, r.x, r.y)["err"] < 1.5e-4
