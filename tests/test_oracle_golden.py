"""The CPU oracle reproduces the reference's own outputs (golden vectors).

Golden vectors were produced by the reference (``tests/golden/make_golden.py``);
the four Netlib rows also equal the reference's published benchmark rows
(``benchmarks/results/benchmark_comparison.csv:5,9,13,17``).
"""

import os

import numpy as np
import pytest

from fixtures import GOLDEN, load_golden, load_problems
from oracle import kkt, pdhg_ref

PROBLEMS = load_problems()
GOLD = load_golden()

# published CSV rows, reproduced by the reference here
PUBLISHED = {
    "afiro": ("optimal", -464.75314109, 8950),
    "blending": ("optimal", -3200.00034671, 550),
    "adlittle": ("iteration_limit", 225255.19439650, 25000),
    "brandy": ("iteration_limit", 1521.20660887, 25000),
}


@pytest.mark.parametrize("name", sorted(GOLD))
def test_oracle_matches_reference(name):
    g = GOLD[name]
    r = pdhg_ref.solve(PROBLEMS[name], max_iters=g["max_iters"], tol=g["tol"])
    assert r.status == g["status"]
    assert r.iterations == g["iterations"]
    ref_obj = float(g["objective"])
    assert abs(r.objective - ref_obj) <= 1e-12 * max(1.0, abs(ref_obj))
    if g["x"] is not None:
        np.testing.assert_allclose(r.x, [float(v) for v in g["x"]], rtol=1e-10, atol=1e-12)


@pytest.mark.parametrize("name", sorted(PUBLISHED))
def test_golden_equals_published_rows(name):
    st, obj, it = PUBLISHED[name]
    g = GOLD[name]
    assert g["status"] == st and g["iterations"] == it
    assert abs(float(g["objective"]) - obj) < 1e-8 * abs(obj)


def test_standard_form_matches_reference():
    z = np.load(os.path.join(GOLDEN, "stdform_golden.npz"))
    std = pdhg_ref.to_standard_form(PROBLEMS["mixed_bounds"])
    np.testing.assert_array_equal(std.A.toarray(), z["A"])
    np.testing.assert_array_equal(std.b, z["b"])
    np.testing.assert_array_equal(std.c, z["c"])
    np.testing.assert_array_equal(std.lb_shift, z["lb_shift"])
    tau, sigma = pdhg_ref.diagonal_steps(std.A)
    np.testing.assert_array_equal(tau, z["tau"])
    np.testing.assert_array_equal(sigma, z["sigma"])
    assert std.neg.any() and std.ub_cols.size > 0     # the fixture exercises both branches


def test_kkt_evaluators_on_planted_optimum():
    """The planted (x*, y*) is optimal: both error measures vanish there."""
    import sovereign_solver_gb300.workloads as wl
    p, info = wl.planted_lp(seed=3)
    box = kkt.box_rel_kkt(p, info["x_star"], info["y_star"])
    ref = kkt.ref_form_error(p, info["x_star"], info["y_star"])
    assert box["err"] < 1e-13 and ref["err"] < 1e-13
    assert abs(box["pobj"] - info["obj_star"]) < 1e-10 * max(1.0, abs(info["obj_star"]))
    # a perturbed point is caught by both
    x = info["x_star"] + 1e-2
    assert kkt.box_rel_kkt(p, x, info["y_star"])["err"] > 1e-4
    assert kkt.ref_form_error(p, x, info["y_star"])["err"] > 1e-4


def test_reference_result_certifies_in_std_form():
    """The reference's own averaged std-form pair meets its tolerance."""
    p = PROBLEMS["planted200x500_s0"]
    r = pdhg_ref.solve(p, max_iters=100000, tol=1e-4)
    std = r.std
    assert pdhg_ref.kkt_error(std.A, std.A.T.tocsr(), std.b, std.c, r.z, r.w)[0] < 1e-4


def test_empty_problem():
    import sovereign_solver_gb300 as sps
    r = pdhg_ref.solve(sps.Problem.empty(4))
    assert r.status == "optimal" and r.iterations == 0 and np.all(r.x == 0)
