"""The C + OpenMP oracle (timed CPU baseline) agrees with the NumPy oracle."""

import pytest

from fixtures import load_golden, load_problems
from oracle import pdhg_ref, pdhg_ref_c

GOLD = load_golden()
PROBLEMS = load_problems()


@pytest.mark.parametrize("name", ["afiro", "blending", "t_2var", "t_random46", "mixed_bounds",
                                  "planted200x500_s0", "planted200x500_s1"])
def test_c_oracle_matches_numpy_oracle(name):
    g = GOLD[name]
    p = PROBLEMS[name]
    a = pdhg_ref.solve(p, max_iters=g["max_iters"], tol=g["tol"])
    b = pdhg_ref_c.solve(p, max_iters=g["max_iters"], tol=g["tol"])
    assert a.status == b.status == g["status"]
    assert a.iterations == b.iterations == g["iterations"]
    assert abs(a.objective - b.objective) <= 1e-9 * max(1.0, abs(a.objective))
