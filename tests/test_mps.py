"""MPS reader: the reference's Netlib instances give the same LP as the
reference's own reader (the committed fixtures), and a synthetic file exercises
every bound type, RANGES on L / G / E rows, OBJSENSE and comments."""

import os

import numpy as np
import pytest

from sovereign_solver_gb300.mps import read_mps
from fixtures import load_golden, load_problems
from oracle import simplex

# the reference checkout's Netlib instances, where a checkout is present (path in
# SPS_REFERENCE_ROOT); the committed fixtures hold what its reader made of them
REF_ROOT = os.environ.get("SPS_REFERENCE_ROOT", "")
REF_INSTANCES = os.path.join(REF_ROOT, "benchmarks", "instances") if REF_ROOT else ""
GOLD = load_golden()
PROBS = load_problems()


def _rows(A, b):
    """Rows of [A | b] as a sorted list (order-free comparison)."""
    M = np.hstack([A.toarray(), np.asarray(b, float)[:, None]])
    return sorted(map(tuple, np.round(M, 12)))


@pytest.mark.parametrize("name", ["afiro", "blending", "adlittle", "brandy"])
def test_netlib_matches_reference_reader(name):
    path = os.path.join(REF_INSTANCES, name + ".mps") if REF_INSTANCES else ""
    if not path or not os.path.exists(path):
        pytest.skip("reference instances not present (set SPS_REFERENCE_ROOT to a reference checkout)")
    p, q = read_mps(path), PROBS[name]
    np.testing.assert_array_equal(p.c, q.c)
    np.testing.assert_array_equal(p.lb, q.lb)
    np.testing.assert_array_equal(p.ub, q.ub)
    assert _rows(p.A_ub, p.b_ub) == _rows(q.A_ub, q.b_ub)
    assert _rows(p.A_eq, p.b_eq) == _rows(q.A_eq, q.b_eq)
    r = simplex.solve(p)
    ref = float(GOLD[name]["simplex_objective"])
    assert r.status == "optimal" and abs(r.objective - ref) <= 1e-9 * (1 + abs(ref))


@pytest.mark.parametrize("name", ["exmip1", "p0033", "p0548"])
def test_milp_files_parse(name):
    path = os.path.join(REF_INSTANCES, name + ".mps") if REF_INSTANCES else ""
    if not path or not os.path.exists(path):
        pytest.skip("reference instances not present (set SPS_REFERENCE_ROOT to a reference checkout)")
    p = read_mps(path)
    p.validate()
    assert p.integer_mask.any()


SYNTHETIC = """\
* a comment line
NAME          TOY
OBJSENSE
    MAX
ROWS
 N  obj
 L  r1
 G  r2
 E  r3
 E  r4
COLUMNS
    MARKER                 'MARKER'                 'INTORG'
    x1        obj       1.0        r1        1.0
    x1        r2        1.0
    MARKER                 'MARKER'                 'INTEND'
    x2        obj       2.0        r1        1.0   $ inline comment
    x2        r3        1.0        r4        1.0
    x3        obj      -1.0        r2        1.0
    x3        r3        2.0
RHS
    rhs       r1        10.0       r2        1.0
    rhs       r3        4.0        r4        2.0
    rhs       obj       99.0
RANGES
    rng       r1        4.0        r2        3.0
    rng       r3        -1.0
BOUNDS
 UP bnd       x1        5.0
 MI bnd       x2
 UP bnd       x3        -1.0
ENDATA
"""


def test_synthetic_file(tmp_path):
    f = tmp_path / "toy.mps"
    f.write_text(SYNTHETIC)
    p = read_mps(f)
    assert p.sense == "max" and p.name == "toy"
    np.testing.assert_array_equal(p.c, [-1.0, -2.0, 1.0])           # stored for minimisation
    np.testing.assert_array_equal(p.integer_mask, [True, False, False])
    np.testing.assert_array_equal(p.lb, [0.0, -np.inf, -np.inf])   # MI; UP < 0 without LO
    np.testing.assert_array_equal(p.ub, [5.0, np.inf, -1.0])
    # r1: 6 <= x1 + x2 <= 10; r2: 1 <= x1 + x3 <= 4; r3 (E, R = -1): 3 <= x2 + 2 x3 <= 4; r4: x2 = 2
    U = p.A_ub.toarray()
    expect = [([1, 1, 0], 10), ([-1, -1, 0], -6), ([-1, 0, -1], -1), ([1, 0, 1], 4),
              ([0, 1, 2], 4), ([0, -1, -2], -3)]
    assert len(U) == len(expect)
    for (row, b), u, bu in zip(expect, U, p.b_ub):
        np.testing.assert_array_equal(u, row)
        assert bu == b
    np.testing.assert_array_equal(p.A_eq.toarray(), [[0, 1, 0]])
    np.testing.assert_array_equal(p.b_eq, [2.0])


def test_solver_read_mps_chains(tmp_path):
    """``Solver().read_mps(path)`` loads the file's LP and returns the solver
    (the reference's loader, ``solver/solver.py:41-44``)."""
    from sovereign_solver_gb300 import Solver
    f = tmp_path / "toy.mps"
    f.write_text(SYNTHETIC)
    s = Solver()
    assert s.read_mps(f) is s
    q = read_mps(f)
    np.testing.assert_array_equal(s.problem.c, q.c)
    np.testing.assert_array_equal(s.problem.A_ub.toarray(), q.A_ub.toarray())
    assert s.problem.sense == "max"
