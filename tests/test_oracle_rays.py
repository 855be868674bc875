"""Infeasibility and unboundedness certificates in the CPU restatement of the
adaptive mode (``oracle/pdlp_ref.py``, the rules of ``csrc/decide.cuh``): the
four small LPs the GPU test uses, in both iterate precisions, and the
reference's own PDHG test LP ``test_pdhg_large_sparse_terminates``
(``tests/test_pdhg.py:137-156``), which is unbounded and which the reference
PDHG runs to its 100 000-iteration cap."""

import numpy as np
import pytest
import scipy.sparse as sp

import sovereign_solver_gb300 as sps
from fixtures import load_stress
from oracle import pdlp_ref

INF = np.inf


def _lp(c, A_ub, b_ub, lb, ub, A_eq=None, b_eq=None):
    n = len(c)
    A_eq = np.zeros((0, n)) if A_eq is None else np.asarray(A_eq, float)
    return sps.Problem(c=np.asarray(c, float), A_ub=sp.csr_matrix(np.asarray(A_ub, float).reshape(-1, n)),
                       b_ub=np.asarray(b_ub, float), A_eq=sp.csr_matrix(A_eq.reshape(-1, n)),
                       b_eq=np.asarray([] if b_eq is None else b_eq, float), lb=np.asarray(lb, float),
                       ub=np.asarray(ub, float), integer_mask=np.zeros(n, dtype=bool))


CASES = {
    "infeasible": (_lp([1, 1], [[1, 1], [-1, -1]], [1, -2], [0, 0], [INF, INF]), "infeasible"),
    "infeasible_eq": (_lp([1, 2, 0], [[1, 1, 0]], [3], [0, 0, 0], [1, INF, INF],
                          A_eq=[[1, 0, 1], [0, 1, -1]], b_eq=[-1, 2]), "infeasible"),
    "unbounded": (_lp([-1, 0], [[1, -1]], [1], [0, 0], [INF, INF]), "unbounded"),
    "free_unbounded": (_lp([1, -1], [[1, 1]], [4], [-INF, 0], [INF, INF]), "unbounded"),
}


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("name", sorted(CASES))
def test_small_certificates(name, dtype):
    p, want = CASES[name]
    r = pdlp_ref.solve(p, tol=1e-6, max_iters=100000, dtype=dtype, interaction="difference")
    assert r["status"] == want and r["iterations"] < 2000, (r["status"], r["iterations"])


def test_reference_test_lp_is_found_unbounded():
    probs, gold = load_stress()
    p = probs["ref_test_large_sparse"]
    r = pdlp_ref.solve(p, tol=1e-6, max_iters=100000, dtype=np.float64, interaction="difference")
    assert r["status"] == "unbounded" and r["iterations"] < gold["ref_test_large_sparse"]["iterations"]
