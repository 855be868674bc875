"""GPU parity at workload scale and on the paths only large or odd LPs take.

* The 1000 x 2000 transportation LP (2M variables, 4M nonzeros: the default
  benchmark workload) solved to 1e-4: the returned (x, y) is re-checked on the
  CPU in FP64 by the oracle (box form, and the reference's own error formula on
  the mapped standard-form pair, ``solver/lp/pdhg.py:181-196``), and its
  objective is compared with the exact optimum (HiGHS dual simplex, committed
  in ``tests/golden/optima.json``).  Its demand rows take the SLAB schedule and
  its supply rows the SEGMENT schedule, which small LPs never reach.
* A power-law LP (the 1M x 2M workload's construction scaled to 20k x 40k):
  with ``kkt_form="pdlp"`` (far finite bounds count as dual residual) it
  reaches 1e-4 in a few thousand attempts, re-checked by the oracle in the same
  form, objective against the planted optimum; in the Lagrangian form (every
  finite bound in the dual objective) a 5k x 10k copy reaches 1e-4 in FP64.
* Columns longer than the device sort's 64 entries (ordered on the host).
* The reference benchmark runner's badly scaled LP
  (``benchmarks/run_benchmarks.py:314-378``), on which the reference PDHG stops
  at its cap with objective 4.15 (``benchmark_comparison.csv:35``; optimum 0).
"""

import json
import os

import numpy as np
import pytest
import scipy.sparse as sp

import sovereign_solver_gb300 as sps
import sovereign_solver_gb300.workloads as wl
from fixtures import GOLDEN, load_stress
from oracle import kkt

pytestmark = pytest.mark.gpu


def _optimum(key):
    with open(os.path.join(GOLDEN, "optima.json")) as f:
        return float(json.load(f)[key]["objective"])


def test_transport_1000x2000_to_1e4():
    p, _ = wl.transportation_lp(1000, 2000, seed=0)
    r = sps.solve_lp_pdhg(p, tol=1e-4)
    assert r.status == "optimal", r
    box = kkt.box_rel_kkt(p, r.x, r.y)
    assert box["err"] < 1.5e-4, box
    assert abs(box["err"] - r.rel_kkt) < 0.5e-4 + 1e-3 * box["err"]     # the device's FP64 check agrees
    ref = kkt.ref_form_error(p, r.x, r.y)
    assert ref["err"] < 1e-3, ref
    opt = _optimum("transport_1000x2000_s0")
    assert abs(r.objective - opt) <= 4e-4 * (1 + abs(opt)), (r.objective, opt)


def _powerlaw(m, nnz_per_row=20, seed=0):
    return wl.powerlaw_lp(m=m, n=2 * m, target_nnz=nnz_per_row * m, seed=seed)


def test_powerlaw_pdlp_form():
    p, info = _powerlaw(20_000)
    r = sps.solve_lp_pdhg(p, tol=1e-4, kkt_form="pdlp", max_iters=20000)
    assert r.status == "optimal", r
    assert r.iterations < 8000, r.iterations
    box = kkt.box_rel_kkt(p, r.x, r.y, form="pdlp")
    assert box["err"] < 1.5e-4, box
    assert abs(box["err"] - r.rel_kkt) < 0.5e-4 + 1e-3 * box["err"]
    star = info["obj_star"]
    assert abs(r.objective - star) <= 1e-3 * (1 + abs(star)), (r.objective, star)
    # the same point in the Lagrangian form, which the engine reports beside it: a valid
    # but far looser certificate on this LP (u = 10 on 2M columns with x* in [0, 1])
    lag = kkt.box_rel_kkt(p, r.x, r.y)
    assert lag["err"] > box["err"]
    assert abs(lag["err"] - r.stats["rel_kkt_lagrangian"]) <= 1e-3 * lag["err"] + 1e-6, (lag, r.stats)


def test_fp32_stall_needs_an_error_below_the_ceiling():
    """On the 1M x 2M power-law LP (21M nonzeros, PDLP form) the FP32 error sits
    near 1.3e-2 for thousands of attempts: that plateau is the method's slow
    progress, and the single-LP stall test may declare a stall (and hand over to
    FP64) only once the best error is at most 1e-3.  Measured: it stops at
    8.2e-4 after 17 216 attempts (before the ceiling: at 1.3e-2 after 3 968)."""
    p, info = wl.powerlaw_lp(seed=0)
    r = sps.solve_lp_pdhg(p, tol=1e-4, kkt_form="pdlp", max_iters=40000, escalate="stop")
    assert r.status in ("stalled", "optimal"), r
    assert r.iterations > 8192, r.iterations
    assert r.rel_kkt < 2e-3, r.rel_kkt


def test_powerlaw_lagrangian_fp64():
    p, info = _powerlaw(5_000)
    r = sps.solve_lp_pdhg(p, tol=1e-4, precision="fp64", max_iters=100000)
    assert r.status == "optimal", r
    box = kkt.box_rel_kkt(p, r.x, r.y)
    assert box["err"] < 1.5e-4, box
    assert r.stats["rel_kkt_lagrangian"] == r.rel_kkt
    star = info["obj_star"]
    assert abs(r.objective - star) <= 1e-3 * (1 + abs(star)), (r.objective, star)


def _long_column_lp(seed=5, m=400, n=800, long_cols=(3, 77, 500), long_len=(150, 260, 399)):
    rng = np.random.default_rng(seed)
    mask = rng.random((m, n)) < 0.02
    for j, L in zip(long_cols, long_len):
        mask[:, j] = False
        mask[rng.choice(m, L, replace=False), j] = True
    empty = np.flatnonzero(~mask.any(0))
    mask[rng.integers(0, m, empty.size), empty] = True
    rows, cols = np.nonzero(mask)
    A = sp.csr_matrix((rng.standard_normal(rows.size), (rows, cols)), shape=(m, n))
    A.sort_indices()
    x_star = np.where(rng.random(n) < 0.6, rng.random(n), 0.0)
    y_star = rng.standard_normal(m)
    s_star = np.where(x_star > 0, 0.0, rng.exponential(1.0, n))
    p = sps.Problem(c=A.T @ y_star + s_star, A_ub=sp.csr_matrix((0, n)), b_ub=np.zeros(0), A_eq=A,
                    b_eq=A @ x_star, lb=np.zeros(n), ub=np.full(n, 2.0),
                    integer_mask=np.zeros(n, dtype=bool), name="long_columns")
    return p, float(A @ x_star @ y_star), A


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_columns_longer_than_the_device_sort(precision):
    p, star, A = _long_column_lp()
    assert np.diff(A.tocsc().indptr).max() > 64
    tol = 1e-4 if precision == "fp32" else 1e-7
    r = sps.solve_lp_pdhg(p, tol=tol, precision=precision)
    assert r.status == "optimal", r
    box = kkt.box_rel_kkt(p, r.x, r.y)
    assert box["err"] < 1.5 * tol, box
    assert abs(r.objective - star) <= 10 * tol * (1 + abs(star)), (r.objective, star)


def test_badly_scaled_1e8_on_the_gpu():
    probs, gold = load_stress()
    p, g = probs["badly_scaled_1e8"], gold["badly_scaled_1e8"]
    r = sps.solve_lp_pdhg(p, tol=1e-6)
    assert r.status == "optimal", r
    assert kkt.box_rel_kkt(p, r.x, r.y)["err"] < 1.5e-6
    opt = float(g["published"]["highs_objective"])
    assert abs(r.objective - opt) <= 1e-5 * (1 + abs(opt)), (r.objective, opt)
    # the reference PDHG ends at its 100 000-iteration cap, objective 4.15 against the optimum 0
    assert float(g["published"]["objective"]) > 4.0 and r.iterations < g["iterations"] / 5
