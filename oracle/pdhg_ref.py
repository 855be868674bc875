"""FP64 restatement of the reference's restarted PDHG — TEST INFRASTRUCTURE ONLY.

Follows the reference function by function:

* ``to_standard_form``   — ``solver/lp/pdhg.py:62-125`` (``_to_standard_form_pdhg``)
* ``diagonal_steps``     — ``solver/lp/pdhg.py:131-147`` (``_compute_step_sizes``)
* ``kkt_error``          — ``solver/lp/pdhg.py:181-196`` (``_kkt_residuals`` with the
                           max(1, ‖·‖) normalisers of ``:181-182``)
* ``solve``              — ``solver/lp/pdhg.py:152-259`` (``solve_lp_pdhg``)

Pinned by ``tests/test_oracle_golden.py`` against vectors the reference itself
produced (``tests/golden/``): iteration counts must match exactly and the
objective to 1e-12 relative.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np
import scipy.sparse as sp

FEAS_TOL = 1e-6          # solver/config.py:10  (row-negation threshold)
CHECK_INTERVAL = 50      # solver/lp/pdhg.py:207 = max(10, min(PDHG_RESTART_PERIOD=50, 100))
RESTART_FACTOR = 0.5     # solver/lp/pdhg.py:238
DEFAULT_MAX_ITERS = 100_000   # solver/config.py:37
DEFAULT_TOL = 1e-6            # solver/config.py:12


@dataclass
class StdForm:
    """Equality standard form ``min cᵀz, A z = b, z ≥ 0`` of a box-form LP.

    Column layout: original variables shifted by their finite lower bound,
    then one slack per ≤ row (original ≤ rows first, then one row per finite
    upper bound, in column order).  ``neg`` marks rows that were negated
    because their shifted rhs was below −1e-6.
    """
    c: np.ndarray
    A: sp.csr_matrix
    b: np.ndarray
    lb_shift: np.ndarray     # finite part of lb (0 where lb = −inf)
    n_orig: int
    m_ub: int
    ub_cols: np.ndarray      # columns that received an upper-bound row
    neg: np.ndarray          # bool, per std row


def to_standard_form(problem) -> StdForm:
    n = problem.n_vars
    m_ub, m_eq = problem.n_ineq, problem.n_eq
    lb_shift = np.where(np.isfinite(problem.lb), problem.lb, 0.0)
    A_ub = sp.csr_matrix(problem.A_ub, dtype=float)
    A_eq = sp.csr_matrix(problem.A_eq, dtype=float)
    rhs_ub = np.asarray(problem.b_ub, float) - A_ub @ lb_shift
    rhs_eq = np.asarray(problem.b_eq, float) - A_eq @ lb_shift

    ub_cols = np.flatnonzero(np.isfinite(problem.ub))
    k = ub_cols.size
    if k:
        bound_rows = sp.csr_matrix((np.ones(k), (np.arange(k), ub_cols)), shape=(k, n))
        A_le = sp.vstack([A_ub, bound_rows], format="csr")
        rhs_le = np.concatenate([rhs_ub, (problem.ub - lb_shift)[ub_cols]])
    else:
        A_le, rhs_le = A_ub, rhs_ub
    m_le = A_le.shape[0]
    n_full = n + m_le

    blocks = []
    if m_le:
        blocks.append(sp.hstack([A_le, sp.identity(m_le, format="csr")], format="csr"))
    if m_eq:
        blocks.append(sp.hstack([A_eq, sp.csr_matrix((m_eq, m_le))], format="csr"))
    A = sp.vstack(blocks, format="csr") if blocks else sp.csr_matrix((0, n_full))
    b = np.concatenate([rhs_le, rhs_eq])

    neg = b < -FEAS_TOL
    if neg.any():
        A = sp.csr_matrix(sp.diags(np.where(neg, -1.0, 1.0)) @ A)
        b = np.where(neg, -b, b)
    c = np.concatenate([np.asarray(problem.c, float), np.zeros(m_le)])
    A.sort_indices()
    return StdForm(c=c, A=A, b=b, lb_shift=lb_shift, n_orig=n, m_ub=m_ub,
                   ub_cols=ub_cols, neg=neg)


def diagonal_steps(A: sp.csr_matrix) -> tuple[np.ndarray, np.ndarray]:
    """τ_j = 0.999 / max(Σ_i|A_ij|, 1e-4),  σ_i = 0.999 / max(Σ_j|A_ij|, 1e-4)."""
    absA = abs(A)
    col = np.asarray(absA.sum(axis=0)).ravel()
    row = np.asarray(absA.sum(axis=1)).ravel()
    return 0.999 / np.maximum(col, 1e-4), 0.999 / np.maximum(row, 1e-4)


def kkt_error(A, AT, b, c, x, y, norm_b=None, norm_c=None):
    """Reference KKT error of a std-form pair: (err, rp, rd, gap)."""
    if norm_b is None:
        norm_b = max(1.0, float(np.linalg.norm(b)))
    if norm_c is None:
        norm_c = max(1.0, float(np.linalg.norm(c)))
    rp = float(np.linalg.norm(A @ x - b)) / norm_b
    red = c - AT @ y
    rd = float(np.linalg.norm(np.minimum(red, 0.0))) / norm_c
    po, do = float(c @ x), float(b @ y)
    gap = abs(po - do) / (1.0 + abs(po) + abs(do))
    return max(rp, rd, gap), rp, rd, gap


@dataclass
class RefResult:
    status: str
    x: np.ndarray            # original space, clipped to bounds
    objective: float         # original sense
    iterations: int
    z: np.ndarray = None     # final std-form primal (the returned point)
    w: np.ndarray = None     # final std-form dual
    restarts: int = 0
    kkt_history: list = field(default_factory=list)   # (iteration, err) at each check
    std: StdForm = None


def solve(problem, max_iters: int = DEFAULT_MAX_ITERS, tol: float = DEFAULT_TOL,
          record_history: bool = False) -> RefResult:
    """Restarted PDHG exactly as the reference runs it (FP64)."""
    std = to_standard_form(problem)
    A, b, c = std.A, std.b, std.c
    m, n = A.shape
    if m == 0 or n == 0:
        return RefResult("optimal", np.zeros(problem.n_vars), 0.0, 0, std=std)

    tau, sigma = diagonal_steps(A)
    AT = A.T.tocsr()
    nb = max(1.0, float(np.linalg.norm(b)))
    nc = max(1.0, float(np.linalg.norm(c)))

    z = np.zeros(n)
    w = np.zeros(m)
    z_acc = np.zeros(n)
    w_acc = np.zeros(m)
    win = 0
    last_err = kkt_error(A, AT, b, c, z, w, nb, nc)[0]
    status = "iteration_limit"
    restarts = 0
    hist = []
    it = 0
    for it in range(1, max_iters + 1):
        z_next = np.maximum(z - tau * (c - AT @ w), 0.0)
        w = w + sigma * (b - A @ (2.0 * z_next - z))
        z = z_next
        z_acc += z
        w_acc += w
        win += 1
        if win % CHECK_INTERVAL == 0:
            z_avg = z_acc / win
            w_avg = w_acc / win
            err = kkt_error(A, AT, b, c, z_avg, w_avg, nb, nc)[0]
            if record_history:
                hist.append((it, err))
            if err < tol:
                z, w = z_avg, w_avg
                status = "optimal"
                break
            if err < RESTART_FACTOR * last_err:
                z, w = z_avg.copy(), w_avg.copy()
                z_acc[:] = 0.0
                w_acc[:] = 0.0
                win = 0
                last_err = err
                restarts += 1

    x = recover_x(problem, std, z)
    obj = float(np.asarray(problem.c, float) @ x)
    if problem.sense == "max":
        obj = -obj
    return RefResult(status, x, obj, it, z=z, w=w, restarts=restarts, kkt_history=hist, std=std)


def recover_x(problem, std: StdForm, z: np.ndarray) -> np.ndarray:
    """Original-space x from std-form z (``solver/lp/pdhg.py:247-253``)."""
    x = z[:std.n_orig] + std.lb_shift
    lo = np.where(np.isfinite(problem.lb), problem.lb, -1e30)
    hi = np.where(np.isfinite(problem.ub), problem.ub, 1e30)
    return np.clip(x, lo, hi)
