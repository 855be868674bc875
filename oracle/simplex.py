"""FP64 bounded revised simplex — TEST INFRASTRUCTURE ONLY (the objective oracle).

Solves the box-form LP the engine takes,

    min c^T x   s.t.  A_ub x <= b_ub,  A_eq x = b_eq,  lb <= x <= ub,

exactly (to round-off) on small problems, so PDHG objectives can be compared
with an optimum this repository computes itself.  Algorithm (textbook bounded
revised simplex, two phases):

* variables are shifted / mirrored / split so that every column has bounds
  [0, u] (u may be +inf), a slack is added to every '<=' row, and rows are
  signed so that the right-hand side is non-negative;
* phase 1 minimises the sum of one artificial per row from the all-artificial
  basis; phase 2 minimises c from the phase-1 basis with the artificials fixed
  at zero;
* each iteration refactors the basis (dense LU), prices all nonbasic columns
  (Dantzig's rule, Bland's rule after a run of degenerate pivots), and takes
  the bounded ratio test, including a bound flip of the entering column.

The basis is dense (LU of m x m, meant for m up to a few hundred rows); the
constraint matrix stays sparse, so pricing costs O(nnz) per iteration.  Phase 1
starts from a slack basis where a row's slack has coefficient +1 (its
artificial only where it has none), and a bound flip keeps the factorization.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import scipy.linalg as la
import scipy.sparse as sp


@dataclass
class SimplexResult:
    status: str                 # "optimal", "infeasible", "unbounded", "iteration_limit"
    x: np.ndarray               # original variables
    objective: float            # c^T x in the problem's sense
    iterations: int


def _standardize(problem):
    """Columns z >= 0 with upper bounds u, rows [A_ub | I; A_eq | 0] z = b.
    Returns (A dense, b, c, u, recover(z) -> x, constant objective offset)."""
    c0 = np.asarray(problem.c, float)
    lb = np.asarray(problem.lb, float)
    ub = np.asarray(problem.ub, float)
    n = c0.size
    K = sp.vstack([sp.csr_matrix(problem.A_ub), sp.csr_matrix(problem.A_eq)]).tocsc()
    rhs = np.concatenate([np.asarray(problem.b_ub, float), np.asarray(problem.b_eq, float)])
    m_ub = problem.A_ub.shape[0]
    costs, uppers, maps = [], [], []                 # maps: (orig j, sign, shift)
    src, sign = [], []                               # column of K and its sign
    shift = np.zeros(n)                              # x_j's value at z = 0 (0 for free columns)
    const = 0.0
    for j in range(n):
        if np.isfinite(lb[j]):                       # x = lb + z, z in [0, ub - lb]
            src.append(j); sign.append(1.0); costs.append(c0[j]); uppers.append(ub[j] - lb[j])
            maps.append((j, 1.0, lb[j])); shift[j] = lb[j]
            const += c0[j] * lb[j]
        elif np.isfinite(ub[j]):                     # x = ub - z, z >= 0
            src.append(j); sign.append(-1.0); costs.append(-c0[j]); uppers.append(np.inf)
            maps.append((j, -1.0, ub[j])); shift[j] = ub[j]
            const += c0[j] * ub[j]
        else:                                        # free: x = z+ - z-
            src.append(j); sign.append(1.0); costs.append(c0[j]); uppers.append(np.inf); maps.append((j, 1.0, 0.0))
            src.append(j); sign.append(-1.0); costs.append(-c0[j]); uppers.append(np.inf); maps.append((j, -1.0, 0.0))
    Z = K[:, src] @ sp.diags(np.asarray(sign, float)) if src else sp.csc_matrix((rhs.size, 0))
    S = sp.eye(rhs.size, m_ub, format="csc")        # slacks of the '<=' rows
    costs += [0.0] * m_ub
    uppers += [np.inf] * m_ub
    maps += [(-1, 0.0, 0.0)] * m_ub
    b = rhs - K @ shift
    sgn = np.where(b < 0, -1.0, 1.0)
    A = (sp.diags(sgn) @ sp.hstack([Z, S], format="csc")).tocsc()
    b = b * sgn

    def recover(z):
        x = np.zeros(n)
        for k, (j, s, sh) in enumerate(maps):
            if j < 0:
                continue
            if s == 1.0 and sh == 0.0 and not np.isfinite(lb[j]):
                x[j] += z[k]
            elif s == -1.0 and sh == 0.0 and not np.isfinite(lb[j]) and not np.isfinite(ub[j]):
                x[j] -= z[k]
            else:
                x[j] = sh + s * z[k]
        return x

    return A, b, np.asarray(costs, float), np.asarray(uppers, float), recover, const


def _simplex(A, b, c, u, basis, at_upper, max_iters, tol=1e-9):
    """Bounded revised simplex from a feasible basis.  `at_upper` marks nonbasic
    columns held at their (finite) upper bound.  Returns (status, z, basis, iters)."""
    m, N = A.shape
    A = sp.csc_matrix(A)
    AT = A.T.tocsr()
    basis = list(basis)
    in_basis = np.zeros(N, bool)
    in_basis[basis] = True
    degenerate = 0
    lu = None
    for it in range(max_iters):
        if lu is None:                               # refactor after a basis change only
            lu = la.lu_factor(A[:, basis].toarray())
            pi = la.lu_solve(lu, c[basis], trans=1)
            d = c - AT @ pi
        zN = np.where(at_upper, u, 0.0)
        zN[in_basis] = 0.0
        xB = la.lu_solve(lu, b - A @ zN)
        d[in_basis] = 0.0
        # candidates: at lower with d < 0, at upper with d > 0
        score = np.where(at_upper, d, -d)
        score[in_basis] = -np.inf
        score[u <= 0.0] = -np.inf                   # fixed columns (phase-2 artificials) never enter
        if degenerate > 50:                         # Bland: smallest eligible index
            elig = np.flatnonzero(score > tol)
            q = int(elig[0]) if elig.size else -1
        else:
            q = int(np.argmax(score)) if N else -1
            if q >= 0 and score[q] <= tol:
                q = -1
        if q < 0:
            z = zN.copy()
            z[basis] = xB
            return "optimal", z, basis, it
        w = la.lu_solve(lu, A[:, [q]].toarray().ravel())
        dirn = -1.0 if at_upper[q] else 1.0         # entering column moves up from 0 or down from u
        # x_B(t) = x_B - t * dirn * w
        step = dirn * w
        t_max = u[q] if np.isfinite(u[q]) else np.inf
        leave, leave_to_upper = -1, False
        # ratio test: pivots below a relative tolerance are ignored; among ratios
        # within 1e-12 of the smallest, the largest pivot leaves (stability)
        ptol = 1e-9 * max(1.0, float(np.abs(step).max()) if m else 1.0)
        ub_b = u[basis]
        with np.errstate(divide="ignore", invalid="ignore"):
            t_low = np.where(step > ptol, np.maximum(xB, 0.0) / step, np.inf)                 # basic hits 0
            t_up = np.where((step < -ptol) & np.isfinite(ub_b), np.minimum(xB - ub_b, 0.0) / step, np.inf)
        t_all = np.minimum(t_low, t_up)
        best = t_max
        if m:
            t_min = float(t_all.min())
            if t_min < best:
                near = np.flatnonzero(t_all <= t_min + 1e-12 * (1.0 + t_min))
                i = int(near[np.argmax(np.abs(step[near]))])
                best, leave, leave_to_upper = t_all[i], i, bool(t_up[i] < t_low[i])
        if not np.isfinite(best):
            return "unbounded", None, basis, it
        degenerate = degenerate + 1 if best <= tol else 0
        if leave < 0:                                # bound flip of the entering column
            at_upper[q] = not at_upper[q]
            continue
        out = basis[leave]
        basis[leave] = q
        in_basis[out] = False
        in_basis[q] = True
        at_upper[q] = False
        at_upper[out] = leave_to_upper
        lu = None
    return "iteration_limit", None, basis, max_iters


def solve(problem, max_iters: int = 50000) -> SimplexResult:
    """Optimal vertex of a small LP (status and x in the problem's variables)."""
    A, b, c, u, recover, _const = _standardize(problem)
    m, N = A.shape
    n = np.asarray(problem.c).size
    if m == 0:
        z = np.where(c < 0, u, 0.0)
        if np.any((c < 0) & ~np.isfinite(u)):
            return SimplexResult("unbounded", np.zeros(n), -np.inf, 0)
        x = recover(z)
        return SimplexResult("optimal", x, float(np.asarray(problem.c) @ x), 0)
    # phase 1: one artificial per row (identity); the starting basis takes a
    # row's slack where its coefficient is +1 (feasible at b >= 0), else the
    # row's artificial
    A1 = sp.hstack([A, sp.eye(m, format="csc")], format="csc")
    u1 = np.concatenate([u, np.full(m, np.inf)])
    c1 = np.concatenate([np.zeros(N), np.ones(m)])
    at_upper = np.zeros(N + m, bool)
    start = list(range(N, N + m))
    m_ub = problem.A_ub.shape[0]
    for i in range(m_ub):
        k = N - m_ub + i                             # slack of row i (the last m_ub columns)
        if A[i, k] > 0:
            start[i] = k
    st, z1, basis, it1 = _simplex(A1, b, c1, u1, start, at_upper, max_iters)
    if st != "optimal":
        return SimplexResult(st, np.zeros(n), np.nan, it1)
    if z1[N:].sum() > 1e-7 * max(1.0, np.abs(b).max()):
        return SimplexResult("infeasible", np.zeros(n), np.nan, it1)
    # phase 2: artificials stay (at zero) only where they are still basic
    u2 = u1.copy()
    u2[N:] = 0.0
    c2 = np.concatenate([c, np.zeros(m)])
    st, z2, basis, it2 = _simplex(A1, b, c2, u2, basis, at_upper, max_iters - it1)
    if st != "optimal":
        return SimplexResult(st, np.zeros(n), np.nan, it1 + it2)
    x = recover(z2[:N])
    obj = float(np.asarray(problem.c, float) @ x)
    if getattr(problem, "sense", "min") == "max":
        obj = -obj
    return SimplexResult("optimal", x, obj, it1 + it2)
