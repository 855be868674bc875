"""FP64 KKT evaluators — TEST INFRASTRUCTURE ONLY.

Two error measures for a primal/dual pair of the box-form LP

    min cᵀx  s.t.  A_ub x ≤ b_ub,  A_eq x = b_eq,  lb ≤ x ≤ ub

with duals ``y`` on the stacked rows K = [A_ub; A_eq] under the Lagrangian
cᵀx − yᵀ(Kx − rhs) (so y ≤ 0 on ≤ rows):

``box_rel_kkt``  the relative KKT error the GPU engine reports:
                 rp = ‖(Kx − rhs) with ≤ rows clipped at 0‖ / (1 + ‖rhs‖),
                 rd = ‖r − λ‖ / (1 + ‖c‖), r = c − Kᵀy, λ = projection of r
                 on the cone the bounds allow, plus any y > 0 on ≤ rows,
                 gap = |cᵀx − d(y)| / (1 + |cᵀx| + |d(y)|),
                 d(y) = rhsᵀy + Σ lb_j λ_j⁺ − Σ ub_j λ_j⁻.

                 With ``form="pdlp"`` a finite bound farther from x_j than |x_j|
                 is left out of λ's cone and of d(y), so the part of r_j it
                 would absorb counts as dual residual (PDLP's default handling
                 of far bounds; the engine's ``kkt_form="pdlp"``).

``ref_form_error`` the reference's own error (``solver/lp/pdhg.py:181-196``)
                 after mapping (x, y) into the reference standard form
                 (``pdhg.py:62-125``): shifted x, slacks max(b − A_ub x, 0),
                 upper-bound slacks max(ub − x, 0), upper-bound-row duals
                 min(0, r_j), dual signs flipped on negated rows.
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp

from . import pdhg_ref


def stacked(problem):
    K = sp.vstack([sp.csr_matrix(problem.A_ub, dtype=float),
                   sp.csr_matrix(problem.A_eq, dtype=float)], format="csr")
    rhs = np.concatenate([np.asarray(problem.b_ub, float), np.asarray(problem.b_eq, float)])
    return K, rhs


def box_rel_kkt(problem, x, y, K=None, rhs=None, form="lagrangian") -> dict:
    if K is None:
        K, rhs = stacked(problem)
    x = np.asarray(x, float)
    y = np.asarray(y, float)
    c = np.asarray(problem.c, float)
    lb, ub = np.asarray(problem.lb, float), np.asarray(problem.ub, float)
    m_ub = problem.n_ineq
    res = K @ x - rhs
    res[:m_ub] = np.maximum(res[:m_ub], 0.0)
    rp = float(np.linalg.norm(res)) / (1.0 + float(np.linalg.norm(rhs)))

    r = c - K.T @ y
    has_l, has_u = np.isfinite(lb), np.isfinite(ub)
    if form == "pdlp":
        with np.errstate(invalid="ignore"):
            has_l = has_l & (np.abs(x - lb) <= np.abs(x))
            has_u = has_u & (np.abs(x - ub) <= np.abs(x))
    elif form != "lagrangian":
        raise ValueError(form)
    lam = np.where(has_l & has_u, r,
          np.where(has_l, np.maximum(r, 0.0), np.where(has_u, np.minimum(r, 0.0), 0.0)))
    dres = np.concatenate([r - lam, np.maximum(y[:m_ub], 0.0)])
    rd = float(np.linalg.norm(dres)) / (1.0 + float(np.linalg.norm(c)))

    pobj = float(c @ x)
    dobj = float(rhs @ y)
    dobj += float(np.sum(np.where(has_l, lb, 0.0) * np.maximum(lam, 0.0)))
    dobj += float(np.sum(np.where(has_u, ub, 0.0) * np.minimum(lam, 0.0)))
    gap = abs(pobj - dobj) / (1.0 + abs(pobj) + abs(dobj))
    return {"err": max(rp, rd, gap), "rp": rp, "rd": rd, "gap": gap,
            "pobj": pobj, "dobj": dobj}


def to_std_pair(problem, x, y, std=None):
    """Map a box-form pair into the reference standard form: (std, z, w)."""
    if std is None:
        std = pdhg_ref.to_standard_form(problem)
    x = np.asarray(x, float)
    y = np.asarray(y, float)
    m_ub = problem.n_ineq
    A_ub = sp.csr_matrix(problem.A_ub, dtype=float)
    z_x = np.maximum(x - std.lb_shift, 0.0)
    s_ub = np.maximum(np.asarray(problem.b_ub, float) - A_ub @ x, 0.0)
    t_ub = np.maximum(np.asarray(problem.ub, float)[std.ub_cols] - x[std.ub_cols], 0.0)
    z = np.concatenate([z_x, s_ub, t_ub])

    K, _ = stacked(problem)
    r = np.asarray(problem.c, float) - K.T @ y
    w_bound = np.minimum(r[std.ub_cols], 0.0)
    w = np.concatenate([y[:m_ub], w_bound, y[m_ub:]])
    w = np.where(std.neg, -w, w)
    return std, z, w


def ref_form_error(problem, x, y, std=None) -> dict:
    std, z, w = to_std_pair(problem, x, y, std)
    A = std.A
    err, rp, rd, gap = pdhg_ref.kkt_error(A, A.T.tocsr(), std.b, std.c, z, w)
    return {"err": err, "rp": rp, "rd": rd, "gap": gap}
