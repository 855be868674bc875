"""CPU restatement of the GPU engine's adaptive mode — TEST INFRASTRUCTURE ONLY.

Same rules as ``SPS_MODE_ADAPTIVE`` (box form, 10 Ruiz + 1 Pock-Chambolle
passes, η₀ = 1/max|K̃|, ω₀ = ‖c̃‖/‖b̃‖, adaptive step, step-weighted averages,
KKT check of average and current every 64 attempts, restart to the better one
on 0.2 / 0.8 / 0.36 criteria, primal-weight update at restarts, termination on
the original problem's relative KKT error, infeasibility and unboundedness
certificates from the change since the last restart), in a chosen iterate
precision.
Used to check the engine's trajectory on small problems and to study the
effect of the iterate precision.

``interaction``: "difference" forms K Δx as K x' − K x of the two products (as
the engine does), "direct" forms it as K (x' − x).

The averages are kept as the engine keeps them, as offsets from the restart
point (x̄ = x_last + Σ w_k (x_k − x_last) / Σ w_k): with FP32 iterates a plain
FP32 sum Σ w_k x_k loses the digits that the restart tests need near
convergence and the method stalls near KKT 1e-3 on some planted LPs, which
the offset form (and FP64 sums) avoid.
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp

from . import kkt


def scale(K: sp.csr_matrix, ruiz: int = 10):
    m, n = K.shape
    dr, dc = np.ones(m), np.ones(n)
    A = abs(K).tocsr()
    for it in range(ruiz + 1):
        S = sp.diags(dr) @ A @ sp.diags(dc)
        if it < ruiz:
            rs = np.asarray(S.max(axis=1).todense()).ravel()
            cs = np.asarray(S.max(axis=0).todense()).ravel()
        else:
            rs = np.asarray(S.sum(axis=1)).ravel()
            cs = np.asarray(S.sum(axis=0)).ravel()
        dr = np.where(rs > 0, dr / np.sqrt(np.where(rs > 0, rs, 1)), dr)
        dc = np.where(cs > 0, dc / np.sqrt(np.where(cs > 0, cs, 1)), dc)
    return dr, dc


RAY_TOL = 1e-6   # a certificate's residual must be at most this fraction of its objective


def ray_status(Ks, KT, c, b, lo, hi, le, dx, dy):
    """Infeasibility / unboundedness test on the change (dx, dy) of the current
    iterate since the last restart, in the scaled space, as the engine's check
    takes it (``csrc/decide.cuh`` ``decide_check``): dy is a Farkas certificate
    when b^T dy plus the bound terms of lambda = -K^T dy is positive and dy's
    violation of the dual cone together with lambda's cone residual is at most
    RAY_TOL of it; dx is an improving ray when c^T dx < 0 and K dx's violation
    of the row cones together with dx's violation of the bounds' recession cone
    is at most RAY_TOL of |c^T dx|.  Returns "infeasible", "unbounded" or None."""
    hl, hh = np.isfinite(lo), np.isfinite(hi)
    kdx = Ks.astype(float) @ dx
    kdx[le] = np.maximum(kdx[le], 0.0)
    dyv = np.where(le, np.maximum(dy, 0.0), 0.0)
    lr = -(KT.astype(float) @ dy)
    lp = np.where(hl & hh, lr, np.where(hl, np.maximum(lr, 0.0), np.where(hh, np.minimum(lr, 0.0), 0.0)))
    bound = float(np.sum(np.where(hl, lo, 0.0) * np.maximum(lp, 0.0)) + np.sum(np.where(hh, hi, 0.0) * np.minimum(lp, 0.0)))
    dual_obj = float(b.astype(float) @ dy) + bound
    if dual_obj > 0.0 and np.sqrt(float((lr - lp) @ (lr - lp)) + float(dyv @ dyv)) <= RAY_TOL * dual_obj:
        return "infeasible"
    vx = np.where(hl & hh, dx, np.where(hl, np.minimum(dx, 0.0), np.where(hh, np.maximum(dx, 0.0), 0.0)))
    cdx = float(c.astype(float) @ dx)
    if cdx < 0.0 and np.sqrt(float(kdx @ kdx) + float(vx @ vx)) <= RAY_TOL * (-cdx):
        return "unbounded"
    return None


def solve(problem, tol=1e-4, max_iters=100000, dtype=np.float32, interaction="direct", check=64,
          kkt_form="lagrangian"):
    K, rhs = kkt.stacked(problem)
    m_ub = problem.n_ineq
    m, n = K.shape
    dr, dc = scale(K)
    Ks = (sp.diags(dr) @ K @ sp.diags(dc)).tocsr().astype(dtype)
    KT = Ks.T.tocsr()
    c = (np.asarray(problem.c, float) * dc).astype(dtype)
    b = (rhs * dr).astype(dtype)
    lo = (np.asarray(problem.lb, float) / dc).astype(dtype)
    hi = (np.asarray(problem.ub, float) / dc).astype(dtype)
    le = np.zeros(m, bool)
    le[:m_ub] = True
    eta = 1.0 / float(abs(Ks).max())
    nc2, nb2 = float(np.dot(c.astype(float), c)), float(np.dot(b.astype(float), b))
    omega = np.sqrt(nc2) / np.sqrt(nb2) if nc2 > 1e-20 and nb2 > 1e-20 else 1.0
    x = np.clip(np.zeros(n, dtype), lo, hi)
    y = np.zeros(m, dtype)
    ax = (Ks @ x).astype(dtype)
    aty = np.zeros(n, dtype)
    xs, ys, wsum = np.zeros(n, dtype), np.zeros(m, dtype), 0.0
    xl, yl = x.copy(), y.copy()
    k, window, restarts = 0, 0, 0
    inv_nb, inv_nc = 1 / (1 + np.linalg.norm(rhs)), 1 / (1 + np.linalg.norm(problem.c))

    def metrics(xv, yv):
        axv = Ks.astype(float) @ xv.astype(float)
        res = axv - b
        res[le] = np.maximum(res[le], 0)
        rc = c.astype(float) - KT.astype(float) @ yv.astype(float)
        hl, hh = np.isfinite(lo), np.isfinite(hi)
        if kkt_form == "pdlp":      # far finite bounds (|x - bound| > |x|) leave the dual objective
            xf = xv.astype(float)
            hl = hl & (np.abs(xf - lo) <= np.abs(xf))
            hh = hh & (np.abs(xf - hi) <= np.abs(xf))
        lam = np.where(hl & hh, rc, np.where(hl, np.maximum(rc, 0), np.where(hh, np.minimum(rc, 0), 0)))
        dres = rc - lam
        po = float(c.astype(float) @ xv)
        do = float(b.astype(float) @ yv) + float(np.sum(np.where(hl, lo, 0) * np.maximum(lam, 0))) \
            + float(np.sum(np.where(hh, hi, 0) * np.minimum(lam, 0)))
        rp = np.linalg.norm(res / dr) * inv_nb
        rd = np.linalg.norm(dres / dc) * inv_nc
        gap = abs(po - do) / (1 + abs(po) + abs(do))
        kw = np.sqrt(omega ** 2 * float(res @ res) + float(dres @ dres) / omega ** 2 + (po - do) ** 2)
        return max(rp, rd, gap), kw, axv, KT.astype(float) @ yv.astype(float)

    _, kw0, _, _ = metrics(x, y)
    kkt_last = kkt_prev = kw0
    status = "iteration_limit"
    while k < max_iters:
        for _ in range(check):
            if k >= max_iters:
                break
            tau, sigma = dtype(eta / omega), dtype(eta * omega)
            x2 = np.clip(x - tau * (c - aty), lo, hi).astype(dtype)
            ax2 = (Ks @ x2).astype(dtype)
            y2 = (y + sigma * (b - (ax2 + ax2 - ax))).astype(dtype)
            y2[le] = np.minimum(y2[le], 0)
            dx, dy = (x2 - x).astype(float), (y2 - y).astype(float)
            kdx = (ax2 - ax).astype(float) if interaction == "difference" else Ks.astype(float) @ dx
            inter = abs(float(dy @ kdx))
            move = omega * float(dx @ dx) + float(dy @ dy) / omega
            k += 1
            window += 1
            lim = move / (2 * inter) if inter > 0 else np.inf
            nxt = min((1 - (k + 1) ** -0.3) * lim, (1 + (k + 1) ** -0.6) * eta)
            if eta <= lim or move == 0:
                xs = (xs + dtype(eta) * (x2 - xl)).astype(dtype)
                ys = (ys + dtype(eta) * (y2 - yl)).astype(dtype)
                wsum += eta
                x, y, ax = x2, y2, ax2
                aty = (KT @ y).astype(dtype)
            eta = nxt
        has_avg = wsum > 0
        xa = (xl + xs.astype(float) / wsum).astype(dtype) if has_avg else x
        ya = (yl + ys.astype(float) / wsum).astype(dtype) if has_avg else y
        ea, ka, axa, atya = metrics(xa, ya)
        ec, kc_, _, _ = metrics(x, y)
        best_avg = has_avg and ea < ec
        optimal = min(ea if has_avg else np.inf, ec) < tol
        ray = None if optimal else ray_status(Ks, KT, c, b, lo, hi, le, (x - xl).astype(float),
                                              (y - yl).astype(float))
        if optimal or ray or k >= max_iters:
            if best_avg:
                x, y = xa, ya
            status = "optimal" if optimal else ray or "iteration_limit"
            break
        cand_avg = has_avg and ka < kc_
        kc = ka if cand_avg else kc_
        restart = kc <= 0.2 * kkt_last or (kc <= 0.8 * kkt_last and kc > kkt_prev) or window >= 0.36 * k
        kkt_prev = kc
        if restart:
            xc, yc = (xa, ya) if cand_avg else (x, y)
            ddx, ddy = np.linalg.norm((xc - xl).astype(float)), np.linalg.norm((yc - yl).astype(float))
            if ddx > 1e-10 and ddy > 1e-10:
                omega = float(np.exp(0.5 * np.log(ddy / ddx) + 0.5 * np.log(omega)))
            if cand_avg:
                x, y = xa, ya
                ax, aty = axa.astype(dtype), atya.astype(dtype)
            xl, yl = x.copy(), y.copy()
            xs[:] = 0
            ys[:] = 0
            wsum = 0.0
            kkt_last = kkt_prev = kc
            restarts += 1
            window = 0
    xo = x.astype(float) * dc
    yo = y.astype(float) * dr
    return {"status": status, "iterations": k, "x": xo, "y": yo, "restarts": restarts,
            "kkt": kkt.box_rel_kkt(problem, np.clip(xo, problem.lb, problem.ub), yo, form=kkt_form)}
