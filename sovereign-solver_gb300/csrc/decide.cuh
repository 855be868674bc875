// decide.cuh — the scalar decisions of adaptive restarted PDHG, shared by the
// single-LP kernels (taken by a kernel's last block) and the batched kernel
// (taken by thread 0 of the block that owns an instance).  All FP64.
#pragma once

#include "engine.cuh"
#include "../../include/sps_pdhg.h"

namespace sps {

enum ApplyBits { AP_LOAD_AVG = 1, AP_RESTART = 2, AP_CANDIDATE = 4, AP_STEP_PENDING = 8,
                 AP_SAVE_BEST = 16,   // copy the best point of this check to xb / yb
                 AP_SAVE_AVG = 32 };  // ... and that point is the average

// Stall test: the best relative KKT error has not halved for
// max(kStallMin, anchor / 2) attempts, anchor = attempt of the last halving.
// With a ceiling (Ctl::stall_ceiling) only an error at or below it can stall,
// and the count starts again when the error first reaches it: above it a
// plateau is the method's slow progress, not the FP32 precision floor.
constexpr int64_t kStallMin = 2048;
// The single-LP engine's ceiling.  FP32 iterates' error floor is far below it
// on any LP they can solve; above it FP64 only makes each attempt dearer (a
// 21M-nonzero power-law LP stalled at 1.3e-2 after 3 968 attempts: 13.7 s to
// 1e-4 with the FP64 continuation, 10.9 s in FP32 alone).
constexpr double kStallCeiling = 1e-3;
// Infeasibility tests on the change since the last restart (scaled space): a
// certificate's residual must be at most kRayTol of its objective.
constexpr double kRayTol = 1e-6;
// Partials of a check: column pass tc[kColPartials], row pass tr[kRowPartials].
constexpr int kColPartials = 14;
constexpr int kRowPartials = 11;
// With the PDLP error form the single-LP column check adds, per point q, the
// Lagrangian form's original-scale dual residual^2 (lag[q]) and bound terms
// (lag[2 + q]), so the returned point's Lagrangian error is reported too.
constexpr int kLagPartials = 4;

// Adaptive step (PDLP): limit = ||dz||_w^2 / (2 |dy^T K dx|); the attempt is
// accepted if eta <= limit; next eta = min((1 - (k+1)^-0.3) limit, (1 + (k+1)^-0.6) eta).
// Returns false (and marks the state done) when the movement is not finite.
__device__ __forceinline__ bool decide_step(Ctl& c, double dy2, double inter_signed) {
    const double w = c.omega, eta = c.eta, dx2 = c.dx2, inter = fabs(inter_signed);
    const double move = w * dx2 + dy2 / w;
    const int64_t k = c.iters + 1;
    if (!isfinite(move) || !isfinite(inter)) {
        c.done = 1;
        c.status = SPS_STATUS_NUMERIC_ERROR;
        c.iters = k;
        return false;
    }
    const double lim = inter > 0.0 ? move / (2.0 * inter) : INFINITY;
    const float kk = float(k + 1);
    const double next = fmin((1.0 - double(powf(kk, -0.3f))) * lim, (1.0 + double(powf(kk, -0.6f))) * eta);
    const bool acc = (eta <= lim) || move == 0.0;
    c.iters = k;
    c.window += 1;
    c.accepted = acc;
    if (acc) {
        c.cur = 1 - c.cur;
        c.eta_used = eta;
        c.w_sum += eta;
        c.accepted_total += 1;
    }
    c.eta = next;
    c.apply = AP_STEP_PENDING;
    return true;
}

// Check of the average (point 0) and the current iterate (point 1).
//   tr[4q + 0..3]: scaled primal residual^2, original primal residual^2, b^T y, ||y - y_last||^2
//   tc[5q + 0..4]: scaled dual residual^2, original dual residual^2, c^T x, bound terms, ||x - x_last||^2
// and, for the change (dx, dy) of the current iterate since the last restart
// (zeros where a caller does not compute them):
//   tr[8]: ||K dx||^2 on the row kinds' cones,  tr[9]: b^T dy,
//   tr[10]: violation^2 of dy against the dual cone (dy <= 0 on '<=' rows)
//   tc[10]: cone residual^2 of lambda = -K^T dy,  tc[11]: its bound terms,
//   tc[12]: violation^2 of dx against the bounds' recession cone,  tc[13]: c^T dx
// Termination on the relative KKT error of the original problem; restart on the
// weighted KKT of the scaled problem (to the better of average and current) when
// it dropped below 0.2x the last restart's, or below 0.8x while rising, or after
// 0.36x of all attempts; primal weight updated at restarts.  With c.stall_on the
// best point of every check that improves on all earlier ones is marked for
// copying (AP_SAVE_BEST, with the primal weight in c.omega_best) and the solve
// finishes with SPS_STATUS_STALLED when the best error stops halving (FP32
// precision floor; the host continues in FP64 from the saved point).  Sets c.apply.
__device__ __forceinline__ void decide_check(Ctl& c, const double (&tc)[kColPartials],
                                             const double (&tr)[kRowPartials], double inv_nb, double inv_nc,
                                             bool stop, const double* lag = nullptr) {
    const bool has_avg = c.w_sum > 0.0;
    const double w = c.omega;
    double rel[2], kw[2], rp[2], rd[2], gp[2], po[2], dob[2], rl[2];
    for (int q = 0; q < 2; ++q) {
        po[q] = tc[5 * q + 2];
        dob[q] = tr[4 * q + 2] + tc[5 * q + 3];
        rp[q] = sqrt(tr[4 * q + 1]) * inv_nb;
        rd[q] = sqrt(tc[5 * q + 1]) * inv_nc;
        gp[q] = fabs(po[q] - dob[q]) / (1.0 + fabs(po[q]) + fabs(dob[q]));
        rel[q] = fmax(rp[q], fmax(rd[q], gp[q]));
        const double g = po[q] - dob[q];
        kw[q] = sqrt(w * w * tr[4 * q + 0] + tc[5 * q + 0] / (w * w) + g * g);
        if (!isfinite(rel[q])) rel[q] = INFINITY;
        if (!isfinite(kw[q])) kw[q] = INFINITY;
        rl[q] = rel[q];
        if (lag) {
            const double dl = tr[4 * q + 2] + lag[2 + q];
            const double gl = fabs(po[q] - dl) / (1.0 + fabs(po[q]) + fabs(dl));
            rl[q] = fmax(rp[q], fmax(sqrt(lag[q]) * inv_nc, gl));
            if (!isfinite(rl[q])) rl[q] = INFINITY;
        }
    }
    c.last_avg_kkt = rel[0];
    c.last_cur_kkt = rel[1];
    if (c.init_phase) {
        c.init_phase = 0;
        c.anchor_rel = rel[1];
        c.anchor_iter = 0;
        c.best_rel = INFINITY;
        c.kkt_last = kw[1];
        c.kkt_prev_cand = kw[1];
        c.rel_kkt = rel[1]; c.rel_p = rp[1]; c.rel_d = rd[1]; c.rel_gap = gp[1];
        c.pobj = po[1]; c.dobj = dob[1]; c.rel_kkt_lagr = rl[1];
        c.apply = AP_CANDIDATE | AP_RESTART;   // the start point is the first restart point
        return;
    }
    const int best = (has_avg && rel[0] < rel[1]) ? 0 : 1;
    const bool bad = !isfinite(rel[1]) && !(has_avg && isfinite(rel[0]));
    bool stalled = false;
    int save = 0;
    if (c.stall_on && !bad) {
        const double r = rel[best];
        if (r < c.best_rel) {
            c.best_rel = r;
            c.omega_best = w;
            c.best_saved = 1;
            save = AP_SAVE_BEST | (best == 0 ? AP_SAVE_AVG : 0);
        }
        if (r <= 0.5 * c.anchor_rel || (c.anchor_rel > c.stall_ceiling && r <= c.stall_ceiling)) {
            c.anchor_rel = r;
            c.anchor_iter = c.iters;
        } else if (c.best_rel <= c.stall_ceiling &&
                   c.iters - c.anchor_iter >= (c.anchor_iter / 2 > kStallMin ? c.anchor_iter / 2 : kStallMin)) {
            stalled = true;
        }
    }
    bool finish = false;
    if (bad) {
        c.status = SPS_STATUS_NUMERIC_ERROR; finish = true;
    } else if (rel[best] < c.tol) {
        c.status = SPS_STATUS_OPTIMAL; finish = true;
    } else if (tr[9] + tc[11] > 0.0 && sqrt(tc[10] + tr[10]) <= kRayTol * (tr[9] + tc[11])) {
        // y's change is a Farkas ray: lambda = -K^T dy lies in the bounds' cone and the
        // dual objective of the ray, b^T dy + bound terms, is positive
        c.status = SPS_STATUS_INFEASIBLE; finish = true;
    } else if (tc[13] < 0.0 && sqrt(tr[8] + tc[12]) <= kRayTol * (-tc[13])) {
        // x's change is an improving ray: K dx on the row cones, dx in the recession cone, c^T dx < 0
        c.status = SPS_STATUS_UNBOUNDED; finish = true;
    } else if (c.iters >= c.max_iters) {
        c.status = SPS_STATUS_ITERATION_LIMIT; finish = true;
    } else if (stop) {
        c.status = SPS_STATUS_TIME_LIMIT; finish = true;
    } else if (stalled) {
        c.status = SPS_STATUS_STALLED; finish = true;
    }
    if (finish) {
        c.done = 1;
        c.choice = best == 0 ? 1 : 0;
        c.rel_kkt = rel[best]; c.rel_p = rp[best]; c.rel_d = rd[best]; c.rel_gap = gp[best];
        c.pobj = po[best]; c.dobj = dob[best]; c.rel_kkt_lagr = rl[best];
        c.apply = (best == 0 ? AP_LOAD_AVG : 0) | save;
        return;
    }
    const int cand = (has_avg && kw[0] < kw[1]) ? 0 : 1;
    const double kc = kw[cand];
    const bool restart = kc <= 0.2 * c.kkt_last || (kc <= 0.8 * c.kkt_last && kc > c.kkt_prev_cand) ||
                         double(c.window) >= 0.36 * double(c.iters);
    c.kkt_prev_cand = kc;
    int apply = 0;
    if (restart) {
        const double dx = sqrt(tc[5 * cand + 4]), dy = sqrt(tr[4 * cand + 3]);
        if (dx > 1e-10 && dy > 1e-10) {
            const double nw = exp(0.5 * log(dy / dx) + 0.5 * log(w));
            if (isfinite(nw) && nw > 0.0) c.omega = nw;
        }
        c.kkt_last = kc;
        c.kkt_prev_cand = kc;
        c.restarts += 1;
        c.window = 0;
        c.last_restart_iter = c.iters;
        apply = AP_RESTART | AP_CANDIDATE | (cand == 0 ? AP_LOAD_AVG : 0);
    }
    c.apply = apply | save;
}

}  // namespace sps
