// batch.cu — batched restarted PDHG (sps_batch_* in include/sps_pdhg.h).
//
// sps_batch_create packs thousands of box-form LPs (CSR of [A_ub; A_eq] plus a
// CSC built on the host by a per-instance counting sort, spread over host
// threads), uploads them once, and scales every instance on the device (one
// block per instance: 10 Ruiz passes + one Pock-Chambolle pass, FP64).
// sps_batch_solve is ONE persistent launch (captured once in a CUDA graph and
// replayed on later calls): each block takes the next-largest unsolved
// instance from an atomic counter and runs the whole adaptive PDHG loop on it
// with per-instance step size, primal weight, restarts and termination.
// The lanes-per-column of the column pass is chosen by a small autotuner that
// times the candidates on a sample of the batch.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <map>
#include <memory>
#include <mutex>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "batch.cuh"
#include "gnn_internal.cuh"
#include "nvtx.cuh"

namespace sps {
void set_create_error(const std::string& msg);
namespace batch {

// Gathers of iterate vectors.  In team mode (coh) the vector is written by
// other SMs during the launch, so it is read through L2 (__ldcg); a block on
// its own reads what it wrote itself and keeps the read-only path.
struct Gather1 {
    const float* x;
    bool coh;
    __device__ __forceinline__ float operator()(int, int j) const { return coh ? __ldcg(x + j) : __ldg(x + j); }
};

// Point 0 of a check is the average, kept as an offset from the restart point
// (x_last + x_sum / w_sum, x_sum = sum of w_k (x_k - x_last)) so that FP32 sums
// stay accurate near convergence; l = null when there is no average yet and
// point 0 aliases the current iterate.
__device__ __forceinline__ float ld_vec(const float* p, bool coh) { return coh ? __ldcg(p) : __ldg(p); }

// Gathers of the FP32 steps from a copy of the vector in shared memory (when
// it fits the 7168-float staging buffer): an instance's gathers are random,
// one 32-byte L1 sector (one L1 wavefront) per nonzero even on an L1 hit,
// while a warp's 32 random shared-memory reads cost a few bank cycles.
struct GatherS {
    const float* s;
    __device__ __forceinline__ float operator()(int, int j) const { return s[j]; }
};

// Copy x[0, n) into the staging buffer (coherent loads in a team, where other
// blocks wrote x).  The first barrier keeps the copy from overwriting entries
// the block's previous pass may still read.
__device__ __forceinline__ void stage_vector(float* s, const float* x, int n, bool coh) {
    __syncthreads();
    for (int j = threadIdx.x; j < n; j += kBlock) s[j] = ld_vec(x + j, coh);
    __syncthreads();
}

__device__ __forceinline__ double avg_at(const float* s, const float* l, double inv_w, int j, bool coh = false) {
    const double v = double(ld_vec(s + j, coh)) * inv_w;
    return l ? v + double(ld_vec(l + j, coh)) : v;
}

struct Gather2 {
    const float *s, *l, *x;
    double inv_w;
    bool coh;
    __device__ __forceinline__ double operator()(int q, int j) const {
        return q == 0 ? avg_at(s, l, inv_w, j, coh) : double(ld_vec(x + j, coh));
    }
};

struct StoreE {
    float* out;
    struct Pre {};
    __device__ __forceinline__ Pre pre(int) const { return Pre{}; }
    __device__ __forceinline__ void operator()(int r, const float (&acc)[1], const Pre&) { out[r] = acc[0]; }
};

// row pass of a step attempt: K x' and y' = proj(y + sigma (b - (2 K x' - K x)))
struct RowStepE {
    const float *b, *axo, *yo;
    const int8_t* kind;
    float *axn, *yn;
    float sigma;
    float dy2 = 0.f, inter = 0.f;
    struct Pre { float ao, yv, br; int kd; };
    __device__ __forceinline__ Pre pre(int r) const { return Pre{axo[r], yo[r], b[r], kind[r]}; }
    __device__ __forceinline__ void operator()(int r, const float (&acc)[1], const Pre& p) {
        const float ax = acc[0];
        axn[r] = ax;
        float y2 = p.yv + sigma * (p.br - (ax + ax - p.ao));
        if (p.kd) y2 = fminf(y2, 0.f);
        yn[r] = y2;
        const float dy = y2 - p.yv;
        dy2 += dy * dy;
        inter += dy * (ax - p.ao);
    }
};

// column pass of an accepted attempt: K^T y', averages, next candidate
struct ColStepE {
    const float *xc, *c, *lo, *hi, *xl;
    float *aty, *xn, *xs;
    float tau, wgt;
    float dx2 = 0.f;
    struct Pre { float xj, cj, l, h, s, r; };
    __device__ __forceinline__ Pre pre(int j) const { return Pre{xc[j], c[j], lo[j], hi[j], xs[j], xl[j]}; }
    __device__ __forceinline__ void operator()(int j, const float (&acc)[1], const Pre& p) {
        aty[j] = acc[0];
        xs[j] = p.s + wgt * (p.xj - p.r);
        const float x2 = fminf(fmaxf(p.xj - tau * (p.cj - acc[0]), p.l), p.h);
        xn[j] = x2;
        const float d = x2 - p.xj;
        dx2 += d * d;
    }
};

// The check epilogues accumulate their FP64 partials in the calling thread's
// own shared-memory slots (p[q * kBlock], q < 8 or 10) rather than registers:
// the check runs once per window and this keeps the step loops' register
// budget.  slot_sums() adds the slots in thread order.
struct RowCheckE {
    const float *b, *ys, *ylb, *yc, *yl;
    const double* dr;
    const int8_t* kind;
    float* axa;
    double inv_w;
    const float* axl;          // K x_last
    double* p;                 // this thread's slots
    struct Pre {};
    __device__ __forceinline__ Pre pre(int) const { return Pre{}; }
    __device__ __forceinline__ void operator()(int r, const double (&acc)[2], const Pre&) {
        const double br = b[r], d = dr[r];
        axa[r] = float(acc[0]);
        for (int q = 0; q < 2; ++q) {
            double res = acc[q] - br;
            if (kind[r]) res = fmax(res, 0.0);
            p[(4 * q + 0) * kBlock] += res * res;
            p[(4 * q + 1) * kBlock] += (res / d) * (res / d);
            const double yv = q == 0 ? avg_at(ys, ylb, inv_w, r) : double(yc[r]);
            p[(4 * q + 2) * kBlock] += br * yv;
            const double dd = yv - double(yl[r]);
            p[(4 * q + 3) * kBlock] += dd * dd;
        }
        double kdx = acc[1] - double(axl[r]);
        if (kind[r]) kdx = fmax(kdx, 0.0);
        p[8 * kBlock] += kdx * kdx;
        const double dy = double(yc[r]) - double(yl[r]);
        p[9 * kBlock] += br * dy;
        if (kind[r]) p[10 * kBlock] += fmax(dy, 0.0) * fmax(dy, 0.0);
    }
};

struct ColCheckE {
    const float *c, *lo, *hi, *xs, *xlb, *xc, *xl;
    const double* dc;
    float* atya;
    double inv_w;
    const float* atyl;         // K^T y_last
    double* p;                 // this thread's slots
    struct Pre {};
    __device__ __forceinline__ Pre pre(int) const { return Pre{}; }
    __device__ __forceinline__ void operator()(int j, const double (&acc)[2], const Pre&) {
        const double cj = c[j], d = dc[j], l = lo[j], h = hi[j];
        const bool hl = isfinite(l), hh = isfinite(h);
        atya[j] = float(acc[0]);
        for (int q = 0; q < 2; ++q) {
            const double rc = cj - acc[q];
            const double lam = (hl && hh) ? rc : hl ? fmax(rc, 0.0) : hh ? fmin(rc, 0.0) : 0.0;
            const double dres = rc - lam;
            p[(5 * q + 0) * kBlock] += dres * dres;
            p[(5 * q + 1) * kBlock] += (dres / d) * (dres / d);
            const double xv = q == 0 ? avg_at(xs, xlb, inv_w, j) : double(xc[j]);
            p[(5 * q + 2) * kBlock] += cj * xv;
            p[(5 * q + 3) * kBlock] += (hl ? l * fmax(lam, 0.0) : 0.0) + (hh ? h * fmin(lam, 0.0) : 0.0);
            const double dd = xv - double(xl[j]);
            p[(5 * q + 4) * kBlock] += dd * dd;
        }
        const double lr = -(acc[1] - double(atyl[j]));
        const double lp = (hl && hh) ? lr : hl ? fmax(lr, 0.0) : hh ? fmin(lr, 0.0) : 0.0;
        p[10 * kBlock] += (lr - lp) * (lr - lp);
        p[11 * kBlock] += (hl ? l * fmax(lp, 0.0) : 0.0) + (hh ? h * fmin(lp, 0.0) : 0.0);
        const double dx = double(xc[j]) - double(xl[j]);
        const double vx = (hl && hh) ? dx : hl ? fmin(dx, 0.0) : hh ? fmax(dx, 0.0) : 0.0;
        p[12 * kBlock] += vx * vx;
        p[13 * kBlock] += cj * dx;
    }
};

struct View {                 // one instance's arrays
    int n, m, G, Gr;              // lanes per column, lanes per row
    const int32_t *rptr, *ridx, *cptr, *cidx;
    const float *rval, *cval;
    const int8_t* kind;
    const float *c, *lo, *hi, *b;
    const double *dc, *dr;
    float *X[2], *ATY[2], *xs, *xl, *atya;
    float *Y[2], *AX[2], *ys, *yl, *axa;
    float *xb, *yb;
    float *axl, *atyl;
};

__device__ __forceinline__ View make_view(const Args& A, const Inst& I, int G) {
    const Arrays& a = A.a;
    View v;
    v.n = I.n; v.m = I.m; v.G = G & 0xFF; v.Gr = G >> 8 ? G >> 8 : 32;
    v.rptr = a.rptr + I.rp; v.ridx = a.ridx + I.re; v.rval = a.rval + I.re;
    v.cptr = a.cptr + I.cp; v.cidx = a.cidx + I.ce; v.cval = a.cval + I.ce;
    v.kind = a.kind + I.vr;
    v.c = a.c + I.vc; v.lo = a.lo + I.vc; v.hi = a.hi + I.vc; v.b = a.b + I.vr;
    v.dc = a.dc + I.vc; v.dr = a.dr + I.vr;
    v.X[0] = a.x0 + I.vc; v.X[1] = a.x1 + I.vc; v.ATY[0] = a.aty0 + I.vc; v.ATY[1] = a.aty1 + I.vc;
    v.xs = a.xs + I.vc; v.xl = a.xl + I.vc; v.atya = a.atya + I.vc;
    v.Y[0] = a.y0 + I.vr; v.Y[1] = a.y1 + I.vr; v.AX[0] = a.ax0 + I.vr; v.AX[1] = a.ax1 + I.vr;
    v.ys = a.ys + I.vr; v.yl = a.yl + I.vr; v.axa = a.axa + I.vr;
    v.xb = a.xb ? a.xb + I.vc : nullptr;
    v.yb = a.yb ? a.yb + I.vr : nullptr;
    v.axl = a.axl + I.vr;
    v.atyl = a.atyl + I.vc;
    return v;
}

// KKT check of average and current point, decision, and the restart copies.
// out[q] = sum over threads (in order) of slots[q * kBlock + t], q < N
template <int N>
__device__ __forceinline__ void slot_sums(const double* slots, double* out) {
    __syncthreads();
    if (threadIdx.x < N) {
        double t = 0.0;
        for (int k = 0; k < kBlock; ++k) t += slots[threadIdx.x * kBlock + k];
        out[threadIdx.x] = t;
    }
    __syncthreads();
}

// Element loops of a team.  A block owns exactly the rows (columns) its warps
// visit in the row (column) passes: chunks of CH = kWarps * (32 / lanes)
// consecutive elements, every size-th chunk from chunk `rank` on, so every
// per-row and per-column array is read and written by one block only (the
// gathers are the only reads across blocks).  The block's threads walk its
// owned elements densely; on its own (size 1) this is the identity.
#define TEAM_OWNED(var, count, CH)                                                                \
    for (int o_ = threadIdx.x, var; (var = (T.rank + (o_ / (CH)) * T.size) * (CH) + o_ % (CH)) < (count); \
         o_ += kBlock)

// Hand-off test of a check: the queue is empty, 7/8 of the launch's blocks have
// left, and this instance is large and has made kHandoffMin attempts.  Each
// block reads the idle counter itself; the team adds the blocks' votes, so all
// its blocks take the same decision.
struct Handoff {
    const uint32_t* idle;
    uint32_t need;
    bool eligible;            // instance large enough (and hand-off on)
};

__device__ bool check_and_apply(const View& v, const Inst& I, Ctl& c, double* sm, double* slots, const uint64_t* dl,
                                const Team& T, const Handoff& H) {
    __shared__ bool s_handoff;
    const int chc = kWarps * (32 / v.G), chr = kWarps * (32 / v.Gr);
    const uint64_t deadline = *dl;
    const bool has_avg = c.w_sum > 0.0;
    const double inv_w = has_avg ? 1.0 / c.w_sum : 1.0;
    const int cur = c.cur;
    double* mine = slots + threadIdx.x;
    for (int q = 0; q < kRowPartials; ++q) mine[q * kBlock] = 0.0;
    RowCheckE er{v.b, has_avg ? v.ys : v.Y[cur], has_avg ? v.yl : nullptr, v.Y[cur], v.yl, v.dr, v.kind, v.axa, inv_w,
                 v.axl, mine};
    group_rows_r<2, double>(v.Gr, v.rptr, v.ridx, v.rval, v.m,
                            Gather2{has_avg ? v.xs : v.X[cur], has_avg ? v.xl : nullptr, v.X[cur], inv_w, T.size > 1}, er,
                            T.rank, T.size);
    slot_sums<kRowPartials>(slots, sm);            // sm[0..10]: row partials
    for (int q = 0; q < kColPartials; ++q) mine[q * kBlock] = 0.0;
    ColCheckE ec{v.c, v.lo, v.hi, has_avg ? v.xs : v.X[cur], has_avg ? v.xl : nullptr, v.X[cur], v.xl, v.dc, v.atya,
                 inv_w, v.atyl, mine};
    group_rows_dyn<2, double>(v.G, v.cptr, v.cidx, v.cval, v.n,
                              Gather2{has_avg ? v.ys : v.Y[cur], has_avg ? v.yl : nullptr, v.Y[cur], inv_w, T.size > 1}, ec,
                              T.rank, T.size);
    slot_sums<kColPartials>(slots, sm + kRowPartials);   // then the column partials
    // team totals of the partials and of the deadline test (any block past it stops all)
    constexpr int NT = kRowPartials + kColPartials;
    double tt[NT + 2];
    if (threadIdx.x == 0) {
        for (int q = 0; q < NT; ++q) tt[q] = sm[q];
        tt[NT] = (deadline && global_ns() > deadline) ? 1.0 : 0.0;
        tt[NT + 1] = (H.eligible && c.iters >= kHandoffMin &&
                      *reinterpret_cast<const volatile uint32_t*>(H.idle) >= H.need) ? 1.0 : 0.0;
    }
    if (!team_total<NT + 2>(tt, T)) return false;
    if (threadIdx.x == 0) {
        double tr[kRowPartials], tc[kColPartials];
        for (int q = 0; q < kRowPartials; ++q) tr[q] = tt[q];
        for (int q = 0; q < kColPartials; ++q) tc[q] = tt[kRowPartials + q];
        decide_check(c, tc, tr, I.inv_nb, I.inv_nc, tt[NT] > 0.0);
        s_handoff = !c.done && tt[NT + 1] > 0.0;
    }
    __syncthreads();
    const int ap = c.apply;
    if (ap == 0) {
        if (s_handoff) {
            if (threadIdx.x == 0) { c.done = 1; c.status = kStatusHandoff; }
            __syncthreads();
        }
        return true;
    }
    const bool load = ap & AP_LOAD_AVG, rst = ap & AP_RESTART, cand = (ap & AP_CANDIDATE) && !c.done;
    const bool save = (ap & AP_SAVE_BEST) && v.xb, save_avg = ap & AP_SAVE_AVG;
    const double iw = block_scalar<double>([&] { return c.w_sum > 0.0 ? 1.0 / c.w_sum : 0.0; });
    const float tau = block_scalar<float>([&] { return c.eta / c.omega; });
    float dx2 = 0.f;
    TEAM_OWNED(j, v.n, chc) {
        if (save) v.xb[j] = save_avg ? float(double(v.xl[j]) + double(v.xs[j]) * iw) : v.X[cur][j];
        float xv;
        if (load) {
            xv = float(double(v.xl[j]) + double(v.xs[j]) * iw);
            v.X[cur][j] = xv;
            v.ATY[cur][j] = v.atya[j];
        } else {
            xv = v.X[cur][j];
        }
        if (rst) {
            v.xl[j] = xv;
            v.xs[j] = 0.f;
            v.atyl[j] = v.ATY[cur][j];
        }
        if (cand) {
            const float x2 = fminf(fmaxf(xv - tau * (v.c[j] - v.ATY[cur][j]), v.lo[j]), v.hi[j]);
            v.X[1 - cur][j] = x2;
            dx2 += (x2 - xv) * (x2 - xv);
        }
    }
    TEAM_OWNED(i, v.m, chr) {
        if (save) v.yb[i] = save_avg ? float(double(v.yl[i]) + double(v.ys[i]) * iw) : v.Y[cur][i];
        float yv;
        if (load) {
            yv = float(double(v.yl[i]) + double(v.ys[i]) * iw);
            v.Y[cur][i] = yv;
            v.AX[cur][i] = v.axa[i];
        } else {
            yv = v.Y[cur][i];
        }
        if (rst) {
            v.yl[i] = yv;
            v.ys[i] = 0.f;
            v.axl[i] = v.AX[cur][i];
        }
    }
    float f[1] = {dx2};
    block_sum<1>(f, reinterpret_cast<float*>(sm));
    double t[1] = {double(f[0])};
    if (!team_total<1>(t, T)) return false;
    if (threadIdx.x == 0) {
        if (cand) c.dx2 = t[0];
        if (rst) c.w_sum = 0.0;
        c.apply = 0;
        // after the restart / averaging above: the handed-off point is the one
        // the instance would have continued from
        if (s_handoff) { c.done = 1; c.status = kStatusHandoff; }
    }
    __syncthreads();
    return true;
}

// Start point of instance k (cold: x = clip(0, lo, hi), y = 0; warm: the caller's
// point scaled and projected, with its primal weight), its products K x0 and
// K^T y0, and the init-phase check that records its relative KKT error.
__device__ bool start_point(const Args& A, int k, const Inst& I, const View& v, bool warm, Ctl& c, double* sm,
                            double* slots, const Team& T) {
    const int chc = kWarps * (32 / v.G), chr = kWarps * (32 / v.Gr);
    if (!team_barrier(T)) return false;
    if (threadIdx.x == 0) {
        c = Ctl{};
        c.status = SPS_STATUS_ITERATION_LIMIT;
        c.init_phase = 1;
        c.max_iters = A.max_iters;
        c.tol = A.tol;
        c.eta = A.a.eta0[k];
        c.omega = warm && A.wom[k] > 0.0 ? A.wom[k] : A.a.omega0[k];
        c.kkt_last = INFINITY;
        c.stall_on = A.stall_on;
        c.stall_ceiling = INFINITY;   // a stalled instance leaves the launch for the FP64 continuation
    }
    TEAM_OWNED(j, v.n, chc) {
        const float x0 = warm ? float(A.wx[I.vc + j] / v.dc[j]) : 0.f;
        const float x = fminf(fmaxf(x0, v.lo[j]), v.hi[j]);
        v.X[0][j] = x;
        v.xl[j] = x;
        v.xs[j] = 0.f;
    }
    TEAM_OWNED(i, v.m, chr) {
        float y = warm ? float(A.wy[I.vr + i] / v.dr[i]) : 0.f;
        if (v.kind[i]) y = fminf(y, 0.f);
        v.Y[0][i] = y;
        v.yl[i] = y;
        v.ys[i] = 0.f;
    }
    if (!team_barrier(T)) return false;
    StoreE sx{v.AX[0]};
    group_rows_r<1, float>(v.Gr, v.rptr, v.ridx, v.rval, v.m, Gather1{v.X[0], T.size > 1}, sx, T.rank, T.size);
    StoreE sy{v.ATY[0]};
    group_rows_dyn<1, float>(v.G, v.cptr, v.cidx, v.cval, v.n, Gather1{v.Y[0], T.size > 1}, sy, T.rank, T.size);
    if (!team_barrier(T)) return false;
    return check_and_apply(v, I, c, sm, slots, A.deadline, T, Handoff{A.idle, A.idle_need, false});
}

// The whole solve of instance k by this block (T.size == 1) or by the team of
// blocks of a cluster.  Returns false when a team barrier timed out.
__device__ bool solve_one(const Args& A, int k, int G, Ctl& c, double* sm, double* slots, const Team& T) {
    const Inst I = A.inst[k];
    const View v = make_view(A, I, G);
    const int chc = kWarps * (32 / v.G), chr = kWarps * (32 / v.Gr);
    const uint64_t t_begin = global_ns();
    const bool warm = A.warm != 0;
    bool used = warm;
    if (warm && A.fallback) {
        // keep the warm point only if its relative KKT error is not above the cold start's
        double cold = A.cold_rel[k];
        if (!(cold >= 0.0)) {
            if (!start_point(A, k, I, v, false, c, sm, slots, T)) return false;
            cold = c.rel_kkt;
            if (threadIdx.x == 0 && T.rank == 0) A.cold_rel[k] = cold;
        }
        if (!start_point(A, k, I, v, true, c, sm, slots, T)) return false;
        if (!(c.rel_kkt <= cold)) {
            used = false;
            if (!start_point(A, k, I, v, false, c, sm, slots, T)) return false;
        }
    } else {
        if (!start_point(A, k, I, v, warm, c, sm, slots, T)) return false;
    }
    // Step sizes of the next attempt, computed once by thread 0 (FP64 products
    // and divisions per thread would occupy this GPU's FP64 pipe, 1/64 of the
    // FP32 rate); the attempt's reductions are FP32 within the block.
    __shared__ float s_sigma, s_tau, s_wgt;
    float* smf = reinterpret_cast<float*>(sm);
    const Handoff H{A.idle, A.idle_need, A.handoff_nnz > 0 && I.nnz >= A.handoff_nnz};
    // the staging buffer shares its memory with the check's partial slots
    float* stage = reinterpret_cast<float*>(slots);
    const bool stage_x = v.n <= A.stage_cap, stage_y = v.m <= A.stage_cap;
    if (threadIdx.x == 0) {
        c.t_begin = t_begin;
        c.warm_used = used ? 1 : 0;
        s_sigma = float(c.eta * c.omega);
    }
    __syncthreads();
    for (;;) {
        for (int w = 0; w < A.check_interval; ++w) {
            if (c.done || c.iters >= c.max_iters) break;
            int cur = c.cur;
            RowStepE er{v.b, v.AX[cur], v.Y[cur], v.kind, v.AX[1 - cur], v.Y[1 - cur], s_sigma};
            if (stage_x) {
                stage_vector(stage, v.X[1 - cur], v.n, T.size > 1);
                group_rows_r<1, float>(v.Gr, v.rptr, v.ridx, v.rval, v.m, GatherS{stage}, er, T.rank, T.size);
            } else {
                group_rows_r<1, float>(v.Gr, v.rptr, v.ridx, v.rval, v.m, Gather1{v.X[1 - cur], T.size > 1}, er,
                                       T.rank, T.size);
            }
            float f2[2] = {er.dy2, er.inter};
            block_sum<2>(f2, smf);
            double t2[2] = {double(f2[0]), double(f2[1])};
            if (!team_total<2>(t2, T)) return false;
            if (threadIdx.x == 0) {
                decide_step(c, t2[0], t2[1]);
                s_tau = float(c.eta / c.omega);
                s_wgt = float(c.eta_used);
            }
            __syncthreads();
            if (c.done) break;
            cur = c.cur;
            const float tau = s_tau, wgt = s_wgt;
            float dx2;
            if (c.accepted) {
                ColStepE ec{v.X[cur], v.c, v.lo, v.hi, v.xl, v.ATY[cur], v.X[1 - cur], v.xs, tau, wgt};
                if (stage_y) {
                    stage_vector(stage, v.Y[cur], v.m, T.size > 1);
                    group_rows_dyn<1, float>(v.G, v.cptr, v.cidx, v.cval, v.n, GatherS{stage}, ec, T.rank, T.size);
                } else {
                    group_rows_dyn<1, float>(v.G, v.cptr, v.cidx, v.cval, v.n, Gather1{v.Y[cur], T.size > 1}, ec,
                                             T.rank, T.size);
                }
                dx2 = ec.dx2;
                TEAM_OWNED(i, v.m, chr) v.ys[i] += wgt * (v.Y[cur][i] - v.yl[i]);
            } else {
                dx2 = 0.f;
                TEAM_OWNED(j, v.n, chc) {
                    const float xj = v.X[cur][j];
                    const float x2 = fminf(fmaxf(xj - tau * (v.c[j] - v.ATY[cur][j]), v.lo[j]), v.hi[j]);
                    v.X[1 - cur][j] = x2;
                    dx2 += (x2 - xj) * (x2 - xj);
                }
            }
            float f1[1] = {dx2};
            block_sum<1>(f1, smf);
            double t1[1] = {double(f1[0])};
            if (!team_total<1>(t1, T)) return false;
            if (threadIdx.x == 0) {
                c.dx2 = t1[0];
                c.apply = 0;
                s_sigma = float(c.eta * c.omega);
            }
            __syncthreads();
        }
        if (c.done) break;
        if (!check_and_apply(v, I, c, sm, slots, A.deadline, T, H)) return false;
        if (c.done) break;
        if (threadIdx.x == 0) s_sigma = float(c.eta * c.omega);
        __syncthreads();
    }
    if (threadIdx.x == 0 && T.rank == 0) {
        c.t_end = global_ns();
        A.out[k] = c;
    }
    return true;
}

// Persistent solver.  Instances are handed out largest first from an atomic
// counter.  With A.team > 1 the launch is made of clusters of A.team blocks:
// while the next instance has at least A.team_nnz nonzeros the cluster's rank
// 0 takes it for the whole cluster (every block reads the index from rank 0's
// shared memory between two team barriers) and the team solves it; from the
// first smaller instance on, every block takes its own instances.
__global__ void __launch_bounds__(kBlock, 4) k_batch_solve(Args A, int G) {
    __shared__ Ctl c;
    __shared__ double sm[kWarps * 10];
    // dynamic: the check partial slots (kColPartials * kBlock doubles), reused as the
    // steps' staging buffer of A.stage_cap floats
    extern __shared__ double slots[];
    __shared__ double xch[2 * kXch];
    __shared__ uint32_t counter;
    __shared__ int s_inst, s_err;
    uint32_t gen = 0;
    int phase = 0;
    const int C = A.team > 1 ? A.team : 1;
    int rank = 0;
    if (threadIdx.x == 0) { counter = 0u; s_err = 0; }
    if (C > 1) {
        uint32_t r;
        asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
        rank = (int)r;
        // every block of the cluster initialises its counter before any block arrives at a team barrier
        asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
    }
    __syncthreads();
    const Team team{C, rank, &counter, &gen, xch, &phase, &s_err};
    const Team solo{1, 0, &counter, &gen, xch, &phase, &s_err};
    bool together = C > 1;
    for (;;) {
        int k;
        if (together) {
            if (threadIdx.x == 0 && rank == 0) {
                const uint32_t q = atomicAdd(A.counter, 1u);
                s_inst = q < (uint32_t)A.count ? A.order[q] : -1;
            }
            if (!team_barrier(team)) break;
            if (threadIdx.x == 0) {
                int r0;
                asm volatile("ld.shared::cluster.s32 %0, [%1];" : "=r"(r0) : "r"(cluster_addr(&s_inst, 0)) : "memory");
                sm[0] = double(r0);
            }
            __syncthreads();
            k = int(sm[0]);
            if (!team_barrier(team)) break;       // rank 0 may overwrite s_inst only after every block read it
            if (k < 0) break;
            if (A.inst[k].nnz >= A.team_nnz) {
                if (!solve_one(A, k, G, c, sm, slots, team)) break;
                continue;
            }
            together = false;                      // smaller instances: one block each from now on
            if (rank != 0) continue;
        } else {
            if (threadIdx.x == 0) {
                const uint32_t q = atomicAdd(A.counter, 1u);
                s_inst = q < (uint32_t)A.count ? A.order[q] : -1;
            }
            __syncthreads();
            k = s_inst;
            if (k < 0) break;
        }
        solve_one(A, k, G, c, sm, slots, solo);
        __syncthreads();
    }
    // this block found the queue empty (or its team gave up): it counts towards
    // the hand-off threshold of the instances still running
    if (threadIdx.x == 0 && A.idle) atomicAdd(A.idle, 1u);
    if (threadIdx.x == 0 && s_err) atomicExch(A.team_error, 1);
    // every block reaches this point once (all loops above are bounded): no block
    // leaves while a peer may still read its shared memory (the barrier counter,
    // the exchange buffers, the instance index)
    if (C > 1) asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}

// ---------------------------------------------------------------------------
// Per-instance scaling, one block per instance.
struct SetupArgs {
    const Inst* inst;
    const int32_t *rptr, *ridx, *cptr, *cidx;
    const double *rv64, *cv64;            // original values
    const double *c64, *lo64, *hi64, *b64;
    double *dr, *dc;
    float *rmax, *cmax;                   // scratch (per row / per column)
    float *rval, *cval, *c, *lo, *hi, *b;
    double *eta0, *omega0;
    int32_t ruiz;
};

// per row (warp each): stat = d_own[r] * max|v d_other| (or the sum)
// short: every row holds at most two entries, and a thread per row computes
// what the warp form does (its butterfly sum of two terms is t0 + t1 too: the
// other lanes add exact zeros), without 30 idle lanes per row
__device__ void row_stat(const int32_t* ptr, const int32_t* idx, const double* v, const double* d_own,
                         const double* d_other, int rows, bool sum, float* out, bool short_rows) {
    if (short_rows) {
        for (int r = threadIdx.x; r < rows; r += kBlock) {
            double a = 0.0;
            for (int k = ptr[r]; k < ptr[r + 1]; ++k) {
                const double t = fabs(v[k] * d_other[idx[k]]);
                a = sum ? a + t : fmax(a, t);
            }
            out[r] = float(a * d_own[r]);
        }
        return;
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int r = warp; r < rows; r += kWarps) {
        double a = 0.0;
        for (int k = ptr[r] + lane; k < ptr[r + 1]; k += 32) {
            const double t = fabs(v[k] * d_other[idx[k]]);
            a = sum ? a + t : fmax(a, t);
        }
        for (int o = 16; o > 0; o >>= 1) {
            const double u = __shfl_xor_sync(0xffffffffu, a, o);
            a = sum ? a + u : fmax(a, u);
        }
        if (lane == 0) out[r] = float(a * d_own[r]);
    }
}

__global__ void __launch_bounds__(kBlock) k_batch_setup(SetupArgs S) {
    const int k = blockIdx.x;
    const Inst I = S.inst[k];
    const int32_t *rptr = S.rptr + I.rp, *ridx = S.ridx + I.re, *cptr = S.cptr + I.cp, *cidx = S.cidx + I.ce;
    const double *rv = S.rv64 + I.re, *cv = S.cv64 + I.ce;
    double *dr = S.dr + I.vr, *dc = S.dc + I.vc;
    float *rm = S.rmax + I.vr, *cm = S.cmax + I.vc;
    __shared__ int longest[2];                  // longest row, longest column
    if (threadIdx.x < 2) longest[threadIdx.x] = 0;
    __syncthreads();
    {
        int lr = 0, lc = 0;
        for (int j = threadIdx.x; j < I.n; j += kBlock) {
            dc[j] = 1.0;
            lc = max(lc, cptr[j + 1] - cptr[j]);
        }
        for (int i = threadIdx.x; i < I.m; i += kBlock) {
            dr[i] = 1.0;
            lr = max(lr, rptr[i + 1] - rptr[i]);
        }
        atomicMax(&longest[0], lr);
        atomicMax(&longest[1], lc);
    }
    __syncthreads();
    const bool short_rows = longest[0] <= 2, short_cols = longest[1] <= 2;
    for (int it = 0; it <= S.ruiz; ++it) {
        const bool pc = it == S.ruiz;           // last pass: Pock-Chambolle (sums), before it Ruiz (max)
        row_stat(rptr, ridx, rv, dr, dc, I.m, pc, rm, short_rows);
        row_stat(cptr, cidx, cv, dc, dr, I.n, pc, cm, short_cols);
        __syncthreads();
        for (int i = threadIdx.x; i < I.m; i += kBlock)
            if (rm[i] > 0.f) dr[i] /= sqrt(double(rm[i]));
        for (int j = threadIdx.x; j < I.n; j += kBlock)
            if (cm[j] > 0.f) dc[j] /= sqrt(double(cm[j]));
        __syncthreads();
    }
    double mx = 0.0, sc = 0.0, sb = 0.0;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // (a thread per row or column where they are short: the same values, the same maximum)
    const int rstep = short_rows ? kBlock : kWarps, rlane = short_rows ? 1 : 32;
    for (int r = short_rows ? threadIdx.x : warp; r < I.m; r += rstep)
        for (int q = rptr[r] + (short_rows ? 0 : lane); q < rptr[r + 1]; q += rlane) {
            const float v = float(rv[q] * dr[r] * dc[ridx[q]]);
            S.rval[I.re + q] = v;
            mx = fmax(mx, fabs(double(v)));
        }
    const int cstep = short_cols ? kBlock : kWarps, clane = short_cols ? 1 : 32;
    for (int j = short_cols ? threadIdx.x : warp; j < I.n; j += cstep)
        for (int q = cptr[j] + (short_cols ? 0 : lane); q < cptr[j + 1]; q += clane)
            S.cval[I.ce + q] = float(cv[q] * dc[j] * dr[cidx[q]]);
    for (int j = threadIdx.x; j < I.n; j += kBlock) {
        const double cs = S.c64[I.vc + j] * dc[j];
        S.c[I.vc + j] = float(cs);
        S.lo[I.vc + j] = float(S.lo64[I.vc + j] / dc[j]);
        S.hi[I.vc + j] = float(S.hi64[I.vc + j] / dc[j]);
        sc += cs * cs;
    }
    for (int i = threadIdx.x; i < I.m; i += kBlock) {
        const double bs = S.b64[I.vr + i] * dr[i];
        S.b[I.vr + i] = float(bs);
        sb += bs * bs;
    }
    __shared__ double sm[kWarps * 3];
    __shared__ double smx[kWarps];
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) smx[warp] = mx;
    double s2[2] = {sc, sb};
    block_sum<2>(s2, sm);
    if (threadIdx.x == 0) {
        for (int w = 1; w < kWarps; ++w) mx = fmax(mx, smx[w]);
        mx = fmax(mx, smx[0]);
        S.eta0[k] = mx > 0.0 ? 1.0 / mx : 1.0;
        S.omega0[k] = (s2[0] > 1e-20 && s2[1] > 1e-20) ? sqrt(s2[0]) / sqrt(s2[1]) : 1.0;
    }
}

// Inputs of the warm-start network for instances s0 .. s0+cnt-1 from the batch's
// scaled data: c = c~ / dc, b = b~ / dr (the original costs and right-hand sides).
__global__ void __launch_bounds__(kBlock) k_gnn_inputs(const Inst* inst, int s0, int cnt, Arrays a, int n, int m,
                                                       double inv_cs, double inv_bs, float* c_in, float* b_in) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)cnt * n; t += stride) {
        const Inst& I = inst[s0 + t / n];
        const int64_t q = I.vc + t % n;
        c_in[t] = float(double(a.c[q]) / a.dc[q] * inv_cs);
    }
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)cnt * m; t += stride) {
        const Inst& I = inst[s0 + t / m];
        const int64_t q = I.vr + t % m;
        b_in[t] = float(double(a.b[q]) / a.dr[q] * inv_bs);
    }
}

// Network outputs of instances s0 .. s0+cnt-1 into the warm-start buffers (the
// start-up kernel projects them on the bounds and signs).
__global__ void __launch_bounds__(kBlock) k_gnn_outputs(const Inst* inst, int s0, int cnt, int n, int m,
                                                        const float* x0, const float* y0, const float* lw, double xs,
                                                        double ys, double* wx, double* wy, double* wom) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)cnt * n; t += stride)
        wx[inst[s0 + t / n].vc + t % n] = double(x0[t]) * xs;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)cnt * m; t += stride)
        wy[inst[s0 + t / m].vr + t % m] = double(y0[t]) * ys;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < cnt; t += stride)
        wom[s0 + t] = exp(fmin(fmax(double(lw[t]), -30.0), 30.0));
}

// Absolute device deadline of a batched solve (0 = none), set at the start of
// the solve so a replayed graph measures the limit from its own launch.
__global__ void k_set_deadline(uint64_t* dl, uint64_t limit_ns) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *dl = limit_ns ? global_ns() + limit_ns : 0;
}

// Unscaled solution of every instance (one block per instance), FP64.
__global__ void __launch_bounds__(kBlock) k_batch_extract(const Inst* inst, const Ctl* out, Arrays a, double* xo,
                                                          double* yo) {
    const int k = blockIdx.x;
    const Inst I = inst[k];
    const int cur = out[k].cur;
    // a stalled instance hands its best point to the FP64 continuation
    const bool best = out[k].status == SPS_STATUS_STALLED && out[k].best_saved && a.xb;
    const float* X = best ? a.xb + I.vc : (cur ? a.x1 : a.x0) + I.vc;
    const float* Y = best ? a.yb + I.vr : (cur ? a.y1 : a.y0) + I.vr;
    for (int j = threadIdx.x; j < I.n; j += kBlock) xo[I.vc + j] = double(X[j]) * a.dc[I.vc + j];
    for (int i = threadIdx.x; i < I.m; i += kBlock) yo[I.vr + i] = double(Y[i]) * a.dr[I.vr + i];
}

}  // namespace batch
}  // namespace sps

// ===========================================================================
// Host side
// ===========================================================================
using sps::Ctl;
using sps::batch::Inst;

// A host array that is not value-initialised on allocation (the batch packing
// writes every element on its own threads).
template <class T>
struct HostBuf {
    std::unique_ptr<T[]> p;
    size_t n = 0;
    HostBuf() = default;
    explicit HostBuf(int64_t count) : p(new T[(size_t)std::max<int64_t>(count, 1)]), n((size_t)std::max<int64_t>(count, 0)) {}
    T* data() { return p.get(); }
    const T* data() const { return p.get(); }
    T& operator[](size_t i) { return p[i]; }
    const T& operator[](size_t i) const { return p[i]; }
    size_t size() const { return n; }
    bool empty() const { return n == 0; }
};

struct sps_batch {
    int32_t count = 0;
    sps_options opt{};
    int32_t G = 8, Gr = 32, blocks = 0;      // lanes per column / per row, persistent blocks
    int32_t stage_cap = 0;                    // floats of the kernel's shared staging buffer
    size_t dyn_smem = 0;                      // dynamic shared memory of the solve launch
    int32_t team = 1;                         // cluster size of the solve launch
    int32_t team_nnz = 65536;                 // instances at least this large are solved by a team
    int32_t* d_team_error = nullptr;
    uint32_t* d_idle = nullptr;               // blocks that found the queue empty (per launch)
    int32_t handoff_nnz = 0;                  // instances this large may leave the tail (0 = never)
    std::vector<int8_t> handed_off;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    std::vector<Inst> inst;
    std::vector<int32_t> order;
    std::vector<void*> dev;                 // device allocations
    Inst* d_inst = nullptr;
    int32_t* d_order = nullptr;
    Ctl* d_out = nullptr;
    uint32_t* d_counter = nullptr;
    double *d_xo = nullptr, *d_yo = nullptr;
    sps::batch::Arrays arr{};
    int64_t sum_n = 0, sum_m = 0;
    HostBuf<double> c_all, lb_all, ub_all;       // original data, packed like the column vectors
    // original rows (local CSR offsets, columns, values) and right-hand sides,
    // kept for the FP64 continuation of stalled instances
    HostBuf<int32_t> h_rptr, h_ridx;
    HostBuf<double> h_rv, h_b;
    std::vector<double> xo, yo;
    std::vector<Ctl> out;
    std::vector<int8_t> escalated;
    std::vector<double> esc_ms;             // wall time of each instance's FP64 continuation
    cudaGraphExec_t gexec = nullptr;
    int32_t gexec_G = -1, gexec_warm = -1;
    uint64_t gexec_tl = 0;
    // warm starts (original space, packed like the vectors) and the cold-start error cache
    double *d_wx = nullptr, *d_wy = nullptr, *d_wom = nullptr, *d_cold_rel = nullptr;
    int32_t warm = 0;
    uint64_t* d_deadline = nullptr;
    double setup_ms = 0.0, solve_ms = 0.0;
    bool solved = false;
    std::string err;

    ~sps_batch() {
        if (gexec) cudaGraphExecDestroy(gexec);
        for (void* p : dev) cudaFree(p);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        if (st) cudaStreamDestroy(st);
    }
    template <class T>
    cudaError_t alloc(T** p, size_t count_) {
        void* q = nullptr;
        const cudaError_t e = cudaMalloc(&q, std::max<size_t>(count_, 1) * sizeof(T));
        if (e == cudaSuccess) dev.push_back(q);
        *p = static_cast<T*>(q);
        return e;
    }
    int fail(int code, const std::string& m) {
        err = m;
        return code;
    }
};

namespace {

#define SPB_CK(call)                                                                           \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return b->fail(e_ == cudaErrorMemoryAllocation ? SPS_ERR_OOM : SPS_ERR_CUDA,        \
                           std::string(#call) + ": " + cudaGetErrorString(e_));                \
    } while (0)

// Host validation of one instance; also sizes.
bool check_instance(const sps_problem_desc& d, std::string& why) {
    if (d.n < 0 || d.m_ub < 0 || d.m_eq < 0) { why = "negative dimension"; return false; }
    auto csr_ok = [&](const int32_t* p, const int32_t* ix, const double* v, int32_t rows) {
        if (rows == 0) return true;
        if (!p || p[0] != 0) return false;
        for (int32_t i = 0; i < rows; ++i)
            if (p[i + 1] < p[i]) return false;
        return p[rows] == 0 || (ix && v);
    };
    if (!csr_ok(d.ub_indptr, d.ub_indices, d.ub_values, d.m_ub) || !csr_ok(d.eq_indptr, d.eq_indices, d.eq_values, d.m_eq)) {
        why = "malformed CSR";
        return false;
    }
    if (d.n > 0 && (!d.c || !d.lb || !d.ub)) { why = "null c/lb/ub"; return false; }
    if ((d.m_ub && !d.b_ub) || (d.m_eq && !d.b_eq)) { why = "null rhs"; return false; }
    for (int32_t j = 0; j < d.n; ++j) {
        const double l = d.lb[j], u = d.ub[j];
        if (!std::isfinite(d.c[j]) || std::isnan(l) || std::isnan(u) || l == INFINITY || u == -INFINITY || l > u + 1e-12) {
            why = "invalid objective or bounds at variable " + std::to_string(j);
            return false;
        }
    }
    for (int32_t i = 0; i < d.m_ub; ++i)
        if (!std::isfinite(d.b_ub[i])) { why = "non-finite right-hand side"; return false; }
    for (int32_t i = 0; i < d.m_eq; ++i)
        if (!std::isfinite(d.b_eq[i])) { why = "non-finite right-hand side"; return false; }
    return true;
}

// Continuation of instance k on the single-LP engine after the persistent
// launch, within the iterations and time left; its result replaces the
// instance's.  A stalled instance continues in FP64 from the best point of the
// FP32 stall test (in xo / yo) with the primal weight it had there; an instance
// handed off from the launch's tail continues in FP32 (with its own stall test
// and FP64 continuation) from its current point and primal weight.
int continue_single(sps_batch* b, int32_t k, double used_s, std::string* why) {
    const Inst& I = b->inst[k];
    Ctl& c = b->out[k];
    const bool handoff = c.status == sps::batch::kStatusHandoff;
    const char* what = handoff ? " continuation after hand-off: " : " FP64 continuation: ";
    if (b->opt.time_limit_s > 0 && used_s >= b->opt.time_limit_s) {
        c.status = SPS_STATUS_TIME_LIMIT;
        return SPS_OK;
    }
    const int32_t* P = b->h_rptr.data() + I.rp;
    const int32_t m_eq = I.m - I.m_ub;
    std::vector<int32_t> eqp(m_eq + 1);
    for (int32_t i = 0; i <= m_eq; ++i) eqp[i] = P[I.m_ub + i] - P[I.m_ub];
    sps_problem_desc d{};
    d.n = I.n;
    d.m_ub = I.m_ub;
    d.m_eq = m_eq;
    d.ub_indptr = P;
    d.ub_indices = b->h_ridx.data() + I.re;
    d.ub_values = b->h_rv.data() + I.re;
    d.eq_indptr = eqp.data();
    d.eq_indices = b->h_ridx.data() + I.re + P[I.m_ub];
    d.eq_values = b->h_rv.data() + I.re + P[I.m_ub];
    d.c = b->c_all.data() + I.vc;
    d.lb = b->lb_all.data() + I.vc;
    d.ub = b->ub_all.data() + I.vc;
    d.b_ub = b->h_b.data() + I.vr;
    d.b_eq = b->h_b.data() + I.vr + I.m_ub;
    sps_options o = b->opt;
    o.precision = handoff ? SPS_FP32 : SPS_FP64;
    o.escalate = handoff ? b->opt.escalate : 0;
    o.max_iters = std::max<int64_t>(b->opt.max_iters - c.iters, 1);
    o.time_limit_s = b->opt.time_limit_s > 0 ? b->opt.time_limit_s - used_s : 0.0;
    sps_handle* h = nullptr;
    int rc = sps_create(&d, &o, &h);
    if (rc != SPS_OK) {
        *why = "instance " + std::to_string(k) + what + sps_last_error(nullptr);
        return rc;
    }
    sps_result r;
    double* x = b->xo.data() + I.vc;
    double* y = b->yo.data() + I.vr;
    rc = sps_set_warm_start(h, x, y, handoff ? c.omega : c.omega_best);
    if (rc == SPS_OK) rc = sps_solve(h, &r);
    if (rc == SPS_OK) rc = sps_get_solution(h, x, y);
    if (rc != SPS_OK) {
        *why = "instance " + std::to_string(k) + what + sps_last_error(h);
        sps_destroy(h);
        return rc;
    }
    sps_destroy(h);
    c.status = r.status;
    c.iters += r.iterations;
    c.accepted_total += r.accepted_steps;
    c.restarts += r.restarts;
    c.rel_kkt = r.rel_kkt; c.rel_p = r.rel_primal; c.rel_d = r.rel_dual; c.rel_gap = r.rel_gap;
    c.omega = r.primal_weight;
    c.eta = r.step_size;
    c.choice = r.returned_average;
    b->escalated[k] = handoff ? (int8_t)r.escalated : 1;
    b->handed_off[k] = handoff ? 1 : 0;
    return SPS_OK;
}

}  // namespace

// Autotuned schedules, kept for the process by a coarse shape of the batch, so
// a caller that creates many similar batches (the children of every node of a
// branch-and-bound search, a repeated workload) times the candidates once:
// device, cluster size, given lanes per column (0 = tuned), and half-octave
// buckets of the instance count, the mean nonzeros per column and per row, and
// the largest instance.
struct ScheduleKey {
    int32_t v[7];
    bool operator<(const ScheduleKey& o) const { return std::lexicographical_compare(v, v + 7, o.v, o.v + 7); }
};
static std::mutex g_schedule_mu;
static std::map<ScheduleKey, std::pair<int32_t, int32_t>> g_schedules;

static int32_t half_octave(double x) { return x > 0.0 ? (int32_t)std::floor(2.0 * std::log2(x)) : -1000; }

extern "C" int sps_batch_create(int32_t count, const sps_problem_desc* probs, const sps_options* opt_in,
                                sps_batch** out) {
    sps::NvtxRange nvtx_range("sps_batch_create");
    if (!out || count <= 0 || !probs) {
        sps::set_create_error("sps_batch_create: need count > 0, problems and an output pointer");
        return SPS_ERR_INVALID;
    }
    *out = nullptr;
    sps_options opt;
    if (opt_in) opt = *opt_in; else sps_options_init(&opt);
    if (opt.mode != SPS_MODE_ADAPTIVE || opt.precision != SPS_FP32) {
        sps::set_create_error("sps_batch_create: the batched solver runs the adaptive mode with FP32 iterates");
        return SPS_ERR_INVALID;
    }
    if (opt.kkt_form != SPS_KKT_LAGRANGIAN) {
        sps::set_create_error("sps_batch_create: the batched solver reports the Lagrangian KKT form only");
        return SPS_ERR_INVALID;
    }
    auto b = std::make_unique<sps_batch>();
    b->count = count;
    b->opt = opt;
    // ---- sizes and validation
    b->inst.resize(count);
    int64_t rp = 0, re = 0, cp = 0, vc = 0, vr = 0;
    for (int32_t k = 0; k < count; ++k) {
        std::string why;
        if (!check_instance(probs[k], why)) {
            sps::set_create_error("instance " + std::to_string(k) + ": " + why);
            return SPS_ERR_INVALID;
        }
        const sps_problem_desc& d = probs[k];
        Inst& I = b->inst[k];
        I.n = d.n;
        I.m = d.m_ub + d.m_eq;
        I.m_ub = d.m_ub;
        const int64_t nz = (int64_t)(d.m_ub ? d.ub_indptr[d.m_ub] : 0) + (d.m_eq ? d.eq_indptr[d.m_eq] : 0);
        I.nnz = (int32_t)std::min<int64_t>(nz, INT32_MAX);
        I.rp = rp; I.re = re; I.cp = cp; I.ce = re; I.vc = vc; I.vr = vr;
        rp += I.m + 1; cp += I.n + 1; re += nz; vc += I.n; vr += I.m;
    }
    if (re > INT32_MAX) {
        sps::set_create_error("sps_batch_create: a batch holds at most 2^31-1 nonzeros in total");
        return SPS_ERR_INVALID;
    }
    const int64_t NNZ = re;
    b->sum_n = vc;
    b->sum_m = vr;
    // ---- host packing (CSR of [A_ub; A_eq] and a CSC by counting sort), spread over host threads
    // not zero-filled: every element is written by the packing threads (gigabytes on
    // large batches, which a value-initialising std::vector cleared on one thread)
    HostBuf<int32_t> rptr(rp), ridx(NNZ), cptr(cp), cidx(NNZ);
    HostBuf<double> rv(NNZ), cv(NNZ), c64(vc), lo64(vc), hi64(vc), b64(vr);
    HostBuf<int8_t> kind(vr);
    std::vector<std::string> errs(count);
    auto pack = [&](int32_t k) {
        const sps_problem_desc& d = probs[k];
        Inst& I = b->inst[k];
        int32_t* P = rptr.data() + I.rp;
        int64_t q = 0;
        P[0] = 0;
        for (int part = 0; part < 2; ++part) {
            const int32_t rows = part ? d.m_eq : d.m_ub;
            const int32_t* ip = part ? d.eq_indptr : d.ub_indptr;
            const int32_t* ix = part ? d.eq_indices : d.ub_indices;
            const double* v = part ? d.eq_values : d.ub_values;
            for (int32_t i = 0; i < rows; ++i) {
                for (int32_t t = ip[i]; t < ip[i + 1]; ++t) {
                    const int32_t j = ix[t];
                    if (j < 0 || j >= d.n) { errs[k] = "column index out of range"; return; }
                    if (!std::isfinite(v[t])) { errs[k] = "non-finite matrix value"; return; }
                    ridx[I.re + q] = j;
                    rv[I.re + q] = v[t];
                    ++q;
                }
                const int32_t r = part ? d.m_ub + i : i;
                P[r + 1] = (int32_t)q;
                kind[I.vr + r] = part ? 0 : 1;
                b64[I.vr + r] = part ? d.b_eq[i] : d.b_ub[i];
            }
        }
        int32_t* C = cptr.data() + I.cp;
        std::fill(C, C + I.n + 1, 0);
        for (int64_t t = 0; t < q; ++t) C[ridx[I.re + t] + 1]++;
        for (int32_t j = 0; j < I.n; ++j) C[j + 1] += C[j];
        std::vector<int32_t> fill(C, C + I.n);
        for (int32_t r = 0; r < I.m; ++r)
            for (int32_t t = P[r]; t < P[r + 1]; ++t) {
                const int32_t j = ridx[I.re + t];
                const int32_t pos = fill[j]++;
                cidx[I.ce + pos] = r;
                cv[I.ce + pos] = rv[I.re + t];
            }
        for (int32_t j = 0; j < I.n; ++j) {
            c64[I.vc + j] = d.c[j];
            lo64[I.vc + j] = d.lb[j];
            hi64[I.vc + j] = d.ub[j];
        }
        double nb = 0, nc = 0;
        for (int32_t r = 0; r < I.m; ++r) nb += b64[I.vr + r] * b64[I.vr + r];
        for (int32_t j = 0; j < I.n; ++j) nc += d.c[j] * d.c[j];
        I.inv_nb = 1.0 / (1.0 + std::sqrt(nb));
        I.inv_nc = 1.0 / (1.0 + std::sqrt(nc));
    };
    {
        const int nt = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
        std::vector<std::thread> pool;
        std::atomic<int32_t> next{0};
        for (int t = 0; t < nt; ++t)
            pool.emplace_back([&]() {
                for (int32_t k; (k = next.fetch_add(1)) < count;) pack(k);
            });
        for (auto& th : pool) th.join();
    }
    for (int32_t k = 0; k < count; ++k)
        if (!errs[k].empty()) {
            sps::set_create_error("instance " + std::to_string(k) + ": " + errs[k]);
            return SPS_ERR_INVALID;
        }
    b->c_all = std::move(c64);
    b->lb_all = std::move(lo64);
    b->ub_all = std::move(hi64);
    // hand-out order: largest instances (nonzeros + rows + columns) first
    std::vector<int64_t> work(count);
    for (int32_t k = 0; k < count; ++k)
        work[k] = ((k + 1 < count ? b->inst[k + 1].re : NNZ) - b->inst[k].re) + b->inst[k].m + b->inst[k].n;
    b->order.resize(count);
    std::iota(b->order.begin(), b->order.end(), 0);
    std::stable_sort(b->order.begin(), b->order.end(), [&](int32_t a, int32_t c) { return work[a] > work[c]; });

    // ---- device
    sps_batch* bp = b.get();
    {
        sps_batch* b = bp;
        SPB_CK(cudaSetDevice(opt.device));
        SPB_CK(cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking));
        SPB_CK(cudaEventCreate(&b->e0));
        SPB_CK(cudaEventCreate(&b->e1));
        SPB_CK(cudaEventRecord(b->e0, b->st));
        sps::batch::Arrays& a = b->arr;
        int32_t *d_rptr, *d_ridx, *d_cptr, *d_cidx;
        float *d_rval, *d_cval, *d_c, *d_lo, *d_hi, *d_b;
        int8_t* d_kind;
        double *d_dr, *d_dc, *d_eta0, *d_om0;
        SPB_CK(b->alloc(&d_rptr, rp)); SPB_CK(b->alloc(&d_ridx, NNZ));
        SPB_CK(b->alloc(&d_cptr, cp)); SPB_CK(b->alloc(&d_cidx, NNZ));
        SPB_CK(b->alloc(&d_rval, NNZ)); SPB_CK(b->alloc(&d_cval, NNZ));
        SPB_CK(b->alloc(&d_c, vc)); SPB_CK(b->alloc(&d_lo, vc)); SPB_CK(b->alloc(&d_hi, vc));
        SPB_CK(b->alloc(&d_b, vr)); SPB_CK(b->alloc(&d_kind, vr));
        SPB_CK(b->alloc(&d_dr, vr)); SPB_CK(b->alloc(&d_dc, vc));
        SPB_CK(b->alloc(&d_eta0, count)); SPB_CK(b->alloc(&d_om0, count));
        float* st_f[14];
        for (int q = 0; q < 7; ++q) SPB_CK(b->alloc(&st_f[q], vc));
        for (int q = 7; q < 14; ++q) SPB_CK(b->alloc(&st_f[q], vr));
        SPB_CK(b->alloc(&b->d_inst, count));
        SPB_CK(b->alloc(&b->d_order, count));
        SPB_CK(b->alloc(&b->d_out, count));
        SPB_CK(b->alloc(&b->d_counter, 1));
        SPB_CK(b->alloc(&b->d_deadline, 1));
        SPB_CK(cudaMemsetAsync(b->d_deadline, 0, sizeof(uint64_t), b->st));
        SPB_CK(b->alloc(&b->d_xo, vc));
        SPB_CK(b->alloc(&b->d_yo, vr));
        SPB_CK(b->alloc(&b->d_cold_rel, count));
        SPB_CK(b->alloc(&b->d_team_error, 1));
        SPB_CK(b->alloc(&b->d_idle, 1));
        SPB_CK(cudaMemsetAsync(b->d_cold_rel, 0xFF, sizeof(double) * count, b->st));   // NaN = unknown
        float *d_xb = nullptr, *d_yb = nullptr, *d_axl, *d_atyl;
        if (opt.escalate != 0) { SPB_CK(b->alloc(&d_xb, vc)); SPB_CK(b->alloc(&d_yb, vr)); }
        SPB_CK(b->alloc(&d_axl, vr)); SPB_CK(b->alloc(&d_atyl, vc));
        double *t_rv, *t_cv, *t_c, *t_lo, *t_hi, *t_b;
        SPB_CK(cudaMalloc(&t_rv, sizeof(double) * std::max<int64_t>(NNZ, 1)));
        SPB_CK(cudaMalloc(&t_cv, sizeof(double) * std::max<int64_t>(NNZ, 1)));
        SPB_CK(cudaMalloc(&t_c, sizeof(double) * (3 * (size_t)vc + vr + 1)));
        t_lo = t_c + vc; t_hi = t_lo + vc; t_b = t_hi + vc;
        auto up = [&](void* dst, const void* src, size_t bytes) {
            return bytes ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, b->st) : cudaSuccess;
        };
        SPB_CK(up(d_rptr, rptr.data(), 4 * rp)); SPB_CK(up(d_ridx, ridx.data(), 4 * NNZ));
        SPB_CK(up(d_cptr, cptr.data(), 4 * cp)); SPB_CK(up(d_cidx, cidx.data(), 4 * NNZ));
        SPB_CK(up(t_rv, rv.data(), 8 * NNZ)); SPB_CK(up(t_cv, cv.data(), 8 * NNZ));
        SPB_CK(up(t_c, b->c_all.data(), 8 * vc)); SPB_CK(up(t_lo, b->lb_all.data(), 8 * vc));
        SPB_CK(up(t_hi, b->ub_all.data(), 8 * vc)); SPB_CK(up(t_b, b64.data(), 8 * vr));
        SPB_CK(up(d_kind, kind.data(), vr));
        SPB_CK(up(b->d_inst, b->inst.data(), sizeof(Inst) * count));
        SPB_CK(up(b->d_order, b->order.data(), 4 * (size_t)count));
        sps::batch::SetupArgs S{b->d_inst, d_rptr, d_ridx, d_cptr, d_cidx, t_rv, t_cv, t_c, t_lo, t_hi, t_b,
                                d_dr, d_dc, /*row stats*/ st_f[7], /*column stats*/ st_f[0], d_rval, d_cval, d_c,
                                d_lo, d_hi, d_b, d_eta0, d_om0,
                                opt.ruiz_iters >= 0 ? opt.ruiz_iters : 10};
        sps::batch::k_batch_setup<<<count, sps::kBlock, 0, b->st>>>(S);
        SPB_CK(cudaGetLastError());
        SPB_CK(cudaStreamSynchronize(b->st));
        cudaFree(t_rv); cudaFree(t_cv); cudaFree(t_c);
        a = sps::batch::Arrays{d_rptr, d_ridx, d_cptr, d_cidx, d_rval, d_cval, d_kind, d_c, d_lo, d_hi, d_b,
                               d_dc, d_dr, d_eta0, d_om0,
                               st_f[0], st_f[1], st_f[2], st_f[3], st_f[4], st_f[5], st_f[6],
                               st_f[7], st_f[8], st_f[9], st_f[10], st_f[11], st_f[12], st_f[13], d_xb, d_yb,
                               d_axl, d_atyl};
        b->handoff_nnz = std::max(opt.batch_handoff_nnz, 0);
        if (opt.escalate == 1 || b->handoff_nnz > 0) {       // host copy for continuations
            b->h_rptr = std::move(rptr);
            b->h_ridx = std::move(ridx);
            b->h_rv = std::move(rv);
            b->h_b = std::move(b64);
        }
        int nb = 0, dev = opt.device, sms = 152;
        // Shared staging buffer of the steps' gathers: the memory of the check's
        // partial slots (7168 floats), which the steps do not use.  A larger
        // buffer would stage longer vectors but, at 4 blocks per SM, leave the SM
        // too little L1 for everything else (measured: slower on the
        // 80k-column transportation family).
        b->dyn_smem = sizeof(double) * sps::kColPartials * sps::kBlock;
        b->stage_cap = (int32_t)(b->dyn_smem / sizeof(float));
        SPB_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, sps::batch::k_batch_solve, sps::kBlock,
                                                             b->dyn_smem));
        SPB_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        const int64_t slots = (int64_t)std::max(nb, 1) * sms;      // resident blocks of one wave
        b->blocks = (int)std::max<int64_t>(1, std::min<int64_t>(count, slots));
        // Large instances are solved by a team of blocks (one thread-block cluster).
        // Large = at least batch_team_nnz nonzeros; by default at least 65536 and,
        // in a batch that fills the GPU, twice the median instance: teams shorten
        // the tail of uneven batches, and in batches of similar sizes they would
        // only halve the instances in flight.  A batch of fewer than half as many
        // instances as resident blocks (strong branching's children) leaves SMs
        // idle instead: there every instance of 65536 nonzeros or more gets a
        // team, 2, 4 or 8 blocks, the largest that still fits the resident wave.
        // Default team in a batch that fills the GPU: 4 blocks (4096 planted LPs of
        // 50-5000 rows: 2.90 s per batch against 3.19 s with 2 and 3.26 s with 8).
        int want = opt.batch_team > 0 ? std::min(opt.batch_team, 8) : 4;
        if (opt.batch_team_nnz > 0) {
            b->team_nnz = opt.batch_team_nnz;
        } else if ((int64_t)count * 2 <= slots) {
            b->team_nnz = sps::batch::kTeamNnz;
            if (opt.batch_team <= 0) {
                want = 2;
                while (want < 8 && (int64_t)count * want * 2 <= slots) want *= 2;
            }
        } else {
            const int32_t med = b->inst[b->order[count / 2]].nnz;
            b->team_nnz = (int32_t)std::max<int64_t>(sps::batch::kTeamNnz, 2LL * med);
        }
        int64_t n_large = 0;
        for (int32_t k = 0; k < count; ++k) n_large += b->inst[k].nnz >= b->team_nnz;
        // clusters for the large instances: used when such a launch can be scheduled
        const int64_t need = std::min<int64_t>(slots, (count - n_large) + n_large * want);
        if (want > 1 && n_large > 0 && need >= want) {
            cudaLaunchConfig_t cfg = {};
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeClusterDimension;
            attr[0].val.clusterDim.x = want;
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.gridDim = dim3((unsigned)((need / want) * want));
            cfg.blockDim = dim3(sps::kBlock);
            cfg.dynamicSmemBytes = b->dyn_smem;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            int ncl = 0;
            if (cudaOccupancyMaxActiveClusters(&ncl, sps::batch::k_batch_solve, &cfg) == cudaSuccess && ncl > 0) {
                b->team = want;
                b->blocks = (int)((need / want) * want);
            }
            cudaGetLastError();
        }
        SPB_CK(cudaEventRecord(b->e1, b->st));
        SPB_CK(cudaStreamSynchronize(b->st));
        float ms = 0;
        cudaEventElapsedTime(&ms, b->e0, b->e1);
        b->setup_ms = ms;
    }
    // ---- lanes per column: given, or timed on a sample of the batch
    // schedule: lanes per column given (batch_group) or timed; lanes per row timed
    // second with the chosen column schedule (32 attempts and one check per
    // candidate on a sample of the largest instances)
    ScheduleKey key{};
    {
        int64_t nz = 0, nn = 0, mm = 0, big = 0;
        for (const Inst& I : b->inst) { nz += I.nnz; nn += I.n; mm += I.m; big = std::max<int64_t>(big, I.nnz); }
        key = ScheduleKey{{opt.device, b->team, opt.batch_group, half_octave(double(count)),
                           half_octave(nn ? double(nz) / double(nn) : 0.0), half_octave(mm ? double(nz) / double(mm) : 0.0),
                           half_octave(double(big))}};
        std::lock_guard<std::mutex> lk(g_schedule_mu);
        auto it = g_schedules.find(key);
        if (it != g_schedules.end()) {
            b->G = it->second.first;
            b->Gr = it->second.second;
            *out = b.release();
            return SPS_OK;
        }
    }
    {
        sps_batch* bb = bp;
        // A sample spread over the whole size range (every stride-th instance of the
        // largest-first order); a candidate's cost is the SUM of its instances' device
        // times for 32 attempts and one check each (throughput, not the sample's
        // makespan, which only reflects its largest instance).
        const int32_t sample = std::min<int32_t>(count, 2 * bb->blocks);
        std::vector<int32_t> pick(sample);
        for (int32_t q = 0; q < sample; ++q) pick[q] = bb->order[(int64_t)q * count / sample];
        int32_t* d_pick = nullptr;
        SPB_CK(bb->alloc(&d_pick, sample));
        SPB_CK(cudaMemcpyAsync(d_pick, pick.data(), sizeof(int32_t) * sample, cudaMemcpyHostToDevice, bb->st));
        std::vector<Ctl> outs(count);
        auto time_one = [&](int sched, float* cost) -> bool {
            sps::batch::Args A{bb->d_inst, d_pick, sample, 32, 32, 0.0, bb->d_deadline, bb->arr, bb->d_out,
                               bb->d_counter, 0};
            A.stage_cap = bb->stage_cap;
            cudaMemsetAsync(bb->d_counter, 0, sizeof(uint32_t), bb->st);
            sps::batch::k_batch_solve<<<std::min(bb->blocks, sample), sps::kBlock, bb->dyn_smem, bb->st>>>(A, sched);
            cudaMemcpyAsync(outs.data(), bb->d_out, sizeof(Ctl) * count, cudaMemcpyDeviceToHost, bb->st);
            if (cudaStreamSynchronize(bb->st) != cudaSuccess) return false;
            double tot = 0.0;
            for (int32_t q = 0; q < sample; ++q) tot += 1e-6 * double(outs[pick[q]].t_end - outs[pick[q]].t_begin);
            *cost = float(tot);
            return true;
        };
        const int g_opt = opt.batch_group;
        int gc = 0, gr = 32;
        double best = 1e300;
        float ms = 0.f;
        if (g_opt == 1 || g_opt == 2 || g_opt == 4 || g_opt == 8 || g_opt == 16 || g_opt == 32) {
            gc = g_opt;
        } else {
            for (int G : {1, 2, 4, 8, 16, 32}) {
                if (!time_one(sps::batch::pack_schedule(G, 32), &ms)) {
                    sps::set_create_error(std::string("autotune: ") + cudaGetErrorString(cudaGetLastError()));
                    return SPS_ERR_CUDA;
                }
                if (ms < best) { best = ms; gc = G; }
            }
        }
        best = 1e300;
        for (int R : {4, 8, 16, 32}) {
            if (!time_one(sps::batch::pack_schedule(gc, R), &ms)) {
                sps::set_create_error(std::string("autotune: ") + cudaGetErrorString(cudaGetLastError()));
                return SPS_ERR_CUDA;
            }
            if (ms < best) { best = ms; gr = R; }
        }
        bb->G = gc;
        bb->Gr = gr;
        std::lock_guard<std::mutex> lk(g_schedule_mu);
        g_schedules[key] = {gc, gr};
    }
    *out = b.release();
    return SPS_OK;
}

extern "C" int sps_batch_solve(sps_batch* b, sps_batch_stats* stats) {
    sps::NvtxRange nvtx_range("sps_batch_solve");
    if (!b) return SPS_ERR_INVALID;
    SPB_CK(cudaSetDevice(b->opt.device));
    const int64_t W = b->opt.check_interval > 0 ? b->opt.check_interval : 64;
    const uint64_t tl = b->opt.time_limit_s > 0 ? (uint64_t)(b->opt.time_limit_s * 1e9) : 0;
    sps::batch::Args A{b->d_inst, b->d_order, b->count, (int32_t)W, b->opt.max_iters, b->opt.tol, b->d_deadline,
                       b->arr, b->d_out, b->d_counter, b->opt.escalate != 0 ? 1 : 0, b->warm,
                       b->opt.warm_fallback ? 1 : 0, b->d_wx, b->d_wy, b->d_wom, b->d_cold_rel,
                       b->team, b->team_nnz, b->d_team_error, b->stage_cap, b->d_idle,
                       (uint32_t)(b->blocks - b->blocks / 8), b->handoff_nnz};
    auto enqueue = [&](cudaStream_t s) {
        cudaMemsetAsync(b->d_counter, 0, sizeof(uint32_t), s);
        sps::batch::k_set_deadline<<<1, 32, 0, s>>>(b->d_deadline, tl);
        cudaMemsetAsync(b->d_team_error, 0, sizeof(int32_t), s);
        cudaMemsetAsync(b->d_idle, 0, sizeof(uint32_t), s);
        const int sched = sps::batch::pack_schedule(b->G, b->Gr);
        if (b->team > 1) {
            cudaLaunchConfig_t cfg = {};
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeClusterDimension;
            attr[0].val.clusterDim.x = b->team;
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.gridDim = dim3(b->blocks);
            cfg.blockDim = dim3(sps::kBlock);
            cfg.dynamicSmemBytes = b->dyn_smem;
            cfg.stream = s;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            cudaLaunchKernelEx(&cfg, sps::batch::k_batch_solve, A, sched);
        } else {
            sps::batch::k_batch_solve<<<b->blocks, sps::kBlock, b->dyn_smem, s>>>(A, sched);
        }
    };
    SPB_CK(cudaEventRecord(b->e0, b->st));
    if (b->opt.graph_mode != 0) {
        // one graph (counter reset, deadline, persistent solve), built once per
        // schedule and time limit and replayed by later solves
        const int sched = sps::batch::pack_schedule(b->G, b->Gr);
        if (!b->gexec || b->gexec_G != sched || b->gexec_tl != tl || b->gexec_warm != b->warm) {
            if (b->gexec) { cudaGraphExecDestroy(b->gexec); b->gexec = nullptr; }
            cudaGraph_t g;
            cudaStream_t cap;
            SPB_CK(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
            cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
            if (e == cudaSuccess) {
                enqueue(cap);
                e = cudaStreamEndCapture(cap, &g);
            }
            if (e == cudaSuccess) {
                e = cudaGraphInstantiate(&b->gexec, g, 0);
                cudaGraphDestroy(g);
            }
            cudaStreamDestroy(cap);
            SPB_CK(e);
            b->gexec_G = sched;
            b->gexec_tl = tl;
            b->gexec_warm = b->warm;
        }
        SPB_CK(cudaGraphLaunch(b->gexec, b->st));
    } else {
        enqueue(b->st);
        SPB_CK(cudaGetLastError());
    }
    SPB_CK(cudaEventRecord(b->e1, b->st));
    sps::batch::k_batch_extract<<<b->count, sps::kBlock, 0, b->st>>>(b->d_inst, b->d_out, b->arr, b->d_xo, b->d_yo);
    SPB_CK(cudaGetLastError());
    b->out.resize(b->count);
    b->xo.resize(b->sum_n);
    b->yo.resize(b->sum_m);
    SPB_CK(cudaMemcpyAsync(b->out.data(), b->d_out, sizeof(Ctl) * b->count, cudaMemcpyDeviceToHost, b->st));
    SPB_CK(cudaMemcpyAsync(b->xo.data(), b->d_xo, sizeof(double) * b->sum_n, cudaMemcpyDeviceToHost, b->st));
    SPB_CK(cudaMemcpyAsync(b->yo.data(), b->d_yo, sizeof(double) * b->sum_m, cudaMemcpyDeviceToHost, b->st));
    SPB_CK(cudaStreamSynchronize(b->st));
    float ms = 0;
    cudaEventElapsedTime(&ms, b->e0, b->e1);
    int32_t team_err = 0;
    SPB_CK(cudaMemcpy(&team_err, b->d_team_error, sizeof(int32_t), cudaMemcpyDeviceToHost));
    if (team_err) return b->fail(SPS_ERR_CUDA, "a team barrier of the batched solve timed out");
    b->escalated.assign(b->count, 0);
    b->handed_off.assign(b->count, 0);
    b->esc_ms.assign(b->count, 0.0);
    int32_t n_esc = 0, n_hand = 0;
    double esc_ms = 0.0;
    {
        // Continuations on the single-LP engine, all at once (up to 32 host
        // threads; each has its own engine and stream, and their latency-bound
        // kernels overlap on the GPU): FP64 for the instances that stalled in FP32
        // (escalate = 1), FP32 for the ones handed off from the launch's tail.
        const auto t0 = std::chrono::steady_clock::now();
        std::vector<int32_t> todo;
        for (int32_t k = 0; k < b->count; ++k) {
            const int32_t st = b->out[k].status;
            if ((st == SPS_STATUS_STALLED && b->opt.escalate == 1) || st == sps::batch::kStatusHandoff) todo.push_back(k);
        }
        std::vector<int> rcs(todo.size(), SPS_OK);
        std::vector<std::string> whys(todo.size());
        std::atomic<size_t> next{0};
        auto work = [&]() {
            for (size_t i; (i = next.fetch_add(1)) < todo.size();) {
                const int32_t k = todo[i];
                const auto t1 = std::chrono::steady_clock::now();
                const double used = ms * 1e-3 + std::chrono::duration<double>(t1 - t0).count();
                rcs[i] = continue_single(b, k, used, &whys[i]);
                b->esc_ms[k] = 1e3 * std::chrono::duration<double>(std::chrono::steady_clock::now() - t1).count();
            }
        };
        const int nt = (int)std::min<size_t>(todo.size(), 32);
        std::vector<std::thread> pool;
        for (int t = 1; t < nt; ++t) pool.emplace_back(work);
        if (!todo.empty()) work();
        for (auto& th : pool) th.join();
        for (size_t i = 0; i < todo.size(); ++i)
            if (rcs[i] != SPS_OK) return b->fail(rcs[i], whys[i]);
        for (int32_t k : todo) {
            n_esc += b->escalated[k];
            n_hand += b->handed_off[k];
        }
        esc_ms = todo.empty() ? 0.0 : 1e3 * std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    b->solve_ms = ms + esc_ms;
    b->solved = true;
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->setup_ms = b->setup_ms;
        stats->solve_ms = b->solve_ms;
        stats->lanes_per_column = b->G;
        stats->lanes_per_row = b->Gr;
        stats->team = b->team;
        stats->blocks = b->blocks;
        stats->escalated = n_esc;
        stats->handed_off = n_hand;
        for (const Ctl& c : b->out) {
            stats->total_iterations += c.iters;
            if (c.status == SPS_STATUS_OPTIMAL) stats->optimal += 1;
        }
    }
    return SPS_OK;
}

extern "C" int sps_batch_set_warm_starts(sps_batch* b, const double* x0, const double* y0, const double* omega0) {
    if (!b) return SPS_ERR_INVALID;
    if (!x0 && !y0) {
        b->warm = 0;
        return SPS_OK;
    }
    if (b->opt.mode != SPS_MODE_ADAPTIVE) return b->fail(SPS_ERR_STATE, "warm starts need the adaptive mode");
    SPB_CK(cudaSetDevice(b->opt.device));
    if (!b->d_wx) {
        SPB_CK(b->alloc(&b->d_wx, b->sum_n));
        SPB_CK(b->alloc(&b->d_wy, b->sum_m));
        SPB_CK(b->alloc(&b->d_wom, b->count));
    }
    auto finite = [](const double* v, int64_t len) {
        for (int64_t t = 0; t < len; ++t)
            if (!std::isfinite(v[t])) return false;
        return true;
    };
    if ((x0 && !finite(x0, b->sum_n)) || (y0 && !finite(y0, b->sum_m)))
        return b->fail(SPS_ERR_INVALID, "non-finite warm start");
    std::vector<double> om(b->count, -1.0);
    if (omega0)
        for (int32_t k = 0; k < b->count; ++k) om[k] = std::isfinite(omega0[k]) ? omega0[k] : -1.0;
    if (x0) SPB_CK(cudaMemcpyAsync(b->d_wx, x0, sizeof(double) * b->sum_n, cudaMemcpyHostToDevice, b->st));
    else SPB_CK(cudaMemsetAsync(b->d_wx, 0, sizeof(double) * b->sum_n, b->st));
    if (y0) SPB_CK(cudaMemcpyAsync(b->d_wy, y0, sizeof(double) * b->sum_m, cudaMemcpyHostToDevice, b->st));
    else SPB_CK(cudaMemsetAsync(b->d_wy, 0, sizeof(double) * b->sum_m, b->st));
    SPB_CK(cudaMemcpyAsync(b->d_wom, om.data(), sizeof(double) * b->count, cudaMemcpyHostToDevice, b->st));
    SPB_CK(cudaStreamSynchronize(b->st));
    b->warm = 1;
    return SPS_OK;
}

extern "C" int sps_batch_set_warm_starts_gnn(sps_batch* b, sps_gnn* g, const double* scales) {
    sps::NvtxRange nvtx_range("sps_batch_set_warm_starts_gnn");
    if (!b) return SPS_ERR_INVALID;
    if (!g || !scales) return b->fail(SPS_ERR_INVALID, "need a network and its four scales");
    for (int q = 0; q < 4; ++q)
        if (!(scales[q] > 0.0) || !std::isfinite(scales[q])) return b->fail(SPS_ERR_INVALID, "scales must be positive");
    sps::gnn::DeviceIO io{};
    if (sps::gnn::device_io(g, &io) != 0) return b->fail(SPS_ERR_INVALID, "invalid network");
    if (!io.lp_features) return b->fail(SPS_ERR_INVALID, "the network must take LP features (lp_features = 1)");
    if (io.device != b->opt.device) return b->fail(SPS_ERR_INVALID, "the network lives on another device");
    if (b->opt.mode != SPS_MODE_ADAPTIVE) return b->fail(SPS_ERR_STATE, "warm starts need the adaptive mode");
    for (int32_t k = 0; k < b->count; ++k)
        if (b->inst[k].n != io.n || b->inst[k].m != io.m)
            return b->fail(SPS_ERR_INVALID, "instance " + std::to_string(k) + " does not have the network's shape");
    SPB_CK(cudaSetDevice(b->opt.device));
    if (!b->d_wx) {
        SPB_CK(b->alloc(&b->d_wx, b->sum_n));
        SPB_CK(b->alloc(&b->d_wy, b->sum_m));
        SPB_CK(b->alloc(&b->d_wom, b->count));
    }
    for (int32_t s0 = 0; s0 < b->count; s0 += io.max_batch) {
        const int cnt = std::min<int32_t>(io.max_batch, b->count - s0);
        const int64_t work = (int64_t)cnt * std::max(io.n, io.m);
        const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((work + 255) / 256, 152 * 8));
        sps::batch::k_gnn_inputs<<<grid, sps::kBlock, 0, io.stream>>>(b->d_inst, s0, cnt, b->arr, io.n, io.m,
                                                                      1.0 / scales[0], 1.0 / scales[1], io.c_in,
                                                                      io.b_in);
        SPB_CK(cudaGetLastError());
        if (int rc = sps::gnn::forward_in_place(g, cnt))
            return b->fail(rc == -1 ? SPS_ERR_INVALID : SPS_ERR_CUDA, std::string("network: ") + sps_gnn_last_error(g));
        sps::batch::k_gnn_outputs<<<grid, sps::kBlock, 0, io.stream>>>(b->d_inst, s0, cnt, io.n, io.m, io.x0, io.y0,
                                                                       io.log_omega, scales[2], scales[3], b->d_wx,
                                                                       b->d_wy, b->d_wom);
        SPB_CK(cudaGetLastError());
    }
    SPB_CK(cudaStreamSynchronize(io.stream));
    if (sps::gnn::check_device_error(g) != 0)
        return b->fail(SPS_ERR_CUDA, std::string("network: ") + sps_gnn_last_error(g));
    b->warm = 1;
    return SPS_OK;
}

extern "C" int sps_batch_get(sps_batch* b, int32_t k, double* x, double* y, sps_result* res) {
    if (!b || k < 0 || k >= b->count) return SPS_ERR_INVALID;
    if (!b->solved) return b->fail(SPS_ERR_STATE, "call sps_batch_solve first");
    const Inst& I = b->inst[k];
    const Ctl& c = b->out[k];
    double obj = 0.0;
    for (int32_t j = 0; j < I.n; ++j) {
        const double lo = std::isfinite(b->lb_all[I.vc + j]) ? b->lb_all[I.vc + j] : -1e30;
        const double hi = std::isfinite(b->ub_all[I.vc + j]) ? b->ub_all[I.vc + j] : 1e30;
        const double v = std::min(std::max(b->xo[I.vc + j], lo), hi);
        if (x) x[j] = v;
        obj += b->c_all[I.vc + j] * v;
    }
    if (y) std::memcpy(y, b->yo.data() + I.vr, sizeof(double) * I.m);
    if (res) {
        std::memset(res, 0, sizeof(*res));
        res->status = c.status;
        res->restarts = c.restarts;
        res->iterations = c.iters;
        res->accepted_steps = c.accepted_total;
        res->objective = obj;
        res->rel_kkt = c.rel_kkt;
        res->rel_kkt_lagrangian = c.rel_kkt;
        res->rel_primal = c.rel_p;
        res->rel_dual = c.rel_d;
        res->rel_gap = c.rel_gap;
        res->primal_weight = c.omega;
        res->step_size = c.eta;
        res->setup_ms = b->setup_ms;
        res->solve_ms = 1e-6 * double(c.t_end - c.t_begin) + b->esc_ms[k];
        res->kernel_launches = 1;
        res->returned_average = c.choice;
        res->escalated = b->escalated[k];
        res->warm_start_used = c.warm_used;
    }
    return SPS_OK;
}

extern "C" const char* sps_batch_last_error(const sps_batch* b) { return b ? b->err.c_str() : ""; }

extern "C" void sps_batch_destroy(sps_batch* b) { delete b; }
