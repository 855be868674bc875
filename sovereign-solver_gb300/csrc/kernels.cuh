// kernels.cuh — PDHG iteration, check and apply kernels (templated on V).
//
// Adaptive mode, one step attempt = two kernels:
//   ad_row_step  (CSR pass)  K x'  fused with the dual update and projection,
//                            partials of ||y'-y||^2 and (y'-y)^T K (x'-x);
//                            its last block takes the step-size decision.
//   ad_col_step  (CSC pass)  K^T y' (only if the attempt was accepted) fused
//                            with the weighted-average update and the NEXT
//                            primal candidate x'' = proj(x - tau (c - K^T y)).
// Every `check_interval` attempts:
//   ad_row_check / ad_col_check  FP64 KKT of the average and of the current
//                            point (both gathers share one matrix read); the
//                            last block decides termination / restart / weight.
//   ad_apply                 restart copies, new candidate, loop condition.
//
// Reference mode (solver/lp/pdhg.py:209-244), one iteration = two kernels:
//   rf_col_step  (CSC pass)  A^T y fused with x' = max(0, x - tau (c - A^T y)),
//                            x_bar = 2x' - x and the x sum.
//   rf_row_step  (CSR pass)  A x_bar fused with y += sigma (b - A x_bar) and the y sum.
// Every 50 iterations: rf_row_check / rf_col_check (KKT of the average in
// FP64, decision in the last block), rf_apply.
#pragma once

#include "decide.cuh"

namespace sps {

template <class V>
struct Args {
    int32_t n, m;
    Layout<V> csr, csc;
    BinTable rows, cols;
    BinTable rows_chk, cols_chk;   // the same bins with the check kernels' block shares (one wave
                                   // at their own occupancy: they hold more registers)
    int32_t col_tail_blocks;   // extra blocks of ad_col_step (0: its column blocks also sweep the rows)
    int32_t apply_blocks;
    const V* c; const V* b; const V* lo; const V* hi;
    V lo_u, hi_u;
    int32_t uniform_bounds;
    int32_t far_residual;      // SPS_KKT_PDLP: far finite bounds leave the dual objective
    const double* dr; const double* dc;
    const double* idr; const double* idc;    // adaptive: 1 / dr, 1 / dc (the checks multiply)
    const V* tau; const V* sigma;
    double inv_nb, inv_nc;     // normalisers of the reported relative error
    V* X[2]; V* Y[2]; V* AX[2]; V* ATY[2];
    V* xs; V* ys; V* xl; V* yl; V* AXa; V* ATYa; V* xbar;
    V* xb; V* yb;              // best point of the stall test (null unless it is on)
    V* AXl; V* ATYl;           // adaptive: K x_last, K^T y_last (infeasibility tests)
    double* px[2]; double* py[2];   // adaptive: the check's two points (average, current) in FP64
    double* part_row; double* part_col; double* part_aux;
    Ctl* ctl;
    const volatile int32_t* abort_flag;
    cudaGraphConditionalHandle cond;
    int32_t has_cond;
    int32_t pdl;               // launch the step kernels' programmatic-dependent instantiations
    int32_t check_interval;
    int64_t max_windows;
};


// iteration kernels: register budget for kPassMinBlocks resident blocks per SM;
// check kernels (FP64 accumulators, once per window) get the default budget
#define SPS_PASS_KERNEL __global__ void __launch_bounds__(kBlock, kPassMinBlocks)
#define SPS_CHECK_KERNEL __global__ void __launch_bounds__(kBlock)

// --- precision helpers -------------------------------------------------------
__device__ __forceinline__ float rn_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double rn_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float rn_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double rn_sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float rn_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double rn_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float rn_div(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double rn_div(double a, double b) { return __ddiv_rn(a, b); }

template <class V>
__device__ __forceinline__ V lo_at(const Args<V>& a, int j) { return a.uniform_bounds ? a.lo_u : a.lo[j]; }
template <class V>
__device__ __forceinline__ V hi_at(const Args<V>& a, int j) { return a.uniform_bounds ? a.hi_u : a.hi[j]; }
template <class V>
__device__ __forceinline__ V clampv(V x, V lo, V hi) { return fmin(fmax(x, lo), hi); }

// Loop condition of the device-driven while graph: set by one thread only.
template <class V>
__device__ __forceinline__ void set_loop_condition(const Args<V>& a, Ctl* ctl) {
    ctl->windows += 1;
    const bool keep = !ctl->done && ctl->iters < ctl->max_iters && ctl->windows < a.max_windows;
    if (a.has_cond) cudaGraphSetConditional(a.cond, keep ? 1u : 0u);
}

// Shared stop conditions checked at every KKT check: device deadline and host abort.
__device__ __forceinline__ bool stop_requested(const Ctl* ctl, const volatile int32_t* abort_flag) {
    if (abort_flag && *abort_flag) return true;
    return ctl->deadline_ns && global_ns() > ctl->deadline_ns;
}

template <class V>
struct GatherOne {
    const V* x;
    __device__ __forceinline__ V operator()(int, int j) const { return __ldg(x + j); }
};

// ============================================================================
// Adaptive mode
// ============================================================================

template <class V>
struct AdRowStepEpi {
    const V *b, *axo, *yo;
    V *axn, *yn;
    V sigma;
    V dy2 = V(0), inter = V(0);          // per-thread partials; FP64 from the block sum on
    struct Pre { V ao, yv, br; };
    static constexpr int NP = 2;
    using R = V;
    __device__ __forceinline__ void zero() { dy2 = inter = V(0); }
    __device__ __forceinline__ void export_to(R* d) const { d[0] = dy2; d[1] = inter; }
    __device__ __forceinline__ Pre pre(int r) const { return Pre{axo[r], yo[r], b[r]}; }
    __device__ __forceinline__ void operator()(int r, int kind, const V (&acc)[1], const Pre& p) {
        const V ax = acc[0];
        axn[r] = ax;
        V y2 = p.yv + sigma * (p.br - (ax + ax - p.ao));
        if (kind) y2 = fmin(y2, V(0));
        yn[r] = y2;
        const V dy = y2 - p.yv;
        dy2 += dy * dy;
        inter += dy * (ax - p.ao);
    }
};

// Operands of row r in both state buffers (the pass reads one of them).
template <class V>
struct RowTouch {
    const Args<V>* a;
    __device__ __forceinline__ void operator()(int r) const {
        prefetch_l1(a->b + r);
        prefetch_l1(a->AX[0] + r);
        prefetch_l1(a->AX[1] + r);
        prefetch_l1(a->Y[0] + r);
        prefetch_l1(a->Y[1] + r);
    }
};

// Pdl: launched as a programmatic dependent (a separate instantiation, so the
// plain kernel's code is not touched by the prologue).
template <class V, bool Pdl = false>
SPS_PASS_KERNEL ad_row_step(Args<V> a) {
    if constexpr (Pdl) {
        prefetch_first_unit(a.rows, blockIdx.x, a.csr, RowTouch<V>{&a});
        grid_dep_wait();
    }
    Ctl* ctl = a.ctl;
    if (ctl->done || ctl->iters >= ctl->max_iters) return;
    __shared__ V sm[kWarps * 4];
    __shared__ bool last;
    const int cur = ctl->cur;
    const V sigma = block_scalar<V>([&] { return ctl->eta * ctl->omega; });
    AdRowStepEpi<V> e{a.b, a.AX[cur], a.Y[cur], a.AX[1 - cur], a.Y[1 - cur], sigma};
    visit_bins<1, V>(a.rows, blockIdx.x, a.csr, GatherOne<V>{a.X[1 - cur]}, e);
    if constexpr (Pdl) grid_dep_launch_dependents();
    // reductions in V: FP32 sums in the FP32 engine (the step rule's inputs)
    V v[2] = {e.dy2, e.inter};
    V* part = reinterpret_cast<V*>(a.part_row);
    if (!publish_partials<2>(v, part, &ctl->ticket[T_ROW_STEP], sm, &last)) return;
    V t[2];
    gather_all_partials<2>(t, part, gridDim.x, a.csr, sm);
    if (threadIdx.x != 0) return;
    ctl->ticket[T_ROW_STEP] = 0;
    decide_step(*ctl, double(t[0]), double(t[1]));
}

template <class V>
struct AdColStepEpi {
    const Args<V>* a;
    const V *xc, *cc, *atyo;
    const V* xl;
    V *aty, *xn, *xs;
    V tau, wgt;
    bool accepted;
    V dx2 = V(0);
    struct Pre { V xj, cj, lo, hi, s, l; };
    static constexpr int NP = 1;
    using R = V;
    __device__ __forceinline__ void zero() { dx2 = V(0); }
    __device__ __forceinline__ void export_to(R* d) const { d[0] = dx2; }
    __device__ __forceinline__ Pre pre(int j) const {
        Pre p;
        p.xj = xc[j];
        p.cj = cc[j];
        p.lo = lo_at(*a, j);
        p.hi = hi_at(*a, j);
        p.s = accepted ? xs[j] : V(0);
        p.l = accepted ? xl[j] : V(0);
        return p;
    }
    __device__ __forceinline__ void finish(int j, V atyj, const Pre& p) {
        if (accepted) { aty[j] = atyj; xs[j] = p.s + wgt * (p.xj - p.l); }
        const V x2 = clampv(p.xj - tau * (p.cj - atyj), p.lo, p.hi);
        xn[j] = x2;
        const V d = x2 - p.xj;
        dx2 += d * d;
    }
    __device__ __forceinline__ void operator()(int j, int, const V (&acc)[1], const Pre& p) { finish(j, acc[0], p); }
};

// Operands of column j in both state buffers (the pass reads one of them).
template <class V>
struct ColTouch {
    const Args<V>* a;
    __device__ __forceinline__ void operator()(int j) const {
        prefetch_l1(a->X[0] + j);
        prefetch_l1(a->X[1] + j);
        prefetch_l1(a->c + j);
        prefetch_l1(a->xs + j);
        prefetch_l1(a->xl + j);
    }
};

template <class V, bool Pdl = false>
SPS_PASS_KERNEL ad_col_step(Args<V> a) {
    if constexpr (Pdl) {
        prefetch_first_unit(a.cols, blockIdx.x, a.csc, ColTouch<V>{&a});
        grid_dep_wait();
    }
    Ctl* ctl = a.ctl;
    if (ctl->apply != AP_STEP_PENDING) return;
    __shared__ V sm[kWarps * 2];
    __shared__ bool last;
    const int cur = ctl->cur;
    const bool acc = ctl->accepted;
    const V tau = block_scalar<V>([&] { return ctl->eta / ctl->omega; });
    const V wgt = block_scalar<V>([&] { return ctl->eta_used; });
    AdColStepEpi<V> e{&a, a.X[cur], a.c, a.ATY[cur], a.xl, a.ATY[cur], a.X[1 - cur], a.xs, tau, wgt, acc};
    const int colblocks = a.cols.total_blocks;
    if (acc) {
        visit_bins<1, V>(a.cols, blockIdx.x, a.csc, GatherOne<V>{a.Y[cur]}, e);
        // the dual average's running sum, in the same blocks (extra blocks for it ran
        // as a second wave after the columns; it adds nothing to the step partials)
        const V* yc = a.Y[cur];
        for (int i = blockIdx.x * kBlock + threadIdx.x; i < a.m; i += colblocks * kBlock)
            a.ys[i] += wgt * (yc[i] - a.yl[i]);
    } else {
        for (int j = blockIdx.x * kBlock + threadIdx.x; j < a.n; j += colblocks * kBlock)
            e.finish(j, e.atyo[j], e.pre(j));
    }
    if constexpr (Pdl) grid_dep_launch_dependents();
    V v[1] = {e.dx2};
    V* part = reinterpret_cast<V*>(a.part_col);
    if (!publish_partials<1>(v, part, &ctl->ticket[T_COL_STEP], sm, &last)) return;
    V t[1];
    gather_all_partials<1>(t, part, gridDim.x, a.csc, sm);
    if (threadIdx.x != 0) return;
    ctl->ticket[T_COL_STEP] = 0;
    ctl->dx2 = double(t[0]);
    ctl->apply = 0;
}

// ---- checks -----------------------------------------------------------------
// Point 0 = weighted average, point 1 = current iterate.  The average is kept
// as an offset from the restart point: x_avg = x_last + x_sum / w_sum with
// x_sum = sum of w_k (x_k - x_last).  Near convergence the offsets are small,
// so FP32 sums keep the average accurate where a plain FP32 sum of w_k x_k
// loses the last digits and stalls the restarts.  With no average yet point 0
// aliases the current iterate (s = current, l = null, inv_w = 1).

template <class V>
__device__ __forceinline__ double avg_at(const V* s, const V* l, double inv_w, int j) {
    const double v = double(__ldg(s + j)) * inv_w;
    return l ? v + double(__ldg(l + j)) : v;
}

// The check's two points in FP64 (written by ad_check_prep), gathered as is.
struct GatherPts {
    const double *p0, *p1;
    __device__ __forceinline__ double operator()(int q, int j) const { return __ldg((q == 0 ? p0 : p1) + j); }
};

template <class V>
struct AdRowCheckEpi {
    const Args<V>* a;
    const V *ys, *ylb, *yc, *yl;
    V* axa;
    double inv_w;
    // per point q: res_scaled^2, res_orig^2, b^T y, ||y - y_last||^2; then ||K dx||^2 (row cones),
    // b^T dy, and dy's violation of the dual cone
    double p[kRowPartials] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    using Pre = NoPre;
    static constexpr int NP = kRowPartials;
    using R = double;
    __device__ __forceinline__ void zero() { for (int q = 0; q < NP; ++q) p[q] = 0.0; }
    __device__ __forceinline__ void export_to(double* d) const { for (int q = 0; q < NP; ++q) d[q] = p[q]; }
    __device__ __forceinline__ Pre pre(int) const { return Pre{}; }
    __device__ __forceinline__ void operator()(int r, int kind, const double (&acc)[2], const Pre&) {
        const double br = double(a->b[r]), idr = a->idr[r];
        axa[r] = V(acc[0]);
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            double res = acc[q] - br;
            if (kind) res = fmax(res, 0.0);
            p[4 * q + 0] += res * res;
            const double ro = res * idr;
            p[4 * q + 1] += ro * ro;
            const double yv = __ldg(a->py[q] + r);
            p[4 * q + 2] += br * yv;
            const double d = yv - double(yl[r]);
            p[4 * q + 3] += d * d;
        }
        double kdx = acc[1] - double(a->AXl[r]);
        if (kind) kdx = fmax(kdx, 0.0);
        p[8] += kdx * kdx;
        const double dy = __ldg(a->py[1] + r) - double(yl[r]);
        p[9] += br * dy;
        if (kind) p[10] += fmax(dy, 0.0) * fmax(dy, 0.0);
    }
};

// The check's two points as FP64 vectors, once per check: the average
// x_last + x_sum / w_sum (the current iterate while there is no average yet) and
// the current iterate, for x and y.  The checks then gather and read doubles
// (no conversion or average per nonzero on GB300's slow FP64 pipe); the values
// are the ones the checks computed per nonzero before, so every sum is unchanged.
template <class V>
__global__ void __launch_bounds__(kBlock) ad_check_prep(Args<V> a) {
    const Ctl* ctl = a.ctl;
    if (ctl->done) return;
    const int cur = ctl->cur;
    const bool has_avg = ctl->w_sum > 0.0;
    const double inv_w = has_avg ? 1.0 / ctl->w_sum : 1.0;
    const int stride = gridDim.x * kBlock;
    for (int j = blockIdx.x * kBlock + threadIdx.x; j < a.n; j += stride) {
        const double xc = double(a.X[cur][j]);
        a.px[0][j] = has_avg ? avg_at(a.xs, a.xl, inv_w, j) : xc;
        a.px[1][j] = xc;
    }
    for (int i = blockIdx.x * kBlock + threadIdx.x; i < a.m; i += stride) {
        const double yc = double(a.Y[cur][i]);
        a.py[0][i] = has_avg ? avg_at(a.ys, a.yl, inv_w, i) : yc;
        a.py[1][i] = yc;
    }
}

template <class V>
SPS_CHECK_KERNEL ad_row_check(Args<V> a) {
    Ctl* ctl = a.ctl;
    if (ctl->done) return;
    __shared__ double sm[kWarps * kRowPartials];
    const int cur = ctl->cur;
    // with no average yet, point 0 aliases the current iterate
    const bool has_avg = ctl->w_sum > 0.0;
    const double inv_w = has_avg ? 1.0 / ctl->w_sum : 1.0;
    GatherPts g{a.px[0], a.px[1]};
    AdRowCheckEpi<V> e{&a, has_avg ? a.ys : a.Y[cur], has_avg ? a.yl : nullptr, a.Y[cur], a.yl, a.AXa, inv_w};
    visit_bins<2, double>(a.rows_chk, blockIdx.x, a.csr, g, e);
    block_sum<kRowPartials>(e.p, sm);
    if (threadIdx.x == 0)
        for (int q = 0; q < kRowPartials; ++q) a.part_row[(size_t)blockIdx.x * kRowPartials + q] = e.p[q];
}

// Far = true: the PDLP error form (far finite bounds leave the dual objective),
// with the Lagrangian form's dual residual and bound terms as kLagPartials more
// partials; Far = false: the Lagrangian form (the default).
template <class V, bool Far>
struct AdColCheckEpi {
    static constexpr int NP = kColPartials + (Far ? kLagPartials : 0);
    const Args<V>* a;
    const V *xs, *xlb, *xc, *xl;
    V* atya;
    double inv_w;
    // per point: dres_s^2, dres_o^2, c^T x, bound terms, ||x - x_last||^2; then for the
    // change since the last restart: cone residual^2 of -K^T dy, its bound terms,
    // recession-cone violation^2 of dx, c^T dx; with Far, the Lagrangian form's
    // dres_o^2 of both points, then its bound terms of both points
    double p[NP] = {};
    bool nonneg;               // every column in [0, +inf): the bound terms vanish
    using Pre = NoPre;
    using R = double;
    __device__ __forceinline__ void zero() { for (int q = 0; q < NP; ++q) p[q] = 0.0; }
    __device__ __forceinline__ void export_to(double* d) const { for (int q = 0; q < NP; ++q) d[q] = p[q]; }
    __device__ __forceinline__ Pre pre(int) const { return Pre{}; }
    __device__ __forceinline__ void operator()(int j, int, const double (&acc)[2], const Pre&) {
        if (nonneg) nonneg_column(j, acc);
        else general_column(j, acc);
    }
    // x >= 0 only (lo = 0, hi = +inf): lambda = max(rc, 0), so the dual residual is
    // min(rc, 0) and every bound term lo * max(lambda, 0) + hi * min(lambda, 0) is 0;
    // the same partials as the general case with ~20 fewer FP64 operations per column
    __device__ __forceinline__ void nonneg_column(int j, const double (&acc)[2]) {
        const double cj = double(a->c[j]), idc = a->idc[j];
        atya[j] = V(acc[0]);
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const double dres = fmin(cj - acc[q], 0.0);
            p[5 * q + 0] += dres * dres;
            const double dor = dres * idc;
            p[5 * q + 1] += dor * dor;
            const double xv = __ldg(a->px[q] + j);
            p[5 * q + 2] += cj * xv;
            const double d = xv - double(xl[j]);
            p[5 * q + 4] += d * d;
            if constexpr (Far) p[kColPartials + q] += dor * dor;   // a zero lower bound is never far
        }
        const double lv = fmin(double(a->ATYl[j]) - acc[1], 0.0);
        p[10] += lv * lv;
        const double dx = __ldg(a->px[1] + j) - double(xl[j]);
        const double vx = fmin(dx, 0.0);
        p[12] += vx * vx;
        p[13] += cj * dx;
    }
    __device__ __forceinline__ void general_column(int j, const double (&acc)[2]) {
        const double cj = double(a->c[j]), idc = a->idc[j];
        const double lo = double(lo_at(*a, j)), hi = double(hi_at(*a, j));
        const bool hl = isfinite(lo), hh = isfinite(hi);
        atya[j] = V(acc[0]);
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const double rc = cj - acc[q];
            const double xv = __ldg(a->px[q] + j);
            // PDLP form: a bound farther from x than |x| (a scale-free test) takes no part of rc
            const bool nl = hl && (!Far || fabs(xv - lo) <= fabs(xv));
            const bool nh = hh && (!Far || fabs(xv - hi) <= fabs(xv));
            const double lam = (nl && nh) ? rc : nl ? fmax(rc, 0.0) : nh ? fmin(rc, 0.0) : 0.0;
            const double dres = rc - lam;
            p[5 * q + 0] += dres * dres;
            const double dor = dres * idc;
            p[5 * q + 1] += dor * dor;
            p[5 * q + 2] += cj * xv;
            p[5 * q + 3] += (nl ? lo * fmax(lam, 0.0) : 0.0) + (nh ? hi * fmin(lam, 0.0) : 0.0);
            const double d = xv - double(xl[j]);
            p[5 * q + 4] += d * d;
            if constexpr (Far) {    // the Lagrangian form of the same point
                const double lg = (hl && hh) ? rc : hl ? fmax(rc, 0.0) : hh ? fmin(rc, 0.0) : 0.0;
                const double dl = (rc - lg) * idc;
                p[kColPartials + q] += dl * dl;
                p[kColPartials + 2 + q] += (hl ? lo * fmax(lg, 0.0) : 0.0) + (hh ? hi * fmin(lg, 0.0) : 0.0);
            }
        }
        const double lr = -(acc[1] - double(a->ATYl[j]));
        const double lp = (hl && hh) ? lr : hl ? fmax(lr, 0.0) : hh ? fmin(lr, 0.0) : 0.0;
        p[10] += (lr - lp) * (lr - lp);
        p[11] += (hl ? lo * fmax(lp, 0.0) : 0.0) + (hh ? hi * fmin(lp, 0.0) : 0.0);
        const double dx = __ldg(a->px[1] + j) - double(xl[j]);
        const double vx = (hl && hh) ? dx : hl ? fmin(dx, 0.0) : hh ? fmax(dx, 0.0) : 0.0;
        p[12] += vx * vx;
        p[13] += cj * dx;
    }
};

template <class V, bool Far>
SPS_CHECK_KERNEL ad_col_check(Args<V> a) {
    using Epi = AdColCheckEpi<V, Far>;
    constexpr int NP = Epi::NP;
    Ctl* ctl = a.ctl;
    if (ctl->done) return;
    __shared__ double sm[kWarps * NP];
    __shared__ bool last;
    const int cur = ctl->cur;
    const bool has_avg = ctl->w_sum > 0.0;
    const double inv_w = has_avg ? 1.0 / ctl->w_sum : 1.0;
    GatherPts g{a.py[0], a.py[1]};
    Epi e{&a, has_avg ? a.xs : a.X[cur], has_avg ? a.xl : nullptr, a.X[cur], a.xl, a.ATYa, inv_w};
    e.nonneg = a.uniform_bounds && a.lo_u == V(0) && isinf(a.hi_u) && a.hi_u > V(0);
    visit_bins<2, double>(a.cols_chk, blockIdx.x, a.csc, g, e);
    if (!publish_partials<NP>(e.p, a.part_col, &ctl->ticket[T_COL_CHECK], sm, &last)) return;
    double tc[NP], tr[kRowPartials];
    gather_partials<NP>(tc, a.part_col, gridDim.x, sm);
    gather_partials<kRowPartials>(tr, a.part_row, a.rows_chk.total_blocks, sm);
    add_segment_rows<NP>(tc, a.csc, sm);
    add_segment_rows<kRowPartials>(tr, a.csr, sm);
    if (threadIdx.x != 0) return;
    ctl->ticket[T_COL_CHECK] = 0;
    decide_check(*ctl, reinterpret_cast<const double(&)[kColPartials]>(tc), tr, a.inv_nb, a.inv_nc,
                 stop_requested(ctl, a.abort_flag), Far ? tc + kColPartials : nullptr);
}

template <class V>
__global__ void __launch_bounds__(kBlock) ad_apply(Args<V> a) {
    Ctl* ctl = a.ctl;
    const int ap = ctl->apply;
    __shared__ V sm[kWarps];
    __shared__ bool last;
    if (ap != 0 && ap != AP_STEP_PENDING) {
        const int cur = ctl->cur;
        const bool load = ap & AP_LOAD_AVG, rst = ap & AP_RESTART, cand = (ap & AP_CANDIDATE) && !ctl->done;
        const bool save = (ap & AP_SAVE_BEST) && a.xb, save_avg = ap & AP_SAVE_AVG;
        const double inv_w = block_scalar<double>([&] { return ctl->w_sum > 0.0 ? 1.0 / ctl->w_sum : 0.0; });
        const V tau = block_scalar<V>([&] { return ctl->eta / ctl->omega; });
        V dx2 = V(0);
        const int stride = gridDim.x * kBlock;
        for (int j = blockIdx.x * kBlock + threadIdx.x; j < a.n; j += stride) {
            if (save) a.xb[j] = save_avg ? V(double(a.xl[j]) + double(a.xs[j]) * inv_w) : a.X[cur][j];
            V xv;
            if (load) {
                xv = V(double(a.xl[j]) + double(a.xs[j]) * inv_w);
                a.X[cur][j] = xv;
                a.ATY[cur][j] = a.ATYa[j];
            } else {
                xv = a.X[cur][j];
            }
            if (rst) {
                a.xl[j] = xv;
                a.xs[j] = V(0);
                a.ATYl[j] = a.ATY[cur][j];
            }
            if (cand) {
                const V x2 = clampv(xv - tau * (a.c[j] - a.ATY[cur][j]), lo_at(a, j), hi_at(a, j));
                a.X[1 - cur][j] = x2;
                const V d = x2 - xv;
                dx2 += d * d;
            }
        }
        for (int i = blockIdx.x * kBlock + threadIdx.x; i < a.m; i += stride) {
            if (save) a.yb[i] = save_avg ? V(double(a.yl[i]) + double(a.ys[i]) * inv_w) : a.Y[cur][i];
            V yv;
            if (load) {
                yv = V(double(a.yl[i]) + double(a.ys[i]) * inv_w);
                a.Y[cur][i] = yv;
                a.AX[cur][i] = a.AXa[i];
            } else {
                yv = a.Y[cur][i];
            }
            if (rst) {
                a.yl[i] = yv;
                a.ys[i] = V(0);
                a.AXl[i] = a.AX[cur][i];
            }
        }
        V v[1] = {dx2};
        V* part = reinterpret_cast<V*>(a.part_aux);
        if (publish_partials<1>(v, part, &ctl->ticket[T_APPLY], sm, &last)) {
            V t[1];
            gather_partials<1>(t, part, gridDim.x, sm);
            if (threadIdx.x == 0) {
                ctl->ticket[T_APPLY] = 0;
                if (cand) ctl->dx2 = double(t[0]);
                if (rst) ctl->w_sum = 0.0;
                ctl->apply = 0;
                set_loop_condition(a, ctl);
            }
        }
        return;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) set_loop_condition(a, ctl);
}

// Plain SpMV passes used at start-up: out = K x (rows) or out = K^T y (columns).
template <class V>
struct StoreEpi {
    V* out;
    using Pre = NoPre;
    static constexpr int NP = 0;
    __device__ __forceinline__ Pre pre(int) const { return Pre{}; }
    __device__ __forceinline__ void operator()(int r, int, const V (&acc)[1], const Pre&) { out[r] = acc[0]; }
};

template <class V>
SPS_CHECK_KERNEL spmv_rows(Args<V> a, const V* x, V* out) {
    StoreEpi<V> e{out};
    visit_bins<1, V>(a.rows, blockIdx.x, a.csr, GatherOne<V>{x}, e);
}

template <class V>
SPS_CHECK_KERNEL spmv_cols(Args<V> a, const V* y, V* out) {
    StoreEpi<V> e{out};
    visit_bins<1, V>(a.cols, blockIdx.x, a.csc, GatherOne<V>{y}, e);
}

// ============================================================================
// Reference mode (standard form: every row '=', x >= 0; tau, sigma vectors)
// Elementwise arithmetic is rounded op by op (no FMA contraction) in the
// reference's own order of operations.
// ============================================================================

template <class V>
struct RfColStepEpi {
    const V *tau, *c;
    V *x, *xbar, *xs;
    struct Pre { V xv, t, cj, s; };
    static constexpr int NP = 0;
    __device__ __forceinline__ Pre pre(int j) const { return Pre{x[j], tau[j], c[j], xs[j]}; }
    __device__ __forceinline__ void operator()(int j, int, const V (&acc)[1], const Pre& p) {
        V x2 = rn_sub(p.xv, rn_mul(p.t, rn_sub(p.cj, acc[0])));
        x2 = fmax(x2, V(0));
        xbar[j] = rn_sub(rn_mul(V(2), x2), p.xv);
        x[j] = x2;
        xs[j] = rn_add(p.s, x2);
    }
};

template <class V>
SPS_PASS_KERNEL rf_col_step(Args<V> a) {
    Ctl* ctl = a.ctl;
    if (ctl->done || ctl->iters >= ctl->max_iters) return;
    RfColStepEpi<V> e{a.tau, a.c, a.X[0], a.xbar, a.xs};
    visit_bins<1, V>(a.cols, blockIdx.x, a.csc, GatherOne<V>{a.Y[0]}, e);
}

template <class V>
struct RfRowStepEpi {
    const V *sigma, *b;
    V *y, *ys;
    struct Pre { V yv, s, br, acc_s; };
    static constexpr int NP = 0;
    __device__ __forceinline__ Pre pre(int r) const { return Pre{y[r], sigma[r], b[r], ys[r]}; }
    __device__ __forceinline__ void operator()(int r, int, const V (&acc)[1], const Pre& p) {
        const V y2 = rn_add(p.yv, rn_mul(p.s, rn_sub(p.br, acc[0])));
        y[r] = y2;
        ys[r] = rn_add(p.acc_s, y2);
    }
};

template <class V>
SPS_PASS_KERNEL rf_row_step(Args<V> a) {
    Ctl* ctl = a.ctl;
    if (ctl->done || ctl->iters >= ctl->max_iters) return;
    __shared__ bool last;
    RfRowStepEpi<V> e{a.sigma, a.b, a.Y[0], a.ys};
    visit_bins<1, V>(a.rows, blockIdx.x, a.csr, GatherOne<V>{a.xbar}, e);
    __syncthreads();
    if (threadIdx.x == 0) {
        last = ticket_release(&ctl->ticket[T_ROW_STEP]) == gridDim.x - 1;
        if (last) {
            ctl->ticket[T_ROW_STEP] = 0;
            ctl->iters += 1;
            ctl->window += 1;
        }
    }
}

// Gather of the point being checked: the average x_sum / window (reference
// division), or the current iterate.
template <class V>
struct RfGather {
    const V* v;
    V win;
    bool avg;
    __device__ __forceinline__ double operator()(int, int j) const {
        return avg ? double(rn_div(__ldg(v + j), win)) : double(__ldg(v + j));
    }
};

template <class V>
struct RfRowCheckEpi {
    const V *b, *yv;
    V win;
    bool avg;
    double p[2] = {0, 0};     // ||A x - b||^2, b^T y
    using Pre = NoPre;
    static constexpr int NP = 2;
    using R = double;
    __device__ __forceinline__ void zero() { p[0] = p[1] = 0.0; }
    __device__ __forceinline__ void export_to(double* d) const { d[0] = p[0]; d[1] = p[1]; }
    __device__ __forceinline__ Pre pre(int) const { return Pre{}; }
    __device__ __forceinline__ void operator()(int r, int, const double (&acc)[1], const Pre&) {
        const double res = acc[0] - double(b[r]);
        p[0] += res * res;
        const double y = avg ? double(rn_div(yv[r], win)) : double(yv[r]);
        p[1] += double(b[r]) * y;
    }
};

// mode: 0 = scheduled check of the average (only when window % interval == 0),
//       1 = evaluate the current iterate (start-up error / final report).
template <class V>
SPS_CHECK_KERNEL rf_row_check(Args<V> a, int mode) {
    Ctl* ctl = a.ctl;
    if (mode == 0 && (ctl->done || ctl->window == 0 || ctl->window % a.check_interval != 0)) return;
    __shared__ double sm[kWarps * 2];
    const bool avg = mode == 0;
    const V win = V(ctl->window);
    RfGather<V> g{avg ? a.xs : a.X[0], win, avg};
    RfRowCheckEpi<V> e{a.b, avg ? a.ys : a.Y[0], win, avg};
    visit_bins<1, double>(a.rows_chk, blockIdx.x, a.csr, g, e);
    block_sum<2>(e.p, sm);
    if (threadIdx.x == 0) {
        a.part_row[(size_t)blockIdx.x * 2 + 0] = e.p[0];
        a.part_row[(size_t)blockIdx.x * 2 + 1] = e.p[1];
    }
}

template <class V>
struct RfColCheckEpi {
    const V *c, *xv;
    V win;
    bool avg;
    double p[2] = {0, 0};     // ||min(c - A^T y, 0)||^2, c^T x
    using Pre = NoPre;
    static constexpr int NP = 2;
    using R = double;
    __device__ __forceinline__ void zero() { p[0] = p[1] = 0.0; }
    __device__ __forceinline__ void export_to(double* d) const { d[0] = p[0]; d[1] = p[1]; }
    __device__ __forceinline__ Pre pre(int) const { return Pre{}; }
    __device__ __forceinline__ void operator()(int j, int, const double (&acc)[1], const Pre&) {
        const double rc = double(c[j]) - acc[0];
        const double neg = fmin(rc, 0.0);
        p[0] += neg * neg;
        const double x = avg ? double(rn_div(xv[j], win)) : double(xv[j]);
        p[1] += double(c[j]) * x;
    }
};

template <class V>
SPS_CHECK_KERNEL rf_col_check(Args<V> a, int mode) {
    Ctl* ctl = a.ctl;
    if (mode == 0 && (ctl->done || ctl->window == 0 || ctl->window % a.check_interval != 0)) return;
    __shared__ double sm[kWarps * 2];
    __shared__ bool last;
    const bool avg = mode == 0;
    const V win = V(ctl->window);
    RfGather<V> g{avg ? a.ys : a.Y[0], win, avg};
    RfColCheckEpi<V> e{a.c, avg ? a.xs : a.X[0], win, avg};
    visit_bins<1, double>(a.cols_chk, blockIdx.x, a.csc, g, e);
    if (!publish_partials<2>(e.p, a.part_col, &ctl->ticket[T_COL_CHECK], sm, &last)) return;
    double tc[2], tr[2];
    gather_partials<2>(tc, a.part_col, gridDim.x, sm);
    gather_partials<2>(tr, a.part_row, a.rows_chk.total_blocks, sm);
    add_segment_rows<2>(tc, a.csc, sm);
    add_segment_rows<2>(tr, a.csr, sm);
    if (threadIdx.x != 0) return;
    ctl->ticket[T_COL_CHECK] = 0;
    const double rp = sqrt(tr[0]) * a.inv_nb;
    const double rd = sqrt(tc[0]) * a.inv_nc;
    const double po = tc[1], dob = tr[1];
    const double gap = fabs(po - dob) / (1.0 + fabs(po) + fabs(dob));
    double err = fmax(rp, fmax(rd, gap));
    if (isnan(err)) err = INFINITY;
    ctl->rel_p = rp; ctl->rel_d = rd; ctl->rel_gap = gap; ctl->pobj = po; ctl->dobj = dob;
    ctl->rel_kkt = err;
    if (mode == 1) {
        if (ctl->init_phase) { ctl->kkt_last = err; ctl->init_phase = 0; }
        return;
    }
    ctl->last_avg_kkt = err;
    int apply = 0;
    if (err < ctl->tol) {
        ctl->done = 1;
        ctl->status = SPS_STATUS_OPTIMAL;
        ctl->choice = 1;
        apply = AP_LOAD_AVG;
    } else if (err < 0.5 * ctl->kkt_last) {
        ctl->kkt_last = err;
        ctl->restarts += 1;
        apply = AP_LOAD_AVG | AP_RESTART;
    } else if (!isfinite(err)) {
        ctl->done = 1;
        ctl->status = SPS_STATUS_NUMERIC_ERROR;
    } else if (stop_requested(ctl, a.abort_flag)) {
        ctl->done = 1;
        ctl->status = SPS_STATUS_TIME_LIMIT;
    }
    ctl->apply = apply;
}

template <class V>
__global__ void __launch_bounds__(kBlock) rf_apply(Args<V> a) {
    Ctl* ctl = a.ctl;
    const int ap = ctl->apply;
    __shared__ bool last;
    if (ap & AP_LOAD_AVG) {
        const V win = V(ctl->window);
        const bool rst = ap & AP_RESTART;
        const int stride = gridDim.x * kBlock;
        for (int j = blockIdx.x * kBlock + threadIdx.x; j < a.n; j += stride) {
            a.X[0][j] = rn_div(a.xs[j], win);
            if (rst) a.xs[j] = V(0);
        }
        for (int i = blockIdx.x * kBlock + threadIdx.x; i < a.m; i += stride) {
            a.Y[0][i] = rn_div(a.ys[i], win);
            if (rst) a.ys[i] = V(0);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            last = ticket_release(&ctl->ticket[T_APPLY]) == gridDim.x - 1;
            if (last) {
                ctl->ticket[T_APPLY] = 0;
                if (rst) ctl->window = 0;
                ctl->apply = 0;
                set_loop_condition(a, ctl);
            }
        }
        return;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) set_loop_condition(a, ctl);
}

}  // namespace sps
