// api.cu — extern "C" entry points of libsps_gb300.so (declared in
// include/sps_pdhg.h): input validation, the reference standard-form
// conversion for SPS_MODE_REFERENCE, and handle management.
#include <algorithm>
#include <cmath>
#include <chrono>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "engine_impl.cuh"
#include "nvtx.cuh"

using namespace sps;

// A caller problem copied into owned storage (the descriptor's arrays are only
// valid during sps_create); kept when a stalled FP32 solve may continue in FP64.
// The caller's problem kept for an FP64 continuation (the caller's buffers are
// not retained): its constraint arrays and right-hand sides; c, lb and ub
// point at the engine's own copies.
struct ProblemCopy {
    sps_problem_desc d{};
    std::vector<int32_t> ubp, ubi, eqp, eqi;
    std::vector<double> ubv, eqv, bub, beq;
};

struct sps_handle {
    EngineBase* eng = nullptr;
    sps_options opt{};
    std::unique_ptr<ProblemCopy> copy;   // set when escalation is possible
    sps_handle* esc = nullptr;           // FP64 continuation, created at the first stall
    bool last_esc = false;               // the last solve finished in esc
};

namespace {

thread_local std::string g_create_error;

int create_fail(int code, const std::string& msg) {
    g_create_error = msg;
    return code;
}

bool check_csr(const int32_t* ptr, const int32_t* idx, const double* val, int32_t rows, std::string& why,
               const char* name) {
    if (rows == 0) return true;
    if (!ptr) { why = std::string(name) + ": null indptr"; return false; }
    if (ptr[0] != 0) { why = std::string(name) + ": indptr[0] != 0"; return false; }
    for (int32_t i = 0; i < rows; ++i)
        if (ptr[i + 1] < ptr[i]) { why = std::string(name) + ": indptr not monotone"; return false; }
    if (ptr[rows] > 0 && (!idx || !val)) { why = std::string(name) + ": null indices/values"; return false; }
    return true;
}

// Index of the first item in [0, len) that bad() flags, or len: on host threads
// (the set-up's pool) over contiguous chunks when len is large.
template <class F>
int64_t first_bad(int64_t len, F bad) {
    const int64_t hw = std::max<int64_t>(1, std::min<int64_t>(sps::HostPool::kMaxThreads, std::thread::hardware_concurrency()));
    const int nt = (int)std::max<int64_t>(1, std::min<int64_t>(hw, len >> 17));
    std::vector<int64_t> first(nt, len);
    sps::HostPool::run(nt, [&](int t) {
        const int64_t lo = len * t / nt, hi = len * (t + 1) / nt;
        for (int64_t i = lo; i < hi; ++i)
            if (bad(i)) { first[t] = i; return; }
    });
    return *std::min_element(first.begin(), first.end());
}

bool finite_all(const double* v, int64_t len) {
    return first_bad(len, [&](int64_t i) { return !std::isfinite(v[i]); }) == len;
}

// Validation shared by both modes (solver/problem.py:103-142 plus the engine's
// own requirements: finite c and rhs, no lb = +inf / ub = -inf).
int validate(const sps_problem_desc* d) {
    if (!d) return create_fail(SPS_ERR_INVALID, "null problem descriptor");
    if (d->n < 0 || d->m_ub < 0 || d->m_eq < 0) return create_fail(SPS_ERR_INVALID, "negative dimension");
    std::string why;
    if (!check_csr(d->ub_indptr, d->ub_indices, d->ub_values, d->m_ub, why, "A_ub") ||
        !check_csr(d->eq_indptr, d->eq_indices, d->eq_values, d->m_eq, why, "A_eq"))
        return create_fail(SPS_ERR_INVALID, why);
    if ((int64_t)(d->m_ub ? d->ub_indptr[d->m_ub] : 0) + (d->m_eq ? d->eq_indptr[d->m_eq] : 0) > INT32_MAX)
        return create_fail(SPS_ERR_INVALID, "more than 2^31-1 nonzeros");
    if (d->n > 0 && (!d->c || !d->lb || !d->ub)) return create_fail(SPS_ERR_INVALID, "null c/lb/ub");
    if ((d->m_ub && !d->b_ub) || (d->m_eq && !d->b_eq)) return create_fail(SPS_ERR_INVALID, "null rhs");
    if (!finite_all(d->c, d->n)) return create_fail(SPS_ERR_INVALID, "non-finite objective coefficient");
    if (!finite_all(d->b_ub, d->m_ub) || !finite_all(d->b_eq, d->m_eq))
        return create_fail(SPS_ERR_INVALID, "non-finite right-hand side");
    const int64_t bad = first_bad(d->n, [&](int64_t j) {
        const double l = d->lb[j], u = d->ub[j];
        return std::isnan(l) || std::isnan(u) || l == INFINITY || u == -INFINITY || l > u + 1e-12;
    });
    if (bad < d->n) return create_fail(SPS_ERR_INVALID, "invalid bounds at variable " + std::to_string(bad));
    return SPS_OK;
}

// Box form as given: K = [A_ub; A_eq], rows of A_ub are '<='.
void build_box(const sps_problem_desc* d, HostProblem& hp) {
    const int32_t mu = d->m_ub, me = d->m_eq;
    const int32_t nub = mu ? d->ub_indptr[mu] : 0, neq = me ? d->eq_indptr[me] : 0;
    hp.n = d->n;
    hp.m = mu + me;
    hp.ptr.resize(hp.m + 1);
    hp.ptr[0] = 0;
    for (int32_t i = 0; i < mu; ++i) hp.ptr[i + 1] = d->ub_indptr[i + 1];
    for (int32_t i = 0; i < me; ++i) hp.ptr[mu + i + 1] = nub + d->eq_indptr[i + 1];
    hp.segs = {{d->ub_indices, d->ub_values, nub}, {d->eq_indices, d->eq_values, neq}};
    hp.kind.assign(hp.m, 0);
    for (int32_t i = 0; i < mu; ++i) hp.kind[i] = 1;
    hp.c = d->c;
    hp.lb = d->lb;
    hp.ub = d->ub;
    hp.rhs.resize(hp.m);
    for (int32_t i = 0; i < mu; ++i) hp.rhs[i] = d->b_ub[i];
    for (int32_t i = 0; i < me; ++i) hp.rhs[mu + i] = d->b_eq[i];
}

// Reference standard form (solver/lp/pdhg.py:62-125): shift by finite lb,
// one '<=' row per finite ub (column order), a slack per '<=' row, rows with
// rhs < -1e-6 negated; every row '=', every column in [0, inf).
void build_standard(const sps_problem_desc* d, HostProblem& hp, StdMap& s) {
    const int32_t n = d->n, mu = d->m_ub, me = d->m_eq;
    s.n_orig = n;
    s.m_ub = mu;
    s.m_eq = me;
    s.lb_shift.resize(n);
    for (int32_t j = 0; j < n; ++j) s.lb_shift[j] = std::isfinite(d->lb[j]) ? d->lb[j] : 0.0;
    s.ub_cols.clear();
    for (int32_t j = 0; j < n; ++j)
        if (std::isfinite(d->ub[j])) s.ub_cols.push_back(j);
    s.nub = (int32_t)s.ub_cols.size();
    const int32_t m_le = mu + s.nub, m = m_le + me, ns = n + m_le;
    const int64_t nz_ub = mu ? d->ub_indptr[mu] : 0, nz_eq = me ? d->eq_indptr[me] : 0;
    const int64_t nz = nz_ub + nz_eq + 2LL * s.nub + mu;
    hp.own_idx.resize(nz);
    hp.own_val.resize(nz);
    hp.ptr.assign(m + 1, 0);
    hp.rhs.assign(m, 0.0);
    int64_t k = 0;
    auto row_dot_shift = [&](const int32_t* ip, const int32_t* ix, const double* vv, int32_t i) {
        double acc = 0.0;
        for (int32_t q = ip[i]; q < ip[i + 1]; ++q) acc += vv[q] * s.lb_shift[ix[q]];
        return acc;
    };
    for (int32_t i = 0; i < mu; ++i) {
        for (int32_t q = d->ub_indptr[i]; q < d->ub_indptr[i + 1]; ++q) {
            hp.own_idx[k] = d->ub_indices[q];
            hp.own_val[k++] = d->ub_values[q];
        }
        hp.own_idx[k] = n + i;
        hp.own_val[k++] = 1.0;
        hp.ptr[i + 1] = (int32_t)k;
        hp.rhs[i] = d->b_ub[i] - row_dot_shift(d->ub_indptr, d->ub_indices, d->ub_values, i);
    }
    for (int32_t t = 0; t < s.nub; ++t) {
        const int32_t j = s.ub_cols[t];
        hp.own_idx[k] = j;
        hp.own_val[k++] = 1.0;
        hp.own_idx[k] = n + mu + t;
        hp.own_val[k++] = 1.0;
        hp.ptr[mu + t + 1] = (int32_t)k;
        hp.rhs[mu + t] = d->ub[j] - s.lb_shift[j];
    }
    for (int32_t i = 0; i < me; ++i) {
        for (int32_t q = d->eq_indptr[i]; q < d->eq_indptr[i + 1]; ++q) {
            hp.own_idx[k] = d->eq_indices[q];
            hp.own_val[k++] = d->eq_values[q];
        }
        hp.ptr[m_le + i + 1] = (int32_t)k;
        hp.rhs[m_le + i] = d->b_eq[i] - row_dot_shift(d->eq_indptr, d->eq_indices, d->eq_values, i);
    }
    s.neg.assign(m, 0);
    for (int32_t i = 0; i < m; ++i) {
        if (hp.rhs[i] < -1e-6) {
            s.neg[i] = 1;
            hp.rhs[i] = -hp.rhs[i];
            for (int32_t q = hp.ptr[i]; q < hp.ptr[i + 1]; ++q) hp.own_val[q] = -hp.own_val[q];
        }
    }
    hp.n = ns;
    hp.m = m;
    hp.segs = {{hp.own_idx.data(), hp.own_val.data(), k}};
    hp.kind.assign(m, 0);
    hp.own_c.assign(ns, 0.0);
    for (int32_t j = 0; j < n; ++j) hp.own_c[j] = d->c[j];
    hp.own_lb.assign(ns, 0.0);
    hp.own_ub.assign(ns, INFINITY);
    hp.c = hp.own_c.data();
    hp.lb = hp.own_lb.data();
    hp.ub = hp.own_ub.data();
}

std::unique_ptr<ProblemCopy> copy_problem(const sps_problem_desc* d, const EngineBase* e) {
    auto p = std::make_unique<ProblemCopy>();
    const int64_t nub = d->m_ub ? d->ub_indptr[d->m_ub] : 0, neq = d->m_eq ? d->eq_indptr[d->m_eq] : 0;
    auto take = [](auto& v, const auto* src, int64_t len) {
        if (src && len > 0) v.assign(src, src + len);
        return v.empty() ? nullptr : v.data();
    };
    p->d = *d;
    // the nonzero arrays (tens of MB on large LPs) on their own threads
    std::thread t1([&] { p->d.ub_indices = take(p->ubi, d->ub_indices, nub); });
    std::thread t2([&] { p->d.ub_values = take(p->ubv, d->ub_values, nub); });
    std::thread t3([&] { p->d.eq_indices = take(p->eqi, d->eq_indices, neq); });
    p->d.eq_values = take(p->eqv, d->eq_values, neq);
    p->d.ub_indptr = take(p->ubp, d->ub_indptr, d->m_ub ? d->m_ub + 1 : 0);
    p->d.eq_indptr = take(p->eqp, d->eq_indptr, d->m_eq ? d->m_eq + 1 : 0);
    p->d.b_ub = take(p->bub, d->b_ub, d->m_ub);
    p->d.b_eq = take(p->beq, d->b_eq, d->m_eq);
    p->d.c = e->c_user.empty() ? nullptr : e->c_user.data();
    p->d.lb = e->lb_user.empty() ? nullptr : e->lb_user.data();
    p->d.ub = e->ub_user.empty() ? nullptr : e->ub_user.data();
    t1.join();
    t2.join();
    t3.join();
    return p;
}

// A stalled FP32 solve continues in FP64 from the best point it saw, with the
// primal weight it had there, within the iteration and time limits left.
int escalate(sps_handle* h, sps_result* res) {
    const auto t0 = std::chrono::steady_clock::now();
    EngineBase* e = h->eng;
    if (!h->esc) {
        sps_options o = h->opt;
        o.precision = SPS_FP64;
        o.escalate = 0;
        const int rc = sps_create(&h->copy->d, &o, &h->esc);
        if (rc != SPS_OK) return e->fail(rc, "FP64 continuation: " + g_create_error);
    }
    std::vector<double> x(std::max(e->n_user, 1)), y(std::max(e->m_user, 1));
    double omega = 0.0;
    if (int rc = e->get_best(x.data(), y.data(), &omega)) return rc;
    EngineBase* f = h->esc->eng;
    if (int rc = f->warm(x.data(), y.data(), omega)) return e->fail(rc, "FP64 continuation: " + f->err);
    double tl = 0.0;
    if (h->opt.time_limit_s > 0) {
        const double used = res->solve_ms * 1e-3 +
                            std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        tl = h->opt.time_limit_s - used;
        if (tl <= 0) {
            res->status = SPS_STATUS_TIME_LIMIT;
            return SPS_OK;
        }
    }
    f->set_limits(std::max<int64_t>(h->opt.max_iters - res->iterations, 1), tl);
    sps_result r2;
    f->err.clear();
    if (int rc = f->solve(&r2)) return e->fail(rc, "FP64 continuation: " + f->err);
    r2.iterations += res->iterations;
    r2.accepted_steps += res->accepted_steps;
    r2.restarts += res->restarts;
    r2.kernel_launches += res->kernel_launches;
    r2.setup_ms = res->setup_ms;
    r2.solve_ms = res->solve_ms + 1e3 * std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    r2.escalated = 1;
    *res = r2;
    h->last_esc = true;
    return SPS_OK;
}

}  // namespace

namespace sps {
// Message returned by sps_last_error(NULL) for calls without a handle.
void set_create_error(const std::string& msg) { g_create_error = msg; }
}  // namespace sps

extern "C" {

int sps_options_init(sps_options* o) {
    if (!o) return SPS_ERR_INVALID;
    std::memset(o, 0, sizeof(*o));
    o->mode = SPS_MODE_ADAPTIVE;
    o->precision = SPS_FP32;
    o->max_iters = 100000;
    o->tol = 1e-6;
    o->check_interval = 0;
    o->ruiz_iters = 10;
    o->time_limit_s = 0.0;
    o->graph_mode = 2;
    o->device = 0;
    o->max_blocks = 0;
    o->escalate = 1;
    o->warm_fallback = 1;
    return SPS_OK;
}

int sps_create(const sps_problem_desc* prob, const sps_options* opt_in, sps_handle** out) {
    sps::NvtxRange nvtx_range("sps_create");
    g_create_error.clear();
    if (!out) return create_fail(SPS_ERR_INVALID, "null output handle pointer");
    *out = nullptr;
    sps_options opt;
    if (opt_in) opt = *opt_in; else sps_options_init(&opt);
    if (opt.mode != SPS_MODE_REFERENCE && opt.mode != SPS_MODE_ADAPTIVE)
        return create_fail(SPS_ERR_INVALID, "unknown mode");
    if (opt.precision != SPS_FP32 && opt.precision != SPS_FP64)
        return create_fail(SPS_ERR_INVALID, "unknown precision");
    if (opt.max_iters < 0 || !(opt.tol >= 0) || opt.check_interval < 0 || opt.time_limit_s < 0)
        return create_fail(SPS_ERR_INVALID, "invalid options");
    if (opt.kkt_form != SPS_KKT_LAGRANGIAN && opt.kkt_form != SPS_KKT_PDLP)
        return create_fail(SPS_ERR_INVALID, "unknown kkt_form");
    if (opt.kkt_form == SPS_KKT_PDLP && opt.mode != SPS_MODE_ADAPTIVE)
        return create_fail(SPS_ERR_INVALID, "kkt_form PDLP needs the adaptive mode (the reference mode "
                                            "reports the reference's own error)");
    const CreateTrace trace;
    if (int rc = validate(prob)) return rc;
    trace.mark("host validation");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= opt.device || opt.device < 0) {
        cudaGetLastError();
        return create_fail(SPS_ERR_CUDA, "no usable CUDA device");
    }
    HostProblem hp;
    StdMap sm;
    if (opt.mode == SPS_MODE_REFERENCE) build_standard(prob, hp, sm);
    else build_box(prob, hp);

    sps_handle* h = new sps_handle();
    h->opt = opt;
    h->eng = opt.precision == SPS_FP32 ? make_engine_f32() : make_engine_f64();
    EngineBase* e = h->eng;
    e->n_user = prob->n;
    e->m_user = prob->m_ub + prob->m_eq;
    e->smap = sm;
    e->trace = &trace;
    // the host copies the engine keeps (c and bounds for extraction, the whole problem
    // when a stalled FP32 solve may continue in FP64) on a thread of their own, while
    // the device set-up runs; set-up reads only the caller's arrays and hp
    std::thread copies([&] {
        e->c_user.assign(prob->c, prob->c + prob->n);
        e->lb_user.assign(prob->lb, prob->lb + prob->n);
        e->ub_user.assign(prob->ub, prob->ub + prob->n);
        if (opt.mode == SPS_MODE_ADAPTIVE && opt.precision == SPS_FP32 && opt.escalate == 1)
            h->copy = copy_problem(prob, e);
    });
    const int rc = opt.precision == SPS_FP32 ? setup_f32(e, hp, opt, opt.mode) : setup_f64(e, hp, opt, opt.mode);
    copies.join();
    trace.mark("host copies joined");
    e->trace = nullptr;
    if (rc != SPS_OK) {
        g_create_error = e->err;
        delete e;
        delete h;
        return rc;
    }
    *out = h;
    return SPS_OK;
}

int sps_set_warm_start(sps_handle* h, const double* x0, const double* y0, double omega0) {
    if (!h) return SPS_ERR_INVALID;
    return h->eng->warm(x0, y0, omega0);
}

int sps_solve(sps_handle* h, sps_result* res) {
    sps::NvtxRange nvtx_range("sps_solve");
    if (!h || !res) return SPS_ERR_INVALID;
    h->eng->err.clear();
    h->last_esc = false;
    const int rc = h->eng->solve(res);
    if (rc != SPS_OK || res->status != SPS_STATUS_STALLED || !h->copy) return rc;
    return escalate(h, res);
}

int sps_time_iteration_kernels(sps_handle* h, int32_t reps, double* out) {
    if (!h || !out) return SPS_ERR_INVALID;
    return h->eng->time_kernels(reps, out, false);
}

int sps_time_iteration_kernels_graph(sps_handle* h, int32_t reps, double* out) {
    if (!h || !out) return SPS_ERR_INVALID;
    return h->eng->time_kernels(reps, out, true);
}

int sps_get_solution(sps_handle* h, double* x, double* y) {
    sps::NvtxRange nvtx_range("sps_get_solution");
    if (!h) return SPS_ERR_INVALID;
    if (h->last_esc) {
        const int rc = h->esc->eng->get(x, y);
        if (rc) h->eng->err = h->esc->eng->err;
        return rc;
    }
    return h->eng->get(x, y);
}

const char* sps_last_error(const sps_handle* h) {
    return h ? h->eng->err.c_str() : g_create_error.c_str();
}

void sps_destroy(sps_handle* h) {
    if (!h) return;
    if (h->esc) sps_destroy(h->esc);
    delete h->eng;
    delete h;
}

int sps_pin_host(void* ptr, uint64_t bytes) {
    if (!ptr || !bytes) return SPS_ERR_INVALID;
    if (cudaHostRegister(ptr, bytes, cudaHostRegisterDefault) == cudaSuccess) return SPS_OK;
    cudaGetLastError();   // not sticky: clear it so later calls do not report it
    return SPS_ERR_CUDA;
}

int sps_unpin_host(void* ptr) {
    if (!ptr) return SPS_ERR_INVALID;
    if (cudaHostUnregister(ptr) == cudaSuccess) return SPS_OK;
    cudaGetLastError();
    return SPS_ERR_CUDA;
}

const char* sps_version(void) { return "libsps_gb300 0.1 (sm_103a; FP32/FP64 iterates; reference + adaptive PDHG)"; }

int sps_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

}  // extern "C"
