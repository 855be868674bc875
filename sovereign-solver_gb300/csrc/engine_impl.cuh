// engine_impl.cuh — host side of one solver handle: device layout build,
// solve driver (plain launches, a replayed window graph, or one graph with a
// device-driven while loop), watchdog, and solution extraction.
#pragma once

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "host_pool.cuh"
#include "mem_pool.cuh"
#include "setup.cuh"

namespace sps {

// Problem handed to the device: rows of kind '<=' or '=', box bounds per column.
struct HostProblem {
    int32_t n = 0, m = 0;
    std::vector<int32_t> ptr;                    // m + 1
    struct Seg { const int32_t* idx; const double* val; int64_t cnt; };
    std::vector<Seg> segs;                       // nonzeros, concatenated in row order
    std::vector<int8_t> kind;                    // m: 1 = '<=' row
    const double *c = nullptr, *lb = nullptr, *ub = nullptr;
    std::vector<double> rhs;                     // m
    std::vector<int32_t> own_idx;                // storage of a built standard form
    std::vector<double> own_val, own_c, own_lb, own_ub;
};

// Map between the caller's problem and the reference standard form.
struct StdMap {
    int32_t n_orig = 0, m_ub = 0, m_eq = 0, nub = 0;
    std::vector<int32_t> ub_cols;
    std::vector<int8_t> neg;
    std::vector<double> lb_shift;
};

// Phase times of sps_create on stderr when the environment sets
// SPS_TRACE_CREATE (a diagnostic: which part of set-up a large LP waits on).
struct CreateTrace {
    bool on = std::getenv("SPS_TRACE_CREATE") != nullptr;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    void mark(const char* what) const {
        if (!on) return;
        const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        std::fprintf(stderr, "sps_create %-26s %9.2f ms\n", what, ms);
    }
};

struct EngineBase {
    const CreateTrace* trace = nullptr;   // set during sps_create
    // caller problem (for extraction)
    int32_t n_user = 0, m_user = 0;
    std::vector<double> c_user, lb_user, ub_user;
    StdMap smap;
    virtual ~EngineBase() {}
    virtual int solve(sps_result* res) = 0;
    virtual int warm(const double* x0, const double* y0, double omega0) = 0;
    virtual int get(double* x, double* y) = 0;
    // graph: capture the launches and events into one CUDA graph and replay it
    // (the kernels run back to back from the device, as in the solve's graph)
    virtual int time_kernels(int reps, double* out, bool graph) = 0;
    // Best point of the last solve's stall test in the caller's space, and the
    // primal weight it was taken with (the returned point when none was saved).
    virtual int get_best(double* x, double* y, double* omega) = 0;
    virtual void set_limits(int64_t max_iters, double time_limit_s) = 0;
    std::string err;
    int fail(int code, const std::string& msg) { err = msg; return code; }
};

#define SPS_CK(call)                                                                        \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess)                                                              \
            return fail(e_ == cudaErrorMemoryAllocation ? SPS_ERR_OOM : SPS_ERR_CUDA,       \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                \
    } while (0)

constexpr int kSms = 152;

template <class V>
struct Engine : EngineBase {
    sps_options opt{};
    int mode = SPS_MODE_ADAPTIVE;
    int32_t n = 0, m = 0;
    int64_t nnz = 0;
    bool trivial = false;

    cudaStream_t st = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, evq = nullptr;
    char* arena = nullptr;
    Ctl* d_ctl = nullptr;
    Ctl* h_ctl = nullptr;               // pinned read-back
    int32_t* h_abort = nullptr;         // mapped host flag
    int32_t* d_abort = nullptr;
    int32_t *d_perm_row = nullptr, *d_perm_col = nullptr;
    int8_t* d_rkind = nullptr;
    double *d_xout = nullptr, *d_yout = nullptr, *d_wx = nullptr, *d_wy = nullptr;
    // adaptive mode: the caller's c (and bounds unless uniform) in FP64, caller order, for the
    // solution extracted on the device; the solution then stays there until sps_get_solution
    double *d_cuser = nullptr, *d_lbuser = nullptr, *d_ubuser = nullptr, *d_obj = nullptr;
    bool sol_on_device = false;
    bool have_warm_x = false, have_warm_y = false;
    double warm_omega = 0.0;
    bool warm_used = false;
    double cold_rel = -1.0;      // relative KKT error of the cold start point (cached)
    double eta0 = 1.0, omega0 = 1.0;
    Args<V> args{};
    cudaMemPool_t pool = nullptr;       // device memory (engine_pool; null: the default pool)
    cudaGraphExec_t win_exec = nullptr, loop_exec = nullptr;
    int64_t launches = 0;
    double setup_ms = 0.0;
    std::vector<double> x_sol, y_sol;
    bool solved = false;
    BinTable layout_rows{}, layout_cols{};
    int64_t padded_nnz_rows = 0, padded_nnz_cols = 0;

    ~Engine() override {
        if (win_exec) cudaGraphExecDestroy(win_exec);
        if (loop_exec) cudaGraphExecDestroy(loop_exec);
        if (arena) cudaFreeAsync(arena, st);
        if (st) cudaStreamSynchronize(st);
        if (h_ctl) cudaFreeHost(h_ctl);
        if (h_abort) cudaFreeHost(h_abort);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (evq) cudaEventDestroy(evq);
        if (st) cudaStreamDestroy(st);
    }

    // stream-ordered allocation on the engine's stream, from the engine's pool
    template <class T>
    cudaError_t dalloc(T** p, size_t bytes) {
        return pool ? cudaMallocFromPoolAsync(reinterpret_cast<void**>(p), bytes, pool, st)
                    : cudaMallocAsync(reinterpret_cast<void**>(p), bytes, st);
    }

    static int grid_for(int64_t work, int per_block = kBlock, int cap = kSms * 16) {
        int64_t g = (work + per_block - 1) / per_block;
        return (int)std::max<int64_t>(1, std::min<int64_t>(g, cap));
    }

    // Host plan of one orientation's layout (rows of the CSR or columns of the CSC).
    struct Plan {
        std::vector<int32_t> perm;      // internal -> original
        BinTable bt{};
        std::vector<int32_t> fptr;      // final CSR offsets (R + 1); SLICED rows hold their bin's start
        std::vector<int32_t> soff;      // slice offsets, one sentinel after each SLICED bin
        std::vector<int32_t> unit;      // SEGMENT / SLAB unit descriptors, 8 ints each (Layout::unit)
        int32_t units() const { return (int32_t)(unit.size() / 8); }
        int64_t total = 0;              // final index/value array length (with slice padding)
        int32_t ntickets = 0;           // SEGMENT rows and SLAB slices
        int32_t nslots = 0;             // epilogue partial slots: SEGMENT rows, SLAB slices
        int32_t nslab_units = 0;
        std::vector<int64_t> bin_store; // stored entries per bin (the block shares' work measure)
    };

    // Blocks that give every warp of the bin work for its first step (warps
    // take two units per step, one in SLAB bins).
    static int64_t blocks_needed(const Bin& b) {
        const int per = b.mode == BM_SLAB ? kWarps : 2 * kWarps;
        return (b.units + per - 1) / per;
    }

    static int mode_of(int64_t len, bool slab) {
        return len <= kSliceMax ? BM_SLICED : slab ? BM_SLAB : (len <= kSegment ? BM_WARP : BM_SEGMENT);
    }

    // SLAB choice per group of 32 consecutive long rows of one kind (original
    // order), from the 32-byte sectors of the gathered vector that a warp
    // touches, sampled at up to 32 steps of the group: CSR (a warp reads 32
    // consecutive nonzeros of one row: a new sector where the column leaves the
    // previous one's) against SLAB (a warp reads the k-th nonzero of the 32 rows:
    // the distinct sectors in lane order), plus SLAB's padded entries (index and
    // value reads).  SLAB when it needs at most half of CSR's sectors.  Columns
    // in internal numbering (inv_col).
    static std::vector<uint8_t> choose_slab(const HostProblem& hp, const std::vector<int32_t>& inv_col,
                                            int elem_bytes) {
        const int m = hp.m;
        std::vector<uint8_t> slab(m, 0);
        std::vector<int64_t> seg_end;
        int64_t acc = 0;
        for (const auto& sg : hp.segs) { acc += sg.cnt; seg_end.push_back(acc); }
        auto col = [&](int64_t k) -> int32_t {
            size_t q = 0;
            while (q + 1 < seg_end.size() && k >= seg_end[q]) ++q;
            const int64_t base = q ? seg_end[q - 1] : 0;
            return inv_col[hp.segs[q].idx[k - base]];
        };
        const int sh = elem_bytes == 4 ? 3 : 2;        // log2(elements per 32-byte sector)
        for (int kd = 0; kd < 2; ++kd) {
            std::vector<int32_t> rows;
            for (int i = 0; i < m; ++i)
                if (hp.kind[i] == kd && hp.ptr[i + 1] - hp.ptr[i] > kSliceMax) rows.push_back(i);
            // groups of 32 rows are scored independently: on the host pool, a range
            // of groups per thread (each group's rows are marked by its own thread)
            const int64_t ngroups = ((int64_t)rows.size() + 31) / 32;
            const int nt = (int)std::max<int64_t>(1, std::min<int64_t>(HostPool::kMaxThreads, ngroups / 8));
            HostPool::run(nt, [&](int th) {
            for (size_t g = 32 * (size_t)(ngroups * th / nt); g < 32 * (size_t)(ngroups * (th + 1) / nt) && g < rows.size(); g += 32) {
                const int cnt = (int)std::min<size_t>(32, rows.size() - g);
                int64_t lmin = INT64_MAX, lmax = 0, stored = 0;
                for (int t = 0; t < cnt; ++t) {
                    const int64_t len = hp.ptr[rows[g + t] + 1] - hp.ptr[rows[g + t]];
                    lmin = std::min(lmin, len);
                    lmax = std::max(lmax, len);
                    stored += len;
                }
                const int ns = (int)std::min<int64_t>(32, lmin - 1);
                double csr = 0.0, sl = 0.0;
                for (int q = 0; q < ns; ++q) {
                    const int64_t k = 1 + (lmin - 1) * q / ns;
                    int32_t prev = -1;
                    for (int t = 0; t < cnt; ++t) {
                        const int64_t base = hp.ptr[rows[g + t]];
                        const int32_t a = col(base + k) >> sh, a0 = col(base + k - 1) >> sh;
                        csr += a != a0;
                        sl += a != prev;
                        prev = a;
                    }
                }
                const double per = 1.0 / (double(ns) * cnt);
                const double csr_cost = csr * per * double(stored);
                const double slab_cost = sl * per * double(stored) +
                                         double(32 * lmax - stored) * (4.0 + elem_bytes) / 32.0;
                if (slab_cost <= 0.5 * csr_cost)
                    for (int t = 0; t < cnt; ++t) slab[rows[g + t]] = 1;
            }
            });
        }
        return slab;
    }

    // Columns longer than the device insertion sort takes (kSortMax), ordered
    // by row index on the host: idx / val hold the CSC entries of columns
    // [j0, j1) (cptr[j0] .. cptr[j1]); shorter columns in the range are left as
    // they are.  Columns are independent, so host threads take column ranges.
    static void sort_long_columns(const int32_t* cptr, int32_t j0, int32_t j1, int32_t* idx, double* val) {
        const int64_t base = cptr[j0];
        auto work = [&](int32_t a, int32_t b) {
            std::vector<int64_t> ord;
            std::vector<int32_t> ri2;
            std::vector<double> rv2;
            for (int32_t j = a; j < b; ++j) {
                const int64_t s = cptr[j] - base, len = (int64_t)cptr[j + 1] - cptr[j];
                if (len <= kSortMax) continue;
                int32_t* ri = idx + s;
                double* rv = val + s;
                ord.resize(len);
                std::iota(ord.begin(), ord.end(), 0);
                std::sort(ord.begin(), ord.end(), [&](int64_t x, int64_t y) { return ri[x] < ri[y]; });
                ri2.resize(len);
                rv2.resize(len);
                for (int64_t q = 0; q < len; ++q) { ri2[q] = ri[ord[q]]; rv2[q] = rv[ord[q]]; }
                std::copy(ri2.begin(), ri2.end(), ri);
                std::copy(rv2.begin(), rv2.end(), rv);
            }
        };
        const int64_t cols = (int64_t)j1 - j0;
        const int nt = (int)std::min<int64_t>(std::max(1u, std::min(16u, std::thread::hardware_concurrency())),
                                              std::max<int64_t>(1, cols / 4096));
        HostPool::run(nt, [&](int t) { work((int32_t)(j0 + cols * t / nt), (int32_t)(j0 + cols * (t + 1) / nt)); });
    }

    // Blocks of one launch over the bins: one resident wave (block_cap) shared by
    // the bins in proportion to their work (stored entries plus a per-unit
    // overhead of one 32-entry step), never more than one warp per unit.  The
    // pass kernels and the check kernels (fewer resident blocks: more registers)
    // each get their own shares of the same layout.
    static void share_blocks(BinTable& bt, const std::vector<int64_t>& bin_store, int block_cap) {
        int64_t need_total = 0;
        double work_total = 0.0;
        std::vector<double> work(bt.nbins);
        for (int i = 0; i < bt.nbins; ++i) {
            const Bin& b = bt.bin[i];
            need_total += blocks_needed(b);
            work[i] = double(bin_store[i]) + 32.0 * b.units;
            work_total += work[i];
        }
        // When every bin's need fits the wave, every bin gets it (one step per
        // warp); a proportional share here left a few warps two units in a row
        // and the pass waited for them.
        // Otherwise the shares are rounded down (at least one block, at most the
        // need) and the blocks left go to the largest remainders, so the bins
        // add up to the wave: rounding every share up put up to one block per
        // bin past it, and those blocks waited for a free slot.
        const int64_t budget = std::min<int64_t>(block_cap, need_total);
        const int nb = bt.nbins;
        std::vector<int64_t> share(nb), need(nb);
        std::vector<double> raw(nb);
        int64_t sum = 0;
        for (int i = 0; i < nb; ++i) {
            need[i] = blocks_needed(bt.bin[i]);
            raw[i] = budget * work[i] / std::max(work_total, 1.0);
            share[i] = need_total <= block_cap
                           ? need[i]
                           : std::max<int64_t>(1, std::min<int64_t>(need[i], (int64_t)std::floor(raw[i])));
            sum += share[i];
        }
        while (sum < budget) {
            int best = -1;
            for (int i = 0; i < nb; ++i)
                if (share[i] < need[i] && (best < 0 || raw[i] - share[i] > raw[best] - share[best])) best = i;
            if (best < 0) break;
            ++share[best];
            ++sum;
        }
        while (sum > budget) {            // one-block floors of small bins: take from the largest share
            int best = -1;
            for (int i = 0; i < nb; ++i)
                if (share[i] > 1 && (best < 0 || share[i] > share[best])) best = i;
            if (best < 0) break;
            --share[best];
            --sum;
        }
        int blocks = 0;
        for (int i = 0; i < nb; ++i) {
            Bin& b = bt.bin[i];
            b.nblocks = (int)share[i];
            b.block_begin = blocks;
            blocks += b.nblocks;
        }
        bt.total_blocks = blocks;
    }

    // Host threads for a loop over R items (one below 2^17 items), and the loop over
    // nt contiguous chunks, chunk t on one of the pool's threads.
    static int host_threads(int64_t R) {
        const int64_t hw = std::max<int64_t>(1, std::min<int64_t>(HostPool::kMaxThreads, std::thread::hardware_concurrency()));
        return (int)std::max<int64_t>(1, std::min<int64_t>(hw, R >> 17));
    }
    template <class F>
    static void for_chunks(int64_t R, int nt, F f) {
        if (nt <= 1) { f(0, 0, (int)R); return; }
        HostPool::run(nt, [&](int t) { f(t, (int)(R * t / nt), (int)(R * (t + 1) / nt)); });
    }

    // out[0] = 0, out[i + 1] = out[i] + len(i): chunk sums on host threads, then
    // each chunk fills its part from its offset.
    template <class F>
    static void prefix_lengths(int R, F len, std::vector<int32_t>& out) {
        const int nt = host_threads(R);
        std::vector<int64_t> part(nt + 1, 0);
        for_chunks(R, nt, [&](int t, int lo, int hi) {
            int64_t acc = 0;
            for (int i = lo; i < hi; ++i) acc += len(i);
            part[t + 1] = acc;
        });
        for (int t = 0; t < nt; ++t) part[t + 1] += part[t];
        out[0] = 0;
        for_chunks(R, nt, [&](int t, int lo, int hi) {
            int64_t acc = part[t];
            for (int i = lo; i < hi; ++i) { acc += len(i); out[i + 1] = (int32_t)acc; }
        });
    }

    // Order: per kind, SLICED rows by decreasing length, then WARP rows, then
    // SEGMENT rows, then SLAB rows (stable counting sort); one bin per (kind,
    // schedule).
    static void make_plan(const std::vector<int64_t>& lens, const std::vector<int8_t>* kinds,
                          const std::vector<uint8_t>* slab, Plan& P, int block_cap,
                          const CreateTrace* tr = nullptr) {
        const int R = (int)lens.size();
        constexpr int NB = kSliceMax + 4;
        auto kind_of = [&](int i) { return kinds ? (int)(*kinds)[i] : 0; };
        auto mode_at = [&](int i) { return mode_of(lens[i], slab && (*slab)[i]); };
        auto bucket = [&](int i) {
            const int md = mode_at(i);
            const int sub = md == BM_SLICED ? (int)(kSliceMax - lens[i])
                                            : kSliceMax + (md == BM_WARP ? 1 : md == BM_SEGMENT ? 2 : 3);
            return kind_of(i) * NB + sub;
        };
        // each row's bucket once (the sort and the bin boundaries read it again);
        // large plans on host threads over contiguous chunks (a 2M-column plan
        // took 12 ms of a 29 ms sps_create on one thread)
        std::vector<uint8_t> bk(R);
        const int nt = host_threads(R);
        std::vector<std::vector<int64_t>> hist(nt, std::vector<int64_t>(2 * NB, 0));
        for_chunks(R, nt, [&](int t, int lo, int hi) {
            if (!kinds && !slab) {   // columns: one kind, no SLAB (the same buckets, branch-free)
                const int64_t* L = lens.data();
                for (int i = lo; i < hi; ++i)
                    bk[i] = (uint8_t)(L[i] <= kSliceMax ? kSliceMax - L[i] : L[i] <= kSegment ? kSliceMax + 1 : kSliceMax + 2);
            } else {
                for (int i = lo; i < hi; ++i) bk[i] = (uint8_t)bucket(i);
            }
            // bucket counts in four interleaved histograms (consecutive rows mostly
            // share a bucket, and one counter would make every increment wait for
            // the previous one)
            std::vector<int64_t> h(4 * 2 * NB, 0);
            const uint8_t* kb = bk.data();
            int i = lo;
            for (; i + 4 <= hi; i += 4) {
                ++h[kb[i]];
                ++h[2 * NB + kb[i + 1]];
                ++h[4 * NB + kb[i + 2]];
                ++h[6 * NB + kb[i + 3]];
            }
            for (; i < hi; ++i) ++h[kb[i]];
            for (int b = 0; b < 2 * NB; ++b) hist[t][b] = h[b] + h[2 * NB + b] + h[4 * NB + b] + h[6 * NB + b];
        });
        if (tr) tr->mark("    buckets + histograms");
        std::vector<int64_t> cnt(2 * NB + 1, 0);
        for (int t = 0; t < nt; ++t)
            for (int b = 0; b < 2 * NB; ++b) cnt[b + 1] += hist[t][b];
        for (int b = 0; b < 2 * NB; ++b) cnt[b + 1] += cnt[b];
        // stable placement: chunk t starts each bucket after the earlier chunks' rows of
        // it, and writes each run of equal buckets as one block
        P.perm.assign(R, 0);
        {
            std::vector<std::vector<int64_t>> pos(nt, std::vector<int64_t>(cnt.begin(), cnt.end() - 1));
            for (int t = 1; t < nt; ++t)
                for (int b = 0; b < 2 * NB; ++b) pos[t][b] = pos[t - 1][b] + hist[t - 1][b];
            int32_t* pm = P.perm.data();
            for_chunks(R, nt, [&](int t, int lo, int hi) {
                std::vector<int64_t>& ps = pos[t];
                for (int i = lo; i < hi;) {
                    const uint8_t b = bk[i];
                    int j = i + 1;
                    while (j < hi && bk[j] == b) ++j;
                    int32_t* dst = pm + ps[b];
                    for (int q = i; q < j; ++q) dst[q - i] = q;
                    ps[b] += j - i;
                    i = j;
                }
            });
        }
        // (kind, schedule) of a bucket: rows of one bin are consecutive buckets
        auto bin_of = [&](int bucket_id) {
            const int kd = bucket_id / NB, sub = bucket_id % NB;
            return kd * 4 + (sub <= kSliceMax ? (int)BM_SLICED : sub == kSliceMax + 1 ? (int)BM_WARP
                                              : sub == kSliceMax + 2 ? (int)BM_SEGMENT : (int)BM_SLAB);
        };
        if (tr) tr->mark("    stable placement");
        P.fptr.assign(R + 1, 0);
        P.bt = BinTable{};
        int64_t off = 0;
        std::vector<int64_t> bin_store;              // stored entries per bin
        for (int r = 0; r < R;) {
            const int kd = kind_of(P.perm[r]), md = mode_at(P.perm[r]);
            const int key = bin_of(bk[P.perm[r]]);
            // the bin ends at the first row of another (kind, schedule): jump bucket by bucket
            int e = r;
            for (int q = bk[P.perm[r]]; q < 2 * NB && bin_of(q) == key; ++q) e = (int)cnt[q + 1];
            Bin b{};
            b.begin = r;
            b.end = e;
            b.mode = md;
            b.kind = kd;
            const int64_t bin_off0 = off;
            if (md == BM_SLICED) {
                b.aux = (int32_t)P.soff.size();
                // rows sorted by decreasing length: first == last means one length
                if (lens[P.perm[r]] == lens[P.perm[e - 1]] && lens[P.perm[r]] > 0) {
                    b.slice0 = (int32_t)off;
                    b.part0 = (int32_t)lens[P.perm[r]];
                }
                for (int q = r; q < e; ++q) P.fptr[q] = (int32_t)off;
                for (int s = r; s < e; s += 32) {
                    P.soff.push_back((int32_t)off);
                    off += 32 * lens[P.perm[s]];          // the slice's first row is its longest
                }
                b.units = (int32_t)P.soff.size() - b.aux;
                P.soff.push_back((int32_t)off);           // sentinel: end of the bin's last slice
            } else if (md == BM_WARP) {
                for (int q = r; q < e; ++q) { P.fptr[q] = (int32_t)off; off += lens[P.perm[q]]; }
                b.units = e - r;
            } else if (md == BM_SEGMENT) {
                b.aux = P.units();
                b.aux2 = P.ntickets;
                b.slot0 = P.nslots;
                b.part0 = e - r <= kSegLoadAcquireRows ? 1 : 0;
                for (int q = r; q < e; ++q) {
                    P.fptr[q] = (int32_t)off;
                    const int64_t len = lens[P.perm[q]];
                    const int64_t ns = (len + kSegment - 1) / kSegment;
                    for (int64_t k = 0; k < ns; ++k) {
                        const int64_t s0 = off + k * kSegment, t0 = std::min(off + len, s0 + kSegment);
                        const int32_t d[8] = {(int32_t)s0, (int32_t)t0, q, (int32_t)ns, (int32_t)k, 0, 0, 0};
                        P.unit.insert(P.unit.end(), d, d + 8);
                    }
                    off += len;
                }
                b.units = P.units() - b.aux;
                P.ntickets += e - r;
                P.nslots += e - r;
            } else {
                // SLAB: slices of 32 rows padded to their longest row, one unit per
                // kSlabSteps steps of a slice (units of one slice consecutive)
                b.aux = P.units();
                b.slice0 = (int32_t)P.soff.size();
                b.aux2 = P.ntickets;
                b.slot0 = P.nslots;
                b.part0 = P.nslab_units;
                for (int q = r; q < e; ++q) P.fptr[q] = (int32_t)off;
                int32_t s = 0;
                for (int q = r; q < e; q += 32, ++s) {
                    int64_t lmax = 0;
                    for (int t = q; t < std::min(e, q + 32); ++t) lmax = std::max(lmax, lens[P.perm[t]]);
                    P.soff.push_back((int32_t)off);
                    const int64_t nu = (lmax + kSlabSteps - 1) / kSlabSteps;
                    for (int64_t c = 0; c < nu; ++c) {
                        const int32_t d[8] = {(int32_t)off, (int32_t)lmax, s, (int32_t)c, 0, 0, 0, 0};
                        P.unit.insert(P.unit.end(), d, d + 8);
                    }
                    off += 32 * lmax;
                }
                P.soff.push_back((int32_t)off);           // sentinel: end of the bin's last slice
                b.units = P.units() - b.aux;
                P.ntickets += s;
                P.nslots += s;                             // one epilogue slot per slice
                P.nslab_units += b.units;
            }
            bin_store.push_back(off - bin_off0);
            P.bt.bin[P.bt.nbins++] = b;
            r = e;
        }
        if (tr) tr->mark("    bins + offsets");
        P.fptr[R] = (int32_t)std::min<int64_t>(off, INT32_MAX);
        P.total = off;
        P.bin_store = bin_store;
        share_blocks(P.bt, P.bin_store, block_cap);
    }



    // Final device layout of one orientation from the internal CSR temporaries.
    int build_layout(const Plan& P, int R, const int32_t* tptr, const int32_t* tidx, const V* tval,
                     Layout<V>& L, int32_t* d_fptr, int32_t* d_soff, int32_t* d_unit,
                     int32_t* d_idx, V* d_val) {
        SPS_CK(cudaMemcpyAsync(d_fptr, P.fptr.data(), sizeof(int32_t) * (R + 1), cudaMemcpyHostToDevice, st));
        if (!P.soff.empty())
            SPS_CK(cudaMemcpyAsync(d_soff, P.soff.data(), sizeof(int32_t) * P.soff.size(), cudaMemcpyHostToDevice, st));
        if (!P.unit.empty())
            SPS_CK(cudaMemcpyAsync(d_unit, P.unit.data(), sizeof(int32_t) * P.unit.size(), cudaMemcpyHostToDevice, st));
        for (int i = 0; i < P.bt.nbins; ++i) {
            const Bin& b = P.bt.bin[i];
            if (b.mode == BM_SLICED)
                k_fill_sliced<V><<<grid_for((int64_t)b.units * 32), kBlock, 0, st>>>(
                    tptr, tidx, tval, d_soff, b.begin, b.end, b.aux, b.units, d_idx, d_val);
            else if (b.mode == BM_SLAB) {
                const int nsl = (b.end - b.begin + 31) / 32;
                k_fill_sliced<V><<<grid_for((int64_t)nsl * 32), kBlock, 0, st>>>(
                    tptr, tidx, tval, d_soff, b.begin, b.end, b.slice0, nsl, d_idx, d_val);
            } else
                k_fill_rows<V><<<grid_for((int64_t)(b.end - b.begin) * 32), kBlock, 0, st>>>(
                    tptr, tidx, tval, d_fptr, b.begin, b.end, d_idx, d_val);
        }
        SPS_CK(cudaGetLastError());
        L.ptr = d_fptr;
        L.idx = d_idx;
        L.val = d_val;
        L.soff = d_soff;
        L.unit = reinterpret_cast<const int4*>(d_unit);
        return SPS_OK;
    }

    int setup(const HostProblem& hp, const sps_options& o, int mode_) {
        opt = o;
        mode = mode_;
        n = hp.n;
        m = hp.m;
        nnz = hp.ptr[m];
        SPS_CK(cudaSetDevice(opt.device));
        cudaGetLastError();   // a stale non-sticky error from an unrelated call must not fail this setup
        SPS_CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        pool = engine_pool(opt.device);
        SPS_CK(cudaEventCreate(&ev0));
        SPS_CK(cudaEventCreate(&ev1));
        SPS_CK(cudaEventCreateWithFlags(&evq, cudaEventDisableTiming));
        SPS_CK(cudaHostAlloc((void**)&h_ctl, sizeof(Ctl), cudaHostAllocDefault));
        SPS_CK(cudaHostAlloc((void**)&h_abort, sizeof(int32_t), cudaHostAllocMapped));
        *h_abort = 0;
        SPS_CK(cudaHostGetDevicePointer((void**)&d_abort, h_abort, 0));
        if (m == 0 || n == 0) { trivial = true; return SPS_OK; }
        SPS_CK(cudaEventRecord(ev0, st));
        const int block_cap = opt.max_blocks > 0 ? opt.max_blocks : kSms * kPassMinBlocks;   // one resident wave

        std::vector<int64_t> rlen(m);
        for (int i = 0; i < m; ++i) rlen[i] = hp.ptr[i + 1] - hp.ptr[i];

        // ---- staging upload and validation
        int32_t *s_ptr, *s_idx, *s_colcount, *s_err;
        double* s_val;
        SPS_CK(dalloc(&s_ptr, sizeof(int32_t) * (m + 1)));
        SPS_CK(dalloc(&s_idx, sizeof(int32_t) * std::max<int64_t>(nnz, 1)));
        SPS_CK(dalloc(&s_val, sizeof(double) * std::max<int64_t>(nnz, 1)));
        SPS_CK(dalloc(&s_colcount, sizeof(int32_t) * (n + 1)));
        SPS_CK(dalloc(&s_err, sizeof(int32_t)));
        SPS_CK(cudaMemcpyAsync(s_ptr, hp.ptr.data(), sizeof(int32_t) * (m + 1), cudaMemcpyHostToDevice, st));
        {
            int64_t off = 0;
            for (const auto& sg : hp.segs) {
                if (sg.cnt == 0) continue;
                SPS_CK(cudaMemcpyAsync(s_idx + off, sg.idx, sizeof(int32_t) * sg.cnt, cudaMemcpyHostToDevice, st));
                SPS_CK(cudaMemcpyAsync(s_val + off, sg.val, sizeof(double) * sg.cnt, cudaMemcpyHostToDevice, st));
                off += sg.cnt;
            }
        }
        SPS_CK(cudaMemsetAsync(s_colcount, 0, sizeof(int32_t) * (n + 1), st));
        SPS_CK(cudaMemsetAsync(s_err, 0, sizeof(int32_t), st));
        if (nnz) k_validate_count<<<grid_for(nnz), kBlock, 0, st>>>(s_idx, s_val, nnz, n, s_colcount, s_err);
        SPS_CK(cudaGetLastError());
        std::vector<int32_t> colcount(n);
        int32_t herr = 0;
        SPS_CK(cudaMemcpyAsync(colcount.data(), s_colcount, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st));
        SPS_CK(cudaMemcpyAsync(&herr, s_err, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
        SPS_CK(cudaStreamSynchronize(st));
        if (herr) {
            cudaFreeAsync(s_ptr, st); cudaFreeAsync(s_idx, st); cudaFreeAsync(s_val, st); cudaFreeAsync(s_colcount, st); cudaFreeAsync(s_err, st);
            return fail(SPS_ERR_INVALID, (herr & SE_INDEX) ? "column index out of range [0, n)"
                                                           : "non-finite constraint matrix value");
        }

        if (trace) trace->mark("upload + validate");
        // ---- column plan
        std::vector<int64_t> clen(n);
        for_chunks(n, host_threads(n), [&](int, int lo, int hi) {
            for (int j = lo; j < hi; ++j) clen[j] = colcount[j];
        });
        Plan cp;
        if (trace) trace->mark("  column lengths");
        make_plan(clen, nullptr, nullptr, cp, block_cap, trace);
        if (trace) trace->mark("  column plan");
        const std::vector<int32_t>& perm_col = cp.perm;
        std::vector<int32_t> inv_col(n);
        for_chunks(n, host_threads(n), [&](int, int lo, int hi) {
            for (int j = lo; j < hi; ++j) inv_col[perm_col[j]] = j;
        });
        if (trace) trace->mark("  inverse column order");

        // ---- row plan: bins by row kind, length and gather locality (SLAB groups)
        Plan rp;
        {
            const std::vector<uint8_t> slab = choose_slab(hp, inv_col, (int)sizeof(V));
            if (trace) trace->mark("  SLAB choice");
            make_plan(rlen, &hp.kind, &slab, rp, block_cap);
            if (trace) trace->mark("  row plan");
        }
        const std::vector<int32_t>& perm_row = rp.perm;
        if (rp.total > INT32_MAX || cp.total > INT32_MAX) {
            cudaFreeAsync(s_ptr, st); cudaFreeAsync(s_idx, st); cudaFreeAsync(s_val, st); cudaFreeAsync(s_colcount, st); cudaFreeAsync(s_err, st);
            return fail(SPS_ERR_INVALID, "padded matrix layout exceeds 2^31-1 entries");
        }
        std::vector<int32_t> nptr(m + 1, 0), cptr(n + 1, 0);
        if (trace) trace->mark("  layout size checks");
        prefix_lengths(m, [&](int r) { return (int32_t)rlen[perm_row[r]]; }, nptr);
        prefix_lengths(n, [&](int j) { return colcount[perm_col[j]]; }, cptr);

        if (trace) trace->mark("host plans");
        // ---- persistent arena
        const int tail = 0;     // the column pass's blocks also update the dual average
        const int apply_blocks = grid_for(std::max(n, m), kBlock, kSms * 8);
        const size_t part_row_n = (size_t)std::max(rp.bt.total_blocks, 1) * kRowPartials;
        const size_t part_col_n = (size_t)(cp.bt.total_blocks + tail) * (kColPartials + kLagPartials);
        const size_t part_aux_n = (size_t)std::max(apply_blocks, kSms * 16) * 3;
        const size_t nseg = (size_t)std::max(std::max(rp.units(), cp.units()), 1);
        const size_t ntk = (size_t)std::max(std::max(rp.ntickets, cp.ntickets), 1);
        const size_t nslab = (size_t)std::max(std::max(rp.nslab_units, cp.nslab_units), 1);
        const bool adaptive = mode == SPS_MODE_ADAPTIVE;
        std::vector<std::pair<void**, size_t>> plan;
        int32_t *d_rptr, *d_ridx, *d_cptr, *d_cidx, *d_rsoff, *d_csoff, *d_runit, *d_cunit;
        V *d_rval, *d_cval, *d_c, *d_b, *d_lo = nullptr, *d_hi = nullptr, *d_tau = nullptr, *d_sigma = nullptr;
        double *d_dr, *d_dc, *d_pr, *d_pc, *d_pa, *d_segpart, *d_slabpart, *d_rowpart_r, *d_rowpart_c;
        double *d_idr = nullptr, *d_idc = nullptr;
        uint32_t* d_tickets;
        V *X0, *X1, *Y0, *Y1, *AX0 = nullptr, *AX1 = nullptr, *ATY0 = nullptr, *ATY1 = nullptr;
        V *xs, *ys, *xl = nullptr, *yl = nullptr, *AXa = nullptr, *ATYa = nullptr, *xbar = nullptr;
        V *xb = nullptr, *yb = nullptr, *AXl = nullptr, *ATYl = nullptr;
        double *d_px = nullptr, *d_py = nullptr;   // FP64 copies of the check's two points

        // uniform bounds: every column [L, U] with L in {0, -inf}, U = +inf
        bool uniform = true;
        const double L0 = hp.lb[0], U0 = hp.ub[0];
        if (!((L0 == 0.0 || std::isinf(L0)) && std::isinf(U0) && U0 > 0)) uniform = false;
        for (int j = 1; j < n && uniform; ++j)
            if (!(hp.lb[j] == L0 && hp.ub[j] == U0)) uniform = false;

        auto add = [&](void* p, size_t bytes) { plan.push_back({(void**)p, (std::max<size_t>(bytes, 4) + 255) & ~size_t(255)}); };
        add(&d_rptr, sizeof(int32_t) * (m + 1));
        add(&d_ridx, sizeof(int32_t) * std::max<int64_t>(rp.total, 1));
        add(&d_rval, sizeof(V) * std::max<int64_t>(rp.total, 1));
        add(&d_rsoff, sizeof(int32_t) * (rp.soff.size() + 1));
        add(&d_runit, sizeof(int32_t) * (rp.unit.size() + 8));
        add(&d_cptr, sizeof(int32_t) * (n + 1));
        add(&d_cidx, sizeof(int32_t) * std::max<int64_t>(cp.total, 1));
        add(&d_cval, sizeof(V) * std::max<int64_t>(cp.total, 1));
        add(&d_csoff, sizeof(int32_t) * (cp.soff.size() + 1));
        add(&d_cunit, sizeof(int32_t) * (cp.unit.size() + 8));
        add(&d_segpart, sizeof(double) * 2 * nseg);
        add(&d_slabpart, sizeof(double) * 64 * nslab);
        add(&d_tickets, sizeof(uint32_t) * ntk);
        add(&d_rowpart_r, sizeof(double) * kMaxEpiPartials * std::max(rp.nslots, 1));
        add(&d_rowpart_c, sizeof(double) * kMaxEpiPartials * std::max(cp.nslots, 1));
        add(&d_perm_row, sizeof(int32_t) * m);
        add(&d_perm_col, sizeof(int32_t) * n);
        add(&d_rkind, m);
        add(&d_c, sizeof(V) * n);
        add(&d_b, sizeof(V) * m);
        if (!uniform) { add(&d_lo, sizeof(V) * n); add(&d_hi, sizeof(V) * n); }
        add(&d_dr, sizeof(double) * m);
        add(&d_dc, sizeof(double) * n);
        add(&d_pr, sizeof(double) * part_row_n);
        add(&d_pc, sizeof(double) * part_col_n);
        add(&d_pa, sizeof(double) * part_aux_n);
        add(&X0, sizeof(V) * n); add(&X1, sizeof(V) * n);
        add(&Y0, sizeof(V) * m); add(&Y1, sizeof(V) * m);
        add(&xs, sizeof(V) * n); add(&ys, sizeof(V) * m);
        if (adaptive) {
            add(&AX0, sizeof(V) * m); add(&AX1, sizeof(V) * m);
            add(&ATY0, sizeof(V) * n); add(&ATY1, sizeof(V) * n);
            add(&xl, sizeof(V) * n); add(&yl, sizeof(V) * m);
            add(&AXa, sizeof(V) * m); add(&ATYa, sizeof(V) * n);
            add(&d_idr, sizeof(double) * m); add(&d_idc, sizeof(double) * n);
            add(&AXl, sizeof(V) * m); add(&ATYl, sizeof(V) * n);
            if (stall_test()) { add(&xb, sizeof(V) * n); add(&yb, sizeof(V) * m); }
            add(&d_px, sizeof(double) * 2 * n); add(&d_py, sizeof(double) * 2 * m);
        } else {
            add(&xbar, sizeof(V) * n);
            add(&d_tau, sizeof(V) * n);
            add(&d_sigma, sizeof(V) * m);
        }
        add(&d_ctl, sizeof(Ctl));
        add(&d_xout, sizeof(double) * n);
        add(&d_yout, sizeof(double) * m);
        if (adaptive) {
            add(&d_cuser, sizeof(double) * n);
            add(&d_obj, sizeof(double) * 2);
            if (!uniform) { add(&d_lbuser, sizeof(double) * n); add(&d_ubuser, sizeof(double) * n); }
        }
        add(&d_wx, sizeof(double) * n);
        add(&d_wy, sizeof(double) * m);
        size_t total = 0;
        for (auto& p : plan) total += p.second;
        SPS_CK(dalloc(&arena, total));
        {
            size_t off = 0;
            for (auto& p : plan) { *p.first = arena + off; off += p.second; }
        }
        SPS_CK(cudaMemsetAsync(d_tickets, 0, sizeof(uint32_t) * ntk, st));

        if (trace) trace->mark("arena");
        // ---- internal CSR and CSC temporaries (FP64 values)
        int32_t *t_inv_col, *t_fill, *t_ptr, *t_idx, *t_cptr, *t_cidx;
        double *t_rval, *t_cval, *t_stat;
        SPS_CK(dalloc(&t_inv_col, sizeof(int32_t) * n));
        SPS_CK(dalloc(&t_fill, sizeof(int32_t) * n));
        SPS_CK(dalloc(&t_ptr, sizeof(int32_t) * (m + 1)));
        SPS_CK(dalloc(&t_cptr, sizeof(int32_t) * (n + 1)));
        SPS_CK(dalloc(&t_idx, sizeof(int32_t) * std::max<int64_t>(nnz, 1)));
        SPS_CK(dalloc(&t_cidx, sizeof(int32_t) * std::max<int64_t>(nnz, 1)));
        SPS_CK(dalloc(&t_rval, sizeof(double) * std::max<int64_t>(nnz, 1)));
        SPS_CK(dalloc(&t_cval, sizeof(double) * std::max<int64_t>(nnz, 1)));
        SPS_CK(dalloc(&t_stat, sizeof(double) * 2 * (size_t)(n + m)));
        SPS_CK(cudaMemcpyAsync(d_perm_row, perm_row.data(), sizeof(int32_t) * m, cudaMemcpyHostToDevice, st));
        SPS_CK(cudaMemcpyAsync(d_perm_col, perm_col.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, st));
        SPS_CK(cudaMemcpyAsync(t_inv_col, inv_col.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, st));
        SPS_CK(cudaMemcpyAsync(t_ptr, nptr.data(), sizeof(int32_t) * (m + 1), cudaMemcpyHostToDevice, st));
        SPS_CK(cudaMemcpyAsync(t_cptr, cptr.data(), sizeof(int32_t) * (n + 1), cudaMemcpyHostToDevice, st));
        {
            std::vector<int8_t> kind_int(m);
            for (int r = 0; r < m; ++r) kind_int[r] = hp.kind[perm_row[r]];
            SPS_CK(cudaMemcpyAsync(d_rkind, kind_int.data(), m, cudaMemcpyHostToDevice, st));
            SPS_CK(cudaStreamSynchronize(st));
        }
        const int warp_grid_m = grid_for((int64_t)m * 32), warp_grid_n = grid_for((int64_t)n * 32);
        if (nnz) {
            k_build_csr<<<warp_grid_m, kBlock, 0, st>>>(s_ptr, s_idx, s_val, d_perm_row, t_inv_col, t_ptr, t_idx,
                                                        t_rval, m);
            SPS_CK(cudaMemsetAsync(t_fill, 0, sizeof(int32_t) * n, st));
            k_scatter_csc<<<warp_grid_m, kBlock, 0, st>>>(t_ptr, t_idx, t_rval, t_cptr, t_fill, t_cidx, t_cval, m);
            k_sort_columns<<<grid_for(n), kBlock, 0, st>>>(t_cptr, t_cidx, t_cval, n);
            SPS_CK(cudaGetLastError());
        }
        SPS_CK(cudaStreamSynchronize(st));
        cudaFreeAsync(s_ptr, st); cudaFreeAsync(s_idx, st); cudaFreeAsync(s_val, st); cudaFreeAsync(s_colcount, st); cudaFreeAsync(s_err, st);
        // columns too long for the device insertion sort: ordered on the host, with
        // one copy each way of the CSC range that holds them (four copies per
        // column cost seconds on the 168k long columns of a 1.1e8-nonzero LP)
        {
            int32_t j0 = -1, j1 = -1;
            for (int j = 0; j < n; ++j)
                if (cptr[j + 1] - cptr[j] > kSortMax) {
                    if (j0 < 0) j0 = j;
                    j1 = j + 1;
                }
            if (j0 >= 0) {
                const int64_t lo = cptr[j0], len = (int64_t)cptr[j1] - cptr[j0];
                std::vector<int32_t> ri(len);
                std::vector<double> rv(len);
                SPS_CK(cudaMemcpyAsync(ri.data(), t_cidx + lo, sizeof(int32_t) * len, cudaMemcpyDeviceToHost, st));
                SPS_CK(cudaMemcpyAsync(rv.data(), t_cval + lo, sizeof(double) * len, cudaMemcpyDeviceToHost, st));
                SPS_CK(cudaStreamSynchronize(st));
                sort_long_columns(cptr.data(), j0, j1, ri.data(), rv.data());
                SPS_CK(cudaMemcpyAsync(t_cidx + lo, ri.data(), sizeof(int32_t) * len, cudaMemcpyHostToDevice, st));
                SPS_CK(cudaMemcpyAsync(t_cval + lo, rv.data(), sizeof(double) * len, cudaMemcpyHostToDevice, st));
                SPS_CK(cudaStreamSynchronize(st));
            }
        }

        if (trace) trace->mark("CSR/CSC build + sort");
        // ---- scaling (adaptive) or reference diagonal steps, on the FP64 temporaries
        double *rmax = t_stat, *rsum = t_stat + m, *cmax = t_stat + 2 * m, *csum = t_stat + 2 * m + n;
        {
            std::vector<double> ones(std::max(n, m), 1.0);
            SPS_CK(cudaMemcpyAsync(d_dr, ones.data(), sizeof(double) * m, cudaMemcpyHostToDevice, st));
            SPS_CK(cudaMemcpyAsync(d_dc, ones.data(), sizeof(double) * n, cudaMemcpyHostToDevice, st));
            SPS_CK(cudaStreamSynchronize(st));
        }
        auto stats = [&]() {
            launch_abs_stats(t_ptr, t_idx, t_rval, d_dr, d_dc, rmax, rsum, m, nnz, kSms * 16, st);
            launch_abs_stats(t_cptr, t_cidx, t_cval, d_dc, d_dr, cmax, csum, n, nnz, kSms * 16, st);
        };
        if (adaptive) {
            const int ruiz = opt.ruiz_iters >= 0 ? opt.ruiz_iters : 10;
            for (int it = 0; it < ruiz; ++it) {
                stats();
                k_rescale<<<grid_for(m), kBlock, 0, st>>>(d_dr, rmax, m);
                k_rescale<<<grid_for(n), kBlock, 0, st>>>(d_dc, cmax, n);
            }
            stats();
            k_rescale<<<grid_for(m), kBlock, 0, st>>>(d_dr, rsum, m);
            k_rescale<<<grid_for(n), kBlock, 0, st>>>(d_dc, csum, n);
        } else {
            stats();
            k_diag_steps<V><<<grid_for(std::max(n, m)), kBlock, 0, st>>>(csum, rsum, d_tau, d_sigma, n, m);
        }
        // scaled values in the iterate precision
        SPS_CK(cudaStreamSynchronize(st));
        cudaFreeAsync(t_stat, st);
        V *t_rvV, *t_cvV;
        SPS_CK(dalloc(&t_rvV, sizeof(V) * std::max<int64_t>(nnz, 1)));
        SPS_CK(dalloc(&t_cvV, sizeof(V) * std::max<int64_t>(nnz, 1)));
        k_finish_values<V><<<warp_grid_m, kBlock, 0, st>>>(t_ptr, t_idx, t_rval, d_dr, d_dc, t_rvV, m);
        k_finish_values<V><<<warp_grid_n, kBlock, 0, st>>>(t_cptr, t_cidx, t_cval, d_dc, d_dr, t_cvV, n);
        SPS_CK(cudaGetLastError());

        if (trace) trace->mark("scaling");
        // ---- final binned layouts
        Layout<V> Lr{}, Lc{};
        if (int rc = build_layout(rp, m, t_ptr, t_idx, t_rvV, Lr, d_rptr, d_rsoff, d_runit, d_ridx, d_rval)) return rc;
        if (int rc = build_layout(cp, n, t_cptr, t_cidx, t_cvV, Lc, d_cptr, d_csoff, d_cunit, d_cidx, d_cval)) return rc;
        Lr.seg_part = Lc.seg_part = d_segpart;
        Lr.slab_part = Lc.slab_part = d_slabpart;
        Lr.seg_ticket = Lc.seg_ticket = d_tickets;
        Lr.seg_rowpart = d_rowpart_r;
        Lc.seg_rowpart = d_rowpart_c;
        Lr.nsegrows = rp.nslots;
        Lc.nsegrows = cp.nslots;

        if (trace) trace->mark("binned layouts");
        // ---- vectors in internal order (uploaded in the caller's order, permuted on the device)
        {
            double *t_c, *t_l, *t_u, *t_b;
            SPS_CK(dalloc(&t_c, sizeof(double) * (3 * (size_t)n + m)));
            t_l = t_c + n; t_u = t_l + n; t_b = t_u + n;
            SPS_CK(cudaMemcpyAsync(t_c, hp.c, sizeof(double) * n, cudaMemcpyHostToDevice, st));
            SPS_CK(cudaMemcpyAsync(t_l, hp.lb, sizeof(double) * n, cudaMemcpyHostToDevice, st));
            SPS_CK(cudaMemcpyAsync(t_u, hp.ub, sizeof(double) * n, cudaMemcpyHostToDevice, st));
            SPS_CK(cudaMemcpyAsync(t_b, hp.rhs.data(), sizeof(double) * m, cudaMemcpyHostToDevice, st));
            k_scale_vectors<V><<<grid_for(std::max(n, m)), kBlock, 0, st>>>(t_c, t_l, t_u, t_b, d_perm_col, d_perm_row,
                                                                           d_dc, d_dr, d_c, d_lo, d_hi, d_b, n, m);
            if (d_idc) k_reciprocals<<<grid_for(std::max(n, m)), kBlock, 0, st>>>(d_dc, d_dr, d_idc, d_idr, n, m);
            if (d_cuser) SPS_CK(cudaMemcpyAsync(d_cuser, t_c, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
            if (d_lbuser) SPS_CK(cudaMemcpyAsync(d_lbuser, t_l, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
            if (d_ubuser) SPS_CK(cudaMemcpyAsync(d_ubuser, t_u, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
            SPS_CK(cudaGetLastError());
            SPS_CK(cudaStreamSynchronize(st));
            cudaFreeAsync(t_c, st);
        }
        cudaFreeAsync(t_inv_col, st); cudaFreeAsync(t_fill, st); cudaFreeAsync(t_ptr, st); cudaFreeAsync(t_cptr, st); cudaFreeAsync(t_idx, st);
        cudaFreeAsync(t_cidx, st); cudaFreeAsync(t_rval, st); cudaFreeAsync(t_cval, st); cudaFreeAsync(t_rvV, st); cudaFreeAsync(t_cvV, st);

        if (trace) trace->mark("vectors");
        // ---- start-up constants: eta0 = 1 / max|K~|, omega0 = ||c~|| / ||b~||
        {
            const int g = kSms * 2;
            double* t_n;
            SPS_CK(dalloc(&t_n, sizeof(double) * 3 * g));
            k_norms<V><<<g, kBlock, 0, st>>>(d_rval, rp.total, d_c, n, d_b, m, t_n);
            std::vector<double> hn(3 * g);
            SPS_CK(cudaMemcpyAsync(hn.data(), t_n, sizeof(double) * 3 * g, cudaMemcpyDeviceToHost, st));
            SPS_CK(cudaStreamSynchronize(st));
            cudaFreeAsync(t_n, st);
            double mx = 0, sc = 0, sb = 0;
            for (int q = 0; q < g; ++q) { mx = std::max(mx, hn[3 * q]); sc += hn[3 * q + 1]; sb += hn[3 * q + 2]; }
            eta0 = mx > 0 ? 1.0 / mx : 1.0;
            omega0 = (sc > 1e-20 && sb > 1e-20) ? std::sqrt(sc) / std::sqrt(sb) : 1.0;
        }

        // ---- normalisers of the reported error (original data, FP64)
        double nb2 = 0, nc2 = 0;
        for (int i = 0; i < m; ++i) nb2 += hp.rhs[i] * hp.rhs[i];
        for (int j = 0; j < n; ++j) nc2 += hp.c[j] * hp.c[j];
        Args<V>& a = args;
        a.n = n; a.m = m;
        a.csr = Lr;
        a.csc = Lc;
        a.rows = rp.bt; a.cols = cp.bt;
        {   // the check kernels' shares: one wave at their own occupancy
            int nr = 0, nc = 0;
            if (adaptive) {
                SPS_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nr, ad_row_check<V>, kBlock, 0));
                if (opt.kkt_form == SPS_KKT_PDLP)
                    SPS_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nc, ad_col_check<V, true>, kBlock, 0));
                else
                    SPS_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nc, ad_col_check<V, false>, kBlock, 0));
            } else {
                SPS_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nr, rf_row_check<V>, kBlock, 0));
                SPS_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nc, rf_col_check<V>, kBlock, 0));
            }
            a.rows_chk = rp.bt;
            a.cols_chk = cp.bt;
            share_blocks(a.rows_chk, rp.bin_store, std::min(block_cap, kSms * std::max(nr, 1)));
            share_blocks(a.cols_chk, cp.bin_store, std::min(block_cap, kSms * std::max(nc, 1)));
        }
        a.col_tail_blocks = tail;
        a.apply_blocks = apply_blocks;
        // Programmatic dependent launch of the step kernels where a pass is short enough
        // for the launch and the first unit's load latency to matter: on GB300 it cut the
        // attempt by 6 % on a 200 x 500 LP and 2 % on a 4M-nonzero transportation LP,
        // and slowed a 21M-nonzero power-law LP's row pass by 4 % (which keeps the plain
        // instantiations).
        a.pdl = adaptive && rp.total + cp.total < (int64_t(1) << 25);
        a.c = d_c; a.b = d_b; a.lo = d_lo; a.hi = d_hi;
        a.uniform_bounds = uniform;
        a.far_residual = adaptive && opt.kkt_form == SPS_KKT_PDLP;
        a.lo_u = V(L0); a.hi_u = V(U0);
        a.dr = d_dr; a.dc = d_dc;
        a.idr = d_idr; a.idc = d_idc;
        a.tau = d_tau; a.sigma = d_sigma;
        if (adaptive) {
            a.inv_nb = 1.0 / (1.0 + std::sqrt(nb2));
            a.inv_nc = 1.0 / (1.0 + std::sqrt(nc2));
        } else {
            a.inv_nb = 1.0 / std::max(1.0, std::sqrt(nb2));
            a.inv_nc = 1.0 / std::max(1.0, std::sqrt(nc2));
        }
        a.X[0] = X0; a.X[1] = X1; a.Y[0] = Y0; a.Y[1] = Y1;
        a.AX[0] = AX0; a.AX[1] = AX1; a.ATY[0] = ATY0; a.ATY[1] = ATY1;
        a.xs = xs; a.ys = ys; a.xl = xl; a.yl = yl; a.AXa = AXa; a.ATYa = ATYa; a.xbar = xbar;
        a.xb = xb; a.yb = yb;
        a.AXl = AXl; a.ATYl = ATYl;
        a.px[0] = d_px; a.px[1] = d_px ? d_px + n : nullptr;
        a.py[0] = d_py; a.py[1] = d_py ? d_py + m : nullptr;
        a.part_row = d_pr; a.part_col = d_pc; a.part_aux = d_pa;
        a.ctl = d_ctl;
        a.abort_flag = d_abort;
        a.has_cond = 0;
        a.check_interval = opt.check_interval > 0 ? opt.check_interval : (adaptive ? 64 : 50);
        layout_rows = rp.bt;
        layout_cols = cp.bt;
        padded_nnz_rows = rp.total;
        padded_nnz_cols = cp.total;
        SPS_CK(cudaMemsetAsync(d_ctl, 0, sizeof(Ctl), st));
        SPS_CK(cudaEventRecord(ev1, st));
        SPS_CK(cudaStreamSynchronize(st));
        float ms = 0;
        cudaEventElapsedTime(&ms, ev0, ev1);
        setup_ms = ms;
        if (trace) trace->mark("device set-up done");
        return SPS_OK;
    }

    // ---------------------------------------------------------------- solve
    int nodes_per_window() const { return 2 * args.check_interval + (mode == SPS_MODE_ADAPTIVE ? 4 : 3); }

    // column check in the error form the options ask for (the PDLP form's kernel adds
    // the Lagrangian form's partials of the same points)
    void launch_col_check(const Args<V>& a) {
        if (a.far_residual) ad_col_check<V, true><<<a.cols_chk.total_blocks, kBlock, 0, st>>>(a);
        else ad_col_check<V, false><<<a.cols_chk.total_blocks, kBlock, 0, st>>>(a);
    }

    // An adaptive pass kernel as the programmatic dependent of the kernel before it
    // on the stream (its blocks may start during that kernel's last blocks; the
    // kernel waits for it with griddepcontrol.wait before reading what it wrote).
    cudaError_t launch_err = cudaSuccess;
    template <class K>
    void launch_pass(K kernel, int grid, const Args<V>& a) {
        cudaLaunchConfig_t cfg{};
        cfg.gridDim = dim3((unsigned)grid);
        cfg.blockDim = dim3(kBlock);
        cfg.dynamicSmemBytes = 0;
        cfg.stream = st;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        const cudaError_t e = cudaLaunchKernelEx(&cfg, kernel, a);
        if (e != cudaSuccess && launch_err == cudaSuccess) launch_err = e;
    }

    void launch_window(const Args<V>& a) {
        const int W = a.check_interval;
        const int gr = a.rows.total_blocks, gc = a.cols.total_blocks;
        if (mode == SPS_MODE_ADAPTIVE) {
            for (int w = 0; w < W; ++w) {
                if (a.pdl) {
                    launch_pass(ad_row_step<V, true>, gr, a);
                    launch_pass(ad_col_step<V, true>, gc + a.col_tail_blocks, a);
                } else {
                    ad_row_step<V><<<gr, kBlock, 0, st>>>(a);
                    ad_col_step<V><<<gc + a.col_tail_blocks, kBlock, 0, st>>>(a);
                }
            }
            ad_check_prep<V><<<a.apply_blocks, kBlock, 0, st>>>(a);
            ad_row_check<V><<<a.rows_chk.total_blocks, kBlock, 0, st>>>(a);
            launch_col_check(a);
            ad_apply<V><<<a.apply_blocks, kBlock, 0, st>>>(a);
        } else {
            for (int w = 0; w < W; ++w) {
                rf_col_step<V><<<gc, kBlock, 0, st>>>(a);
                rf_row_step<V><<<gr, kBlock, 0, st>>>(a);
            }
            rf_row_check<V><<<a.rows_chk.total_blocks, kBlock, 0, st>>>(a, 0);
            rf_col_check<V><<<a.cols_chk.total_blocks, kBlock, 0, st>>>(a, 0);
            rf_apply<V><<<a.apply_blocks, kBlock, 0, st>>>(a);
        }
    }

    int build_window_graph() {
        cudaGraph_t g;
        SPS_CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        Args<V> a = args;
        a.has_cond = 0;
        launch_err = cudaSuccess;
        launch_window(a);
        cudaError_t le = launch_err;
        SPS_CK(cudaStreamEndCapture(st, &g));
        SPS_CK(le);
        cudaError_t e = cudaGraphInstantiate(&win_exec, g, 0);
        cudaGraphDestroy(g);
        SPS_CK(e);
        return SPS_OK;
    }

    int build_loop_graph() {
        cudaGraph_t g;
        SPS_CK(cudaGraphCreate(&g, 0));
        cudaGraphConditionalHandle h;
        cudaError_t e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault);
        if (e != cudaSuccess) { cudaGraphDestroy(g); SPS_CK(e); }
        cudaGraphNodeParams p{};
        p.type = cudaGraphNodeTypeConditional;
        p.conditional.handle = h;
        p.conditional.type = cudaGraphCondTypeWhile;
        p.conditional.size = 1;
        cudaGraphNode_t node;
        e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &p);
        if (e != cudaSuccess) { cudaGraphDestroy(g); SPS_CK(e); }
        cudaGraph_t body = p.conditional.phGraph_out[0];
        e = cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) { cudaGraphDestroy(g); SPS_CK(e); }
        Args<V> a = args;
        a.cond = h;
        a.has_cond = 1;
        launch_err = cudaSuccess;
        launch_window(a);
        e = cudaStreamEndCapture(st, &body);
        if (e == cudaSuccess) e = launch_err;
        if (e != cudaSuccess) { cudaGraphDestroy(g); SPS_CK(e); }
        e = cudaGraphInstantiate(&loop_exec, g, 0);
        cudaGraphDestroy(g);
        SPS_CK(e);
        return SPS_OK;
    }

    // Wait for the stream with bounded polling; raises the abort flag once the
    // time limit (plus grace) has passed and gives up after a hard limit.
    int wait_stream(std::chrono::steady_clock::time_point t0) {
        SPS_CK(cudaEventRecord(evq, st));
        const double tl = opt.time_limit_s;
        for (;;) {
            cudaError_t q = cudaEventQuery(evq);
            if (q == cudaSuccess) return SPS_OK;
            if (q != cudaErrorNotReady) SPS_CK(q);
            const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            if (tl > 0 && el > tl + 2.0) *(volatile int32_t*)h_abort = 1;
            if (tl > 0 && el > tl + 120.0) return fail(SPS_ERR_TIMEOUT, "device did not stop after the time limit");
            std::this_thread::sleep_for(std::chrono::microseconds(el < 0.01 ? 5 : 100));
        }
    }

    int run_loop(std::chrono::steady_clock::time_point t0) {
        const int64_t W = args.check_interval;
        const int64_t max_windows = opt.max_iters / W + 3;
        args.max_windows = max_windows;
        int gm = opt.graph_mode;
        if (gm == 2) {
            if (!loop_exec && build_loop_graph() != SPS_OK) { cudaGetLastError(); gm = 1; err.clear(); }
            if (gm == 2) {
                SPS_CK(cudaGraphLaunch(loop_exec, st));
                int rc = wait_stream(t0);
                if (rc) return rc;
                SPS_CK(cudaMemcpyAsync(h_ctl, d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
                SPS_CK(cudaStreamSynchronize(st));
                launches += (int64_t)h_ctl->windows * nodes_per_window();
                return SPS_OK;
            }
        }
        if (gm == 1 && !win_exec && build_window_graph() != SPS_OK) { cudaGetLastError(); gm = 0; err.clear(); }
        int64_t batch = 1, run = 0;
        for (;;) {
            for (int64_t b = 0; b < batch; ++b) {
                if (gm == 1) SPS_CK(cudaGraphLaunch(win_exec, st));
                else {
                    launch_err = cudaSuccess;
                    launch_window(args);
                    SPS_CK(launch_err);
                }
            }
            run += batch;
            launches += batch * nodes_per_window();
            SPS_CK(cudaGetLastError());
            SPS_CK(cudaMemcpyAsync(h_ctl, d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
            int rc = wait_stream(t0);
            if (rc) return rc;
            if (h_ctl->done || h_ctl->iters >= opt.max_iters || run >= max_windows) break;
            batch = std::min<int64_t>(batch * 2, 16);
        }
        return SPS_OK;
    }

    int solve(sps_result* res) override {
        SPS_CK(cudaSetDevice(opt.device));
        std::memset(res, 0, sizeof(*res));
        if (trivial) return solve_trivial(res);
        const auto t0 = std::chrono::steady_clock::now();
        const bool adaptive = mode == SPS_MODE_ADAPTIVE;
        Ctl c0{};
        c0.status = SPS_STATUS_ITERATION_LIMIT;
        c0.init_phase = 1;
        c0.max_iters = opt.max_iters;
        c0.tol = opt.tol;
        c0.eta = eta0;
        c0.omega = omega0;
        c0.kkt_last = INFINITY;
        c0.stall_on = stall_test() ? 1 : 0;
        c0.stall_ceiling = kStallCeiling;
        *h_ctl = c0;
        *(volatile int32_t*)h_abort = 0;
        launches = 0;
        const uint64_t tl_ns = opt.time_limit_s > 0 ? (uint64_t)(opt.time_limit_s * 1e9) : 0;
        SPS_CK(cudaEventRecord(ev0, st));
        SPS_CK(cudaMemcpyAsync(d_ctl, h_ctl, sizeof(Ctl), cudaMemcpyHostToDevice, st));
        const int gr = args.rows.total_blocks, gc = args.cols.total_blocks;
        const bool warm = adaptive && (have_warm_x || have_warm_y);
        warm_used = warm;
        if (adaptive) {
            // start-up: the start point, its products, its KKT check (init phase) and the
            // first candidate; with the fallback the warm point's relative KKT error is
            // compared with the cold start's (cached per problem) and the better one kept
            auto start = [&](bool use_warm) -> int {
                Ctl c = c0;
                if (use_warm && warm_omega > 0) c.omega = warm_omega;
                *h_ctl = c;
                SPS_CK(cudaMemcpyAsync(d_ctl, h_ctl, sizeof(Ctl), cudaMemcpyHostToDevice, st));
                k_ad_start<V><<<args.apply_blocks, kBlock, 0, st>>>(args, use_warm && have_warm_x ? d_wx : nullptr,
                                                                   use_warm && have_warm_y ? d_wy : nullptr,
                                                                   d_perm_col, d_perm_row, d_rkind, tl_ns);
                spmv_rows<V><<<gr, kBlock, 0, st>>>(args, args.X[0], args.AX[0]);
                spmv_cols<V><<<gc, kBlock, 0, st>>>(args, args.Y[0], args.ATY[0]);
                ad_check_prep<V><<<args.apply_blocks, kBlock, 0, st>>>(args);
                ad_row_check<V><<<args.rows_chk.total_blocks, kBlock, 0, st>>>(args);
                launch_col_check(args);
                ad_apply<V><<<args.apply_blocks, kBlock, 0, st>>>(args);
                launches += 7;
                SPS_CK(cudaGetLastError());
                return SPS_OK;
            };
            auto start_error = [&](double* rel) -> int {
                SPS_CK(cudaMemcpyAsync(h_ctl, d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
                SPS_CK(cudaStreamSynchronize(st));
                *rel = h_ctl->rel_kkt;
                return SPS_OK;
            };
            if (warm && opt.warm_fallback) {
                if (!(cold_rel >= 0.0)) {
                    if (int rc = start(false)) return rc;
                    if (int rc = start_error(&cold_rel)) return rc;
                }
                double warm_rel = 0.0;
                if (int rc = start(true)) return rc;
                if (int rc = start_error(&warm_rel)) return rc;
                if (!(warm_rel <= cold_rel)) {
                    warm_used = false;
                    if (int rc = start(false)) return rc;
                }
            } else if (int rc = start(warm)) {
                return rc;
            }
        } else {
            k_rf_start<V><<<args.apply_blocks, kBlock, 0, st>>>(args, tl_ns);
            rf_row_check<V><<<args.rows_chk.total_blocks, kBlock, 0, st>>>(args, 1);
            rf_col_check<V><<<args.cols_chk.total_blocks, kBlock, 0, st>>>(args, 1);
            launches += 3;
        }
        SPS_CK(cudaGetLastError());
        int rc = run_loop(t0);
        if (rc) return rc;
        SPS_CK(cudaMemcpyAsync(h_ctl, d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
        SPS_CK(cudaStreamSynchronize(st));
        int status = h_ctl->status;
        if (!h_ctl->done) status = SPS_STATUS_ITERATION_LIMIT;
        if (!adaptive && status != SPS_STATUS_OPTIMAL) {
            // report the error of the returned (current) point
            rf_row_check<V><<<args.rows_chk.total_blocks, kBlock, 0, st>>>(args, 1);
            rf_col_check<V><<<args.cols_chk.total_blocks, kBlock, 0, st>>>(args, 1);
            launches += 2;
        }
        const int cur = adaptive ? h_ctl->cur : 0;
        double obj = 0;
        if (adaptive) {
            // the solution in the caller's order, clipped to the caller's bounds, and c^T x,
            // on the device: it stays there until sps_get_solution asks for it
            SPS_CK(cudaMemsetAsync(d_obj, 0, sizeof(double) * 2, st));
            k_extract_user<V><<<args.apply_blocks, kBlock, 0, st>>>(
                args.X[cur], args.Y[cur], args.dc, args.dr, d_perm_col, d_perm_row, d_cuser, d_lbuser, d_ubuser,
                lb_user.empty() ? 0.0 : lb_user[0], ub_user.empty() ? 0.0 : ub_user[0], d_xout, d_yout, n, m,
                args.part_aux, reinterpret_cast<uint32_t*>(d_obj + 1), d_obj);
        } else {
            k_extract<V><<<args.apply_blocks, kBlock, 0, st>>>(args.X[cur], args.Y[cur], args.dc, args.dr, d_perm_col,
                                                               d_perm_row, d_xout, d_yout, n, m);
        }
        launches += 1;
        SPS_CK(cudaGetLastError());
        SPS_CK(cudaEventRecord(ev1, st));
        SPS_CK(cudaMemcpyAsync(h_ctl, d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
        std::vector<double> xo, yo;
        if (adaptive) {
            SPS_CK(cudaMemcpyAsync(&obj, d_obj, sizeof(double), cudaMemcpyDeviceToHost, st));
        } else {
            xo.resize(n);
            yo.resize(m);
            SPS_CK(cudaMemcpyAsync(xo.data(), d_xout, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
            SPS_CK(cudaMemcpyAsync(yo.data(), d_yout, sizeof(double) * m, cudaMemcpyDeviceToHost, st));
        }
        SPS_CK(cudaStreamSynchronize(st));
        float ms = 0;
        cudaEventElapsedTime(&ms, ev0, ev1);
        sol_on_device = adaptive;
        if (!adaptive) {
            to_user(xo, yo);
            for (int j = 0; j < n_user; ++j) obj += c_user[j] * x_sol[j];
        }
        res->status = status;
        res->restarts = h_ctl->restarts;
        res->iterations = h_ctl->iters;
        res->accepted_steps = adaptive ? h_ctl->accepted_total : h_ctl->iters;
        res->rel_kkt = h_ctl->rel_kkt;
        res->rel_primal = h_ctl->rel_p;
        res->rel_dual = h_ctl->rel_d;
        res->rel_gap = h_ctl->rel_gap;
        res->rel_kkt_lagrangian = adaptive ? h_ctl->rel_kkt_lagr : h_ctl->rel_kkt;
        res->primal_weight = h_ctl->omega;
        res->step_size = h_ctl->eta;
        res->setup_ms = setup_ms;
        res->solve_ms = ms;
        res->kernel_launches = launches;
        res->returned_average = h_ctl->choice;
        res->warm_start_used = warm_used ? 1 : 0;
        res->objective = obj;
        solved = true;
        return SPS_OK;
    }

    // Problems with no rows or no columns: nothing runs on the device.
    int solve_trivial(sps_result* res) {
        sol_on_device = false;
        x_sol.assign(n_user, 0.0);
        y_sol.assign(m_user, 0.0);
        res->status = SPS_STATUS_OPTIMAL;
        if (mode == SPS_MODE_ADAPTIVE) {
            for (int j = 0; j < n_user; ++j) {
                const double c = c_user[j];
                double v = c > 0 ? lb_user[j] : (c < 0 ? ub_user[j] : std::min(std::max(0.0, lb_user[j]), ub_user[j]));
                if (!std::isfinite(v)) { res->status = SPS_STATUS_NUMERIC_ERROR; v = std::min(std::max(0.0, lb_user[j]), ub_user[j]); }
                x_sol[j] = v;
            }
        }
        double obj = 0;
        for (int j = 0; j < n_user; ++j) obj += c_user[j] * x_sol[j];
        res->objective = obj;
        res->setup_ms = setup_ms;
        solved = true;
        return SPS_OK;
    }

    // Device-problem solution -> caller's space.
    void to_user(const std::vector<double>& xo, const std::vector<double>& yo) {
        x_sol.assign(n_user, 0.0);
        y_sol.assign(m_user, 0.0);
        if (mode == SPS_MODE_ADAPTIVE) {
            for (int j = 0; j < n_user; ++j) x_sol[j] = xo[j];
            for (int i = 0; i < m_user; ++i) y_sol[i] = yo[i];
        } else {
            const StdMap& s = smap;
            for (int j = 0; j < n_user; ++j) x_sol[j] = xo[j] + s.lb_shift[j];
            const int m_le = s.m_ub + s.nub;
            for (int i = 0; i < s.m_ub; ++i) y_sol[i] = s.neg[i] ? -yo[i] : yo[i];
            for (int i = 0; i < s.m_eq; ++i) y_sol[s.m_ub + i] = s.neg[m_le + i] ? -yo[m_le + i] : yo[m_le + i];
        }
        for (int j = 0; j < n_user; ++j) {
            const double lo = std::isfinite(lb_user[j]) ? lb_user[j] : -1e30;
            const double hi = std::isfinite(ub_user[j]) ? ub_user[j] : 1e30;
            x_sol[j] = std::min(std::max(x_sol[j], lo), hi);
        }
    }

    int warm(const double* x0, const double* y0, double omega0_) override {
        if (mode != SPS_MODE_ADAPTIVE) return fail(SPS_ERR_STATE, "warm start needs the adaptive mode");
        warm_omega = omega0_;
        have_warm_x = x0 != nullptr;
        have_warm_y = y0 != nullptr;
        if (trivial) return SPS_OK;
        SPS_CK(cudaSetDevice(opt.device));
        if (x0) SPS_CK(cudaMemcpyAsync(d_wx, x0, sizeof(double) * n, cudaMemcpyHostToDevice, st));
        if (y0) SPS_CK(cudaMemcpyAsync(d_wy, y0, sizeof(double) * m, cudaMemcpyHostToDevice, st));
        SPS_CK(cudaStreamSynchronize(st));
        return SPS_OK;
    }

    // Per-launch timing of the two iteration kernels on the resident state.
    // The control block is saved, opened for `reps` more iterations, and restored.
    int time_kernels(int reps, double* out, bool graph) override {
        if (!solved) return fail(SPS_ERR_STATE, "call sps_solve before timing kernels");
        if (reps <= 0) return fail(SPS_ERR_INVALID, "reps must be positive");
        if (trivial) { out[0] = out[1] = 0.0; out[2] = 1.0; return SPS_OK; }
        SPS_CK(cudaSetDevice(opt.device));
        Ctl saved;
        SPS_CK(cudaMemcpy(&saved, d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost));
        Ctl t = saved;
        t.done = 0;
        t.apply = 0;
        t.max_iters = INT64_MAX / 2;
        SPS_CK(cudaMemcpy(d_ctl, &t, sizeof(Ctl), cudaMemcpyHostToDevice));
        std::vector<cudaEvent_t> ev(2 * reps + 1);
        for (auto& e : ev) SPS_CK(cudaEventCreate(&e));
        const int gr = args.rows.total_blocks, gc = args.cols.total_blocks;
        Args<V> a = args;
        a.has_cond = 0;
        if (graph) {
            // two graphs captured from the stream: reps x [row pass, column pass] and reps x
            // [row pass], each timed by events around its replay (no events between the
            // kernels, which would add their own gaps): row = the second / reps, column =
            // (the first - the second) / reps
            float tg[2] = {0.f, 0.f};
            cudaError_t rec = cudaSuccess;
            for (int variant = 0; variant < 2 && rec == cudaSuccess; ++variant) {
                cudaGraph_t g = nullptr;
                cudaGraphExec_t ge = nullptr;
                rec = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
                if (rec != cudaSuccess) break;
                launch_err = cudaSuccess;
                for (int r = 0; r < reps; ++r) {
                    if (mode == SPS_MODE_ADAPTIVE && a.pdl) {
                        launch_pass(ad_row_step<V, true>, gr, a);
                        if (variant == 0) launch_pass(ad_col_step<V, true>, gc + a.col_tail_blocks, a);
                    } else if (mode == SPS_MODE_ADAPTIVE) {
                        ad_row_step<V><<<gr, kBlock, 0, st>>>(a);
                        if (variant == 0) ad_col_step<V><<<gc + a.col_tail_blocks, kBlock, 0, st>>>(a);
                    } else {
                        rf_row_step<V><<<gr, kBlock, 0, st>>>(a);
                        if (variant == 0) rf_col_step<V><<<gc, kBlock, 0, st>>>(a);
                    }
                }
                rec = cudaGetLastError();
                if (rec == cudaSuccess) rec = launch_err;
                const cudaError_t end = cudaStreamEndCapture(st, &g);     // always ends the capture
                if (rec == cudaSuccess) rec = end;
                if (rec == cudaSuccess) rec = cudaGraphInstantiate(&ge, g, 0);
                if (rec == cudaSuccess) rec = cudaGraphLaunch(ge, st);   // warm-up replay
                if (rec == cudaSuccess) rec = cudaEventRecord(ev[0], st);
                if (rec == cudaSuccess) rec = cudaGraphLaunch(ge, st);
                if (rec == cudaSuccess) rec = cudaEventRecord(ev[1], st);
                if (rec == cudaSuccess) rec = cudaStreamSynchronize(st);
                if (rec == cudaSuccess) rec = cudaEventElapsedTime(&tg[variant], ev[0], ev[1]);
                if (ge) cudaGraphExecDestroy(ge);
                if (g) cudaGraphDestroy(g);
                if (variant == 0 && rec == cudaSuccess) {
                    Ctl after;
                    rec = cudaMemcpy(&after, d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost);
                    out[2] = mode == SPS_MODE_ADAPTIVE
                                 ? double(after.accepted_total - t.accepted_total) / (2.0 * reps) : 1.0;
                    if (rec == cudaSuccess) rec = cudaMemcpy(d_ctl, &t, sizeof(Ctl), cudaMemcpyHostToDevice);
                }
            }
            for (auto& e : ev) cudaEventDestroy(e);
            const cudaError_t back = cudaMemcpy(d_ctl, &saved, sizeof(Ctl), cudaMemcpyHostToDevice);
            if (rec == cudaSuccess) rec = back;
            if (rec != cudaSuccess)
                return fail(SPS_ERR_CUDA, std::string("timing the iteration kernels: ") + cudaGetErrorString(rec));
            out[0] = tg[1] / reps;
            out[1] = (tg[0] - tg[1]) / reps;
            return SPS_OK;
        }
        SPS_CK(cudaEventRecord(ev[0], st));
        for (int r = 0; r < reps; ++r) {
            if (mode == SPS_MODE_ADAPTIVE) {
                ad_row_step<V><<<gr, kBlock, 0, st>>>(a);
                SPS_CK(cudaEventRecord(ev[2 * r + 1], st));
                ad_col_step<V><<<gc + a.col_tail_blocks, kBlock, 0, st>>>(a);
            } else {
                rf_row_step<V><<<gr, kBlock, 0, st>>>(a);
                SPS_CK(cudaEventRecord(ev[2 * r + 1], st));
                rf_col_step<V><<<gc, kBlock, 0, st>>>(a);
            }
            SPS_CK(cudaEventRecord(ev[2 * r + 2], st));
        }
        SPS_CK(cudaGetLastError());
        SPS_CK(cudaStreamSynchronize(st));
        double row = 0, col = 0;
        for (int r = 0; r < reps; ++r) {
            float a1 = 0, a2 = 0;
            cudaEventElapsedTime(&a1, ev[2 * r], ev[2 * r + 1]);
            cudaEventElapsedTime(&a2, ev[2 * r + 1], ev[2 * r + 2]);
            row += a1;
            col += a2;
        }
        Ctl after;
        SPS_CK(cudaMemcpy(&after, d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost));
        for (auto& e : ev) cudaEventDestroy(e);
        SPS_CK(cudaMemcpy(d_ctl, &saved, sizeof(Ctl), cudaMemcpyHostToDevice));
        out[0] = row / reps;
        out[1] = col / reps;
        out[2] = mode == SPS_MODE_ADAPTIVE ? double(after.accepted_total - saved.accepted_total) / reps : 1.0;
        return SPS_OK;
    }

    // The stall test runs for adaptive FP32 solves unless escalation is off.
    bool stall_test() const { return mode == SPS_MODE_ADAPTIVE && sizeof(V) == 4 && opt.escalate != 0; }

    void set_limits(int64_t max_iters, double time_limit_s) override {
        opt.max_iters = max_iters;
        opt.time_limit_s = time_limit_s;
    }

    int get_best(double* x, double* y, double* omega) override {
        if (!solved) return fail(SPS_ERR_STATE, "no solution: call sps_solve first");
        if (trivial || !args.xb || !h_ctl->best_saved) {
            *omega = h_ctl->omega;
            return get(x, y);
        }
        SPS_CK(cudaSetDevice(opt.device));
        k_extract<V><<<args.apply_blocks, kBlock, 0, st>>>(args.xb, args.yb, args.dc, args.dr, d_perm_col,
                                                           d_perm_row, d_xout, d_yout, n, m);
        SPS_CK(cudaGetLastError());
        std::vector<double> xo(n), yo(m);
        SPS_CK(cudaMemcpyAsync(xo.data(), d_xout, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
        SPS_CK(cudaMemcpyAsync(yo.data(), d_yout, sizeof(double) * m, cudaMemcpyDeviceToHost, st));
        SPS_CK(cudaStreamSynchronize(st));
        for (int j = 0; j < n_user; ++j) x[j] = std::min(std::max(xo[j], lb_user[j]), ub_user[j]);
        for (int i = 0; i < m_user; ++i) y[i] = yo[i];
        *omega = h_ctl->omega_best;
        return SPS_OK;
    }

    int get(double* x, double* y) override {
        if (!solved) return fail(SPS_ERR_STATE, "no solution: call sps_solve first");
        if (sol_on_device) {
            SPS_CK(cudaSetDevice(opt.device));
            if (x) SPS_CK(cudaMemcpyAsync(x, d_xout, sizeof(double) * n_user, cudaMemcpyDeviceToHost, st));
            if (y) SPS_CK(cudaMemcpyAsync(y, d_yout, sizeof(double) * m_user, cudaMemcpyDeviceToHost, st));
            SPS_CK(cudaStreamSynchronize(st));
            return SPS_OK;
        }
        if (x) std::memcpy(x, x_sol.data(), sizeof(double) * n_user);
        if (y) std::memcpy(y, y_sol.data(), sizeof(double) * m_user);
        return SPS_OK;
    }
};

EngineBase* make_engine_f32();
EngineBase* make_engine_f64();
int setup_f32(EngineBase* e, const HostProblem& hp, const sps_options& o, int mode);
int setup_f64(EngineBase* e, const HostProblem& hp, const sps_options& o, int mode);

}  // namespace sps
