// batch.cuh — batched restarted PDHG: thousands of independent LPs of uneven
// sizes in one persistent launch.
//
// Layout: every instance's CSR (rows: A_ub then A_eq) and CSC are packed back
// to back (offsets inside an instance are local, 0-based); column vectors and
// row vectors likewise.  One block of 256 threads owns one instance at a time
// and runs the whole adaptive PDHG loop on it with block barriers only: rows
// one warp each, columns `G` lanes each (G in 1..32, autotuned), FP32 iterates, FP64
// block reductions, the same step/restart/termination decisions as the
// single-LP kernels (decide.cuh) on a shared-memory control block.
// Instances are handed out largest first from an atomic counter.
#pragma once

#include "decide.cuh"

namespace sps {
namespace batch {

struct Inst {                 // per-instance descriptor
    int32_t n, m, m_ub, nnz;
    int64_t rp, re;           // row-offset base (m + 1 entries), row-entry base
    int64_t cp, ce;           // column-offset base (n + 1 entries), column-entry base
    int64_t vc, vr;           // column-vector base, row-vector base
    double inv_nb, inv_nc;    // 1 / (1 + ||rhs||), 1 / (1 + ||c||) of the original data
};

struct Arrays {
    const int32_t *rptr, *ridx, *cptr, *cidx;
    const float *rval, *cval;
    const int8_t* kind;       // per row: 1 = '<='
    const float *c, *lo, *hi, *b;
    const double *dc, *dr;
    const double *eta0, *omega0;
    float *x0, *x1, *aty0, *aty1, *xs, *xl, *atya;
    float *y0, *y1, *ax0, *ax1, *ys, *yl, *axa;
    float *xb, *yb;           // best point of the stall test (null when it is off)
    float *axl, *atyl;        // K x_last, K^T y_last (infeasibility tests)
};

struct Args {
    const Inst* inst;
    const int32_t* order;     // instances in hand-out order
    int32_t count;
    int32_t check_interval;
    int64_t max_iters;
    double tol;
    const uint64_t* deadline; // device: absolute globaltimer deadline (ns), 0 = none
    Arrays a;
    Ctl* out;                 // per instance final state
    uint32_t* counter;
    int32_t stall_on;         // stall test on (FP64 continuation on the host)
    int32_t warm, fallback;   // warm starts set / cold-start fallback on
    const double *wx, *wy, *wom;   // warm starts (original space, packed like the vectors), omega0
    double* cold_rel;         // per instance: relative KKT error of the cold start (< 0 = unknown)
    int32_t team;             // cluster size of the launch (1 = one block per instance)
    int32_t team_nnz;         // instances with at least this many nonzeros are solved by a whole cluster
    int32_t* team_error;      // set when a team barrier gave up waiting
    int32_t stage_cap;        // floats of the block's shared staging buffer (0 = gathers from global)
    uint32_t* idle;           // blocks that found the instance queue empty (reset per launch)
    uint32_t idle_need;       // hand-off threshold: 7/8 of the launch's blocks
    int32_t handoff_nnz;      // instances this large may be handed off (0 = never)
};

// Internal status of an instance that left the launch's tail for the single-LP
// engine (replaced by the continuation's status before any caller sees it).
constexpr int32_t kStatusHandoff = 100;
constexpr int64_t kHandoffMin = 512;      // attempts an instance makes before it may be handed off

// ---------------------------------------------------------------------------
// Teams: the blocks of one thread-block cluster solving one large instance.
// Rows and columns are split over the team's warps; every reduction is each
// block's partial published in its shared memory and summed by every block in
// rank order, so all blocks take the same decisions without a broadcast.
// The team barrier is a counter in rank 0's shared memory (release-add,
// acquire-poll at cluster scope) with a bounded wait: a block that waits
// longer than kTeamSpin polls (about a second) records an error and leaves.
constexpr int kXch = 32;                  // doubles per exchange buffer
constexpr int32_t kTeamNnz = 65536;       // smallest size solved by a team
constexpr uint32_t kTeamSpin = 1u << 21;

__device__ __forceinline__ uint32_t cluster_addr(const void* p, uint32_t rank) {
    uint32_t a = (uint32_t)__cvta_generic_to_shared(p), r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
    return r;
}
__device__ __forceinline__ void cluster_add_release(uint32_t addr, uint32_t v) {
    asm volatile("red.release.cluster.shared::cluster.add.u32 [%0], %1;" ::"r"(addr), "r"(v) : "memory");
}
__device__ __forceinline__ uint32_t cluster_load_acquire(uint32_t addr) {
    uint32_t v;
    asm volatile("ld.acquire.cluster.shared::cluster.u32 %0, [%1];" : "=r"(v) : "r"(addr) : "memory");
    return v;
}
__device__ __forceinline__ double cluster_load_f64(uint32_t addr) {
    double v;
    asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(addr) : "memory");
    return v;
}

struct Team {
    int size, rank;           // blocks on the instance, this block's cluster rank
    uint32_t* counter;        // barrier counter (this block's copy; rank 0's is the one used)
    uint32_t* gen;            // barriers passed (this block)
    double* xch;              // 2 x kXch exchange buffers (this block)
    int* phase;               // which exchange buffer is next
    int* err;                 // 1 once a barrier timed out
};

// All threads: barrier over the team with global-memory ordering.  Returns false
// (for every thread of the block) when the wait timed out.  The block's barrier
// orders its threads' writes before thread 0's release-add, which publishes them
// to the cluster (a release is cumulative); thread 0's acquire-poll and the
// closing block barrier make the other blocks' writes visible to every thread.
__device__ __forceinline__ bool team_barrier(const Team& T) {
    if (T.size <= 1) {
        __syncthreads();
        return true;
    }
    __syncthreads();
    if (threadIdx.x == 0 && !*T.err) {
        const uint32_t target = (*T.gen + 1) * (uint32_t)T.size;
        const uint32_t a = cluster_addr(T.counter, 0);
        cluster_add_release(a, 1u);
        uint32_t it = 0;
        while (cluster_load_acquire(a) < target) {
            if (++it > kTeamSpin) { *T.err = 1; break; }
            __nanosleep(64);
        }
        *T.gen += 1;
    }
    __syncthreads();
    return !*T.err;
}

// Thread 0 holds a block total in t; afterwards thread 0 holds the team total
// (blocks added in rank order).  Returns false on a barrier timeout.
template <int N>
__device__ __forceinline__ bool team_total(double (&t)[N], const Team& T) {
    static_assert(N <= kXch, "exchange buffer too small");
    if (T.size <= 1) return true;
    double* buf = T.xch + (*T.phase & 1) * kXch;
    if (threadIdx.x == 0)
        for (int q = 0; q < N; ++q) buf[q] = t[q];
    if (!team_barrier(T)) return false;
    if (threadIdx.x == 0) {
        for (int q = 0; q < N; ++q) t[q] = 0.0;
        for (int r = 0; r < T.size; ++r) {
            const uint32_t a = cluster_addr(buf, (uint32_t)r);
            for (int q = 0; q < N; ++q) t[q] += cluster_load_f64(a + 8u * q);
        }
    }
    *T.phase += 1;            // every thread keeps the same count
    return true;
}

// ---------------------------------------------------------------------------
// Group traversal inside one block: G lanes per row, rows [0, count).
// g(q, j) gathers, e.pre(r) / e(r, acc, pre) as in the single-LP visitors.
template <int G, int NV, class Acc, class Gather, class Epi>
__device__ __forceinline__ void group_rows(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                                           const float* __restrict__ val, int count, const Gather& g, Epi& e,
                                           int trank = 0, int tsize = 1) {
    constexpr int per_warp = 32 / G;
    const int warp = threadIdx.x >> 5, wl = threadIdx.x & 31, lane = wl & (G - 1);
    for (int base = (trank * kWarps + warp) * per_warp; base < count; base += tsize * kWarps * per_warp) {
        const int r = base + wl / G;
        const bool valid = r < count;
        typename Epi::Pre pre;
        if (valid && lane == 0) pre = e.pre(r);
        const int s = valid ? __ldg(ptr + r) : 0, t = valid ? __ldg(ptr + r + 1) : 0;
        Acc acc[NV];
#pragma unroll
        for (int q = 0; q < NV; ++q) acc[q] = Acc(0);
        for (int k = s + lane; k < t; k += 4 * G) {
            int j[4];
            Acc a[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int kk = k + u * G;
                const bool ok = kk < t;
                j[u] = ok ? __ldg(idx + kk) : 0;
                a[u] = ok ? Acc(__ldg(val + kk)) : Acc(0);
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int q = 0; q < NV; ++q) acc[q] += a[u] * g(q, j[u]);
        }
#pragma unroll
        for (int q = 0; q < NV; ++q) acc[q] = group_sum<G>(acc[q]);
        if (valid && lane == 0) e(r, acc, pre);
    }
}

template <int NV, class Acc, class Gather, class Epi>
__device__ __forceinline__ void group_rows_dyn(int G, const int32_t* ptr, const int32_t* idx, const float* val,
                                               int count, const Gather& g, Epi& e, int tr = 0, int ts = 1) {
    switch (G) {
        case 1: group_rows<1, NV, Acc>(ptr, idx, val, count, g, e, tr, ts); break;
        case 2: group_rows<2, NV, Acc>(ptr, idx, val, count, g, e, tr, ts); break;
        case 4: group_rows<4, NV, Acc>(ptr, idx, val, count, g, e, tr, ts); break;
        case 8: group_rows<8, NV, Acc>(ptr, idx, val, count, g, e, tr, ts); break;
        case 16: group_rows<16, NV, Acc>(ptr, idx, val, count, g, e, tr, ts); break;
        default: group_rows<32, NV, Acc>(ptr, idx, val, count, g, e, tr, ts); break;
    }
}

// Row passes: G lanes per row in {4, 8, 16, 32} (several rows per warp in flight).
template <int NV, class Acc, class Gather, class Epi>
__device__ __forceinline__ void group_rows_r(int G, const int32_t* ptr, const int32_t* idx, const float* val,
                                             int count, const Gather& g, Epi& e, int tr = 0, int ts = 1) {
    switch (G) {
        case 4: group_rows<4, NV, Acc>(ptr, idx, val, count, g, e, tr, ts); break;
        case 8: group_rows<8, NV, Acc>(ptr, idx, val, count, g, e, tr, ts); break;
        case 16: group_rows<16, NV, Acc>(ptr, idx, val, count, g, e, tr, ts); break;
        default: group_rows<32, NV, Acc>(ptr, idx, val, count, g, e, tr, ts); break;
    }
}

// Schedule of a launch: lanes per column (low byte) and per row (next byte).
__host__ __device__ constexpr int pack_schedule(int gc, int gr) { return gc | (gr << 8); }

}  // namespace batch
}  // namespace sps
