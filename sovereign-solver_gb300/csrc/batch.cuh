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
    int32_t n, m, m_ub, pad;
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
};

// ---------------------------------------------------------------------------
// Group traversal inside one block: G lanes per row, rows [0, count).
// g(q, j) gathers, e.pre(r) / e(r, acc, pre) as in the single-LP visitors.
template <int G, int NV, class Acc, class Gather, class Epi>
__device__ __forceinline__ void group_rows(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                                           const float* __restrict__ val, int count, const Gather& g, Epi& e) {
    constexpr int per_warp = 32 / G;
    const int warp = threadIdx.x >> 5, wl = threadIdx.x & 31, lane = wl & (G - 1);
    for (int base = warp * per_warp; base < count; base += kWarps * per_warp) {
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
                                               int count, const Gather& g, Epi& e) {
    switch (G) {
        case 1: group_rows<1, NV, Acc>(ptr, idx, val, count, g, e); break;
        case 2: group_rows<2, NV, Acc>(ptr, idx, val, count, g, e); break;
        case 4: group_rows<4, NV, Acc>(ptr, idx, val, count, g, e); break;
        case 8: group_rows<8, NV, Acc>(ptr, idx, val, count, g, e); break;
        case 16: group_rows<16, NV, Acc>(ptr, idx, val, count, g, e); break;
        default: group_rows<32, NV, Acc>(ptr, idx, val, count, g, e); break;
    }
}

// Row passes: G lanes per row in {4, 8, 16, 32} (several rows per warp in flight).
template <int NV, class Acc, class Gather, class Epi>
__device__ __forceinline__ void group_rows_r(int G, const int32_t* ptr, const int32_t* idx, const float* val,
                                             int count, const Gather& g, Epi& e) {
    switch (G) {
        case 4: group_rows<4, NV, Acc>(ptr, idx, val, count, g, e); break;
        case 8: group_rows<8, NV, Acc>(ptr, idx, val, count, g, e); break;
        case 16: group_rows<16, NV, Acc>(ptr, idx, val, count, g, e); break;
        default: group_rows<32, NV, Acc>(ptr, idx, val, count, g, e); break;
    }
}

// Schedule of a launch: lanes per column (low byte) and per row (next byte).
__host__ __device__ constexpr int pack_schedule(int gc, int gr) { return gc | (gr << 8); }

}  // namespace batch
}  // namespace sps
