// engine.cuh — device data layout and shared device helpers of the PDHG engine.
//
// Matrix layout in HBM (both orientations: CSR for K x, CSC for K^T y).
// Rows (or columns) are renumbered so that every bin — one row kind ('<=' or
// '=') and one schedule — is a contiguous index range.  Three schedules:
//
//   SLICED   rows with <= 32 nonzeros, sorted by length (descending) inside the
//            bin and stored as SELL-32 slices: the k-th entry of the t-th row of
//            slice s sits at soff[s] + 32 k + t.  One thread per row; a warp's 32
//            loads of step k are one 128-byte line; no offset -> index chain.
//            Short rows are zero-padded to the slice's longest row.
//   WARP     rows with 33..512 nonzeros, CSR; one warp per row.
//   SEGMENT  longer rows, CSR, cut into 512-nonzero segments; one warp per
//            segment; the last warp to finish a row (per-row ticket) adds the
//            segment partials in segment order and runs the row's epilogue.
//   SLAB     longer rows whose neighbours share their column pattern shifted by
//            one (the k-th nonzeros of rows r and r+1 sit in adjacent columns:
//            demand rows of a transportation LP, time-expanded flows), stored
//            SELL-32 like SLICED and cut into units of 32 steps (1024 entries);
//            lane t owns row t of the slice, so the gathers of a step are one
//            128-byte line where CSR would touch 32 sectors.  The last warp to
//            finish a slice (per-slice ticket) adds the units' partials in unit
//            order and runs the slice's 32 epilogues.  The host picks SLAB per
//            group of 32 rows when it touches at most half the sectors of CSR.
//
// Index arrays are int32, values V (float or double); every reduction is FP64
// at block level.  Scale factors are FP64.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace sps {

constexpr int kBlock = 256;          // threads per block of every pass kernel
constexpr int kWarps = kBlock / 32;
constexpr int kMaxBins = 8;
constexpr int kSliceMax = 32;        // rows up to this length are SLICED
#ifndef SPS_SEGMENT_NNZ
#define SPS_SEGMENT_NNZ 512
#endif
#ifndef SPS_SLAB_STEPS
#define SPS_SLAB_STEPS 32
#endif
constexpr int kSegment = SPS_SEGMENT_NNZ;   // WARP rows up to this length; SEGMENT size above it
constexpr int kSlabSteps = SPS_SLAB_STEPS;  // steps (32-entry columns of a slice) per SLAB unit
// SEGMENT bins of at most this many rows: a row's last segment acquires its
// partners' partials by a load of the row's ticket (cheaper on the row's own
// path, but it drops the SM's L1); larger bins acquire by a fence, so the
// gathers of the other warps on the SM keep their L1 lines.  Measured with the
// load for every bin: the transportation LP's row pass (1 000 SEGMENT rows)
// 15.7 -> 14.7 us, the power-law LP's (34k SEGMENT rows) 113.5 -> 117.4 us.
constexpr int kSegLoadAcquireRows = 4096;

enum BinMode { BM_SLICED = 0, BM_WARP = 1, BM_SEGMENT = 2, BM_SLAB = 3 };

// One contiguous range of internal rows (or columns) with one schedule.
struct Bin {
    int32_t begin, end;      // internal rows [begin, end)
    int32_t mode;            // BinMode
    int32_t kind;            // row pass: 1 = '<=' rows, 0 = '=' rows; column pass: 0
    int32_t block_begin;     // first block of this bin in a launch
    int32_t nblocks;
    int32_t units;           // slices (SLICED), rows (WARP), segments (SEGMENT) or units (SLAB)
    int32_t aux;             // SLICED: first global slice; SEGMENT / SLAB: first global unit
    int32_t aux2;            // SEGMENT: first per-row ticket; SLAB: first per-slice ticket
    int32_t slice0;          // SLAB: first global slice; SLICED with uniform length: the bin's offset
    int32_t part0;           // SLAB: first unit in the layout's SLAB partials; SLICED: the uniform
                             // row length of every slice (0 = lengths vary, read soff); SEGMENT:
                             // 1 = rows acquire by a load of their ticket, 0 = by a fence
    int32_t slot0;           // SEGMENT: first row slot of epilogue partials; SLAB: first slice slot
};

struct BinTable {
    int32_t nbins;
    int32_t total_blocks;
    Bin bin[kMaxBins];
};

template <class V>
struct Layout {
    const int32_t* ptr;      // CSR offsets of WARP / SEGMENT rows (m + 1 entries)
    const int32_t* idx;
    const V* val;
    const int32_t* soff;     // slice offsets (slices + 1)
    const int4* unit;        // SEGMENT / SLAB unit descriptors, two int4 (32 bytes) per unit:
                             //   SEGMENT {s, t, r, nseg} {kseg, 0, 0, 0}: nonzeros [s, t) of
                             //     internal row r, segment kseg of its nseg
                             //   SLAB    {off, len, sl, c} {0, 0, 0, 0}: unit c of slice sl of
                             //     the bin, the slice's entries at off, len steps (padded)
                             // one 32-byte read instead of a unit table -> row offset chain
    double* seg_part;        // per-segment partial sums (2 doubles of room each)
    double* slab_part;       // per SLAB unit: 32 lanes' partial sums (64 doubles of room each)
    uint32_t* seg_ticket;    // per-row tickets of SEGMENT rows (left at 0 after every pass)
    double* seg_rowpart;     // per SEGMENT row / SLAB slice: its epilogue's reduction partials
    int32_t nsegrows;        // epilogue slots of this orientation (SEGMENT rows, SLAB slices)
};

constexpr int kMaxEpiPartials = 14;

// Control block, one per handle, in device memory.  Written only by single
// threads of "last blocks" or by block 0 thread 0, read by every kernel.
struct Ctl {
    int32_t done;            // 1 -> every iteration kernel returns at entry
    int32_t status;          // SPS_STATUS_* once done
    int32_t cur;             // adaptive: index of the accepted state buffers
    int32_t accepted;        // adaptive: last attempt accepted
    int32_t apply;           // pending action for the apply kernel (ApplyBits), 8 = step pending
    int32_t restarts;
    int32_t choice;          // returned point: 0 current, 1 average
    int32_t init_phase;      // 1 while the check kernels only record the starting error
    int64_t iters;           // iterations (reference) / attempts (adaptive)
    int64_t accepted_total;
    int64_t window;          // reference: iterations since restart; adaptive: attempts since restart
    int64_t max_iters;
    int64_t last_restart_iter;
    double eta, omega;       // adaptive step size and primal weight
    double eta_used;         // step of the last accepted attempt (averaging weight)
    double w_sum;            // sum of averaging weights
    double dx2;              // ||x' - x||^2 of the pending candidate
    double kkt_last;         // reference: current_kkt; adaptive: weighted KKT at last restart
    double kkt_prev_cand;    // adaptive: weighted KKT of the previous restart candidate
    double tol;
    double norm_b, norm_c;   // normalisers of the reported error
    double rel_kkt, rel_p, rel_d, rel_gap, pobj, dobj;   // last evaluated returned-point metrics
    double last_avg_kkt, last_cur_kkt;
    uint64_t deadline_ns;    // device globaltimer deadline, 0 = none
    uint32_t ticket[8];      // last-block tickets, one per kernel kind
    int32_t abort_seen;
    int32_t windows;         // window bodies executed (loop guard)
    // stall test (adaptive FP32 with escalation)
    int32_t stall_on;        // 1: finish with SPS_STATUS_STALLED when the best error stops halving
    int32_t best_saved;      // 1 once a best point has been copied to xb / yb
    int64_t anchor_iter;     // attempt at which the best error last halved
    double anchor_rel;       // best error at that attempt
    double best_rel;         // best relative KKT error seen at a check
    double omega_best;       // primal weight when the best point was taken
    double stall_ceiling;    // a stall is declared only at or below this error (INFINITY: always)
    uint64_t t_begin, t_end; // batched solver: device clock (ns) at the instance's start and end
    int32_t warm_used;       // batched solver: the instance started from its warm start
    double rel_kkt_lagr;     // the returned point's error in the Lagrangian form (= rel_kkt unless
                             // the single-LP engine measures the PDLP form)
};

enum TicketSlot { T_ROW_STEP = 0, T_COL_STEP, T_ROW_CHECK, T_COL_CHECK, T_APPLY, T_AUX0, T_AUX1, T_AUX2 };

// ---------------------------------------------------------------------------
// reductions

template <int G, class T>
__device__ __forceinline__ T group_sum(T v) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sum NP values over the block; result valid in thread 0.  Fixed order.  T is
// float in the FP32 engine's iteration kernels: this GPU issues FP64 at 1/64 of
// the FP32 rate (2 thread operations per SM cycle), so a 256-thread FP64 shuffle
// tree per block and per attempt costs more than the block's own FP32 work.
template <int NP, class T>
__device__ __forceinline__ void block_sum(T (&v)[NP], T* smem /* kWarps*NP */) {
#pragma unroll
    for (int p = 0; p < NP; ++p) v[p] = group_sum<32>(v[p]);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) {
#pragma unroll
        for (int p = 0; p < NP; ++p) smem[w * NP + p] = v[p];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int p = 0; p < NP; ++p) {
            T s = T(0);
            for (int q = 0; q < kWarps; ++q) s += smem[q * NP + p];
            v[p] = s;
        }
    }
    __syncthreads();
}

// Ticket counters (a kernel's blocks, a SLAB slice's units, a SEGMENT row's
// segments: the one that arrives last combines the others' partials).  Every
// publisher increments with release semantics at GPU scope: its earlier writes,
// and those of the threads that reached a barrier with it before the call, are
// visible to whoever observes a later count.  Only the thread that reads the
// final count then acquires: by a load of the ticket with acquire semantics
// (the increments form one chain of read-modify-writes, so the load synchronises
// with every publisher's release), or by an acquire fence; after a barrier its
// warp or block sees the partials too.  The load is the cheaper acquire for the
// combining thread but it drops the SM's L1 (see kSegLoadAcquireRows).  Same
// box, same sums, against a sequentially consistent fence before every
// increment and after the last: 200x500 LP 7.34 -> 7.14 ms per solve,
// transportation LP 101.0 -> 98.6 ms, power-law LP 804.7 -> 799.5 ms per 4 096
// attempts (all with the fence for SEGMENT rows).
__device__ __forceinline__ uint32_t ticket_release(uint32_t* t) {
    uint32_t old;
    asm volatile("atom.release.gpu.global.add.u32 %0, [%1], 1;" : "=r"(old) : "l"(t) : "memory");
    return old;
}
__device__ __forceinline__ void ticket_acquire(const uint32_t* t) {
    asm volatile("{\n\t.reg .u32 v;\n\tld.acquire.gpu.global.u32 v, [%0];\n\t}" ::"l"(t) : "memory");
}
__device__ __forceinline__ void ticket_acquire_fence() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }

// Write this block's NP partials, then report whether this block is the last
// one of the grid to finish (ticket counter; no waiting).  In the last block the
// barrier after thread 0's acquire makes every block's partials (and the slots
// its threads wrote before its own barrier) visible to all threads.
template <int NP, class T>
__device__ __forceinline__ bool publish_partials(T (&v)[NP], T* partials, uint32_t* ticket,
                                                 T* smem, bool* am_last) {
    block_sum<NP>(v, smem);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int p = 0; p < NP; ++p) partials[(size_t)blockIdx.x * NP + p] = v[p];
        const bool last = ticket_release(ticket) == gridDim.x - 1;
        if (last) ticket_acquire(ticket);
        *am_last = last;
    }
    __syncthreads();
    return *am_last;
}

// In the last block, after publish_partials (or in a later kernel): sum the
// partials of all nblk blocks (fixed order; each thread's loads are issued
// before its adds).
template <int NP, class T>
__device__ __forceinline__ void gather_partials(T (&tot)[NP], const T* partials, int nblk, T* smem) {
    constexpr int B = 4;
#pragma unroll
    for (int p = 0; p < NP; ++p) tot[p] = T(0);
    for (int b0 = threadIdx.x; b0 < nblk; b0 += kBlock * B) {
        T v[B][NP];
#pragma unroll
        for (int u = 0; u < B; ++u) {
            const int b = b0 + u * kBlock;
#pragma unroll
            for (int p = 0; p < NP; ++p) v[u][p] = b < nblk ? __ldcg(partials + (size_t)b * NP + p) : T(0);
        }
#pragma unroll
        for (int u = 0; u < B; ++u)
#pragma unroll
            for (int p = 0; p < NP; ++p) tot[p] += v[u][p];
    }
    block_sum<NP>(tot, smem);
}

// A value every thread of the block needs, computed once by thread 0 (FP64
// divisions and products per thread would occupy the slow FP64 pipe).
template <class T, class F>
__device__ __forceinline__ T block_scalar(F f) {
    __shared__ T s;
    if (threadIdx.x == 0) s = T(f());
    __syncthreads();
    return s;
}

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}


// ---------------------------------------------------------------------------
// Binned traversal.  For every row the epilogue functor provides
//   e.pre(r)                  loads the row's own operands (issued before the
//                             row's dot product, so they overlap its gathers)
//   e(r, kind, acc[NV], pre)  consumes them; called once per row by one thread
// and the gather functor g(q, j) returns vector q at column j (as Acc).
// All control flow below is warp-uniform, so full-mask shuffles are safe.

#ifndef SPS_UNROLL
#define SPS_UNROLL 8
#endif
constexpr int kUnroll = SPS_UNROLL;
// Partial loads in flight when a row's (slice's) last unit adds its units'
// partials (the adds stay in unit order): 16 for one FP32 value per unit (a
// transportation demand slice has 32 units: two round trips instead of four),
// 8 where more registers per partial would spill at the step kernels' budget.
template <int NV, class Acc>
__host__ __device__ constexpr int finish_batch() { return NV * sizeof(Acc) <= 4 ? 16 : 8; }
constexpr int kPassMinBlocks = 5;    // resident blocks per SM the iteration kernels are built for

// SLICED: lane t of the warp owns row begin + 32*slice + t.  Two slices per
// step (the second may be past the bin) so their loads are in flight together.
template <int NV, class Acc, class V, class Gather, class Epi>
__device__ __forceinline__ void visit_slice_pair(const Bin& b, int s0, int s1, const Layout<V>& L,
                                                 const Gather& g, Epi& e) {
    const int lane = threadIdx.x & 31;
    const bool has1 = s1 < b.units;
    int off[2], len[2], r[2];
    typename Epi::Pre pre[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int s = h ? (has1 ? s1 : s0) : s0;
        const int gs = b.aux + s;
        if (b.part0 > 0) {                 // every slice of the bin has part0 steps: no offset reads
            off[h] = b.slice0 + s * 32 * b.part0;
            len[h] = (h && !has1) ? 0 : b.part0;
        } else {
            off[h] = __ldg(L.soff + gs);
            len[h] = (h && !has1) ? 0 : ((__ldg(L.soff + gs + 1) - off[h]) >> 5);
        }
        r[h] = b.begin + s * 32 + lane;
        if (r[h] < b.end && (h == 0 || has1)) pre[h] = e.pre(r[h]);
    }
    Acc acc[2][NV];
#pragma unroll
    for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int q = 0; q < NV; ++q) acc[h][q] = Acc(0);
    const int lmax = max(len[0], len[1]);
    for (int k = 0; k < lmax; k += 4) {
        int j[2][4];
        Acc a[2][4];
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const bool ok = k + u < len[h];
                const int p = off[h] + lane + 32 * (k + u);
                j[h][u] = ok ? __ldg(L.idx + p) : 0;
                a[h][u] = ok ? Acc(__ldg(L.val + p)) : Acc(0);
            }
        // in the two-point FP64 passes (the checks), steps past a slice's length
        // (warp-uniform) add zeros: skip their gathers and products (half the FP64
        // pipe time of a check on 2-nonzero slices); the sums are unchanged.  The
        // one-point passes keep the straight-line form (their register budget).
        if (NV < 2 || (k + 4 <= len[0] && k + 4 <= len[1])) {
#pragma unroll
            for (int h = 0; h < 2; ++h)
#pragma unroll
                for (int u = 0; u < 4; ++u)
#pragma unroll
                    for (int q = 0; q < NV; ++q) acc[h][q] += a[h][u] * g(q, j[h][u]);
        } else {
#pragma unroll
            for (int h = 0; h < 2; ++h)
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (k + u < len[h])
#pragma unroll
                        for (int q = 0; q < NV; ++q) acc[h][q] += a[h][u] * g(q, j[h][u]);
        }
    }
    if (r[0] < b.end) e(r[0], b.kind, acc[0], pre[0]);
    if (has1 && r[1] < b.end) e(r[1], b.kind, acc[1], pre[1]);
}

// SLICED bin whose rows all have LEN nonzeros (slice offsets computed
// from the bin's start): exactly LEN steps, no predicated or padding work —
// the generic loop above runs four steps per iteration and gathers for the
// padded ones too (half the gathers of 2-nonzero columns).  The same additions
// in the same order as the generic loop (its padded steps add zeros).
template <int NV, int LEN, class Acc, class V, class Gather, class Epi>
__device__ __forceinline__ void visit_slice_pair_fixed(const Bin& b, int s0, int s1, const Layout<V>& L,
                                                       const Gather& g, Epi& e) {
    const int lane = threadIdx.x & 31;
    const bool has1 = s1 < b.units;
    const int S[2] = {s0, has1 ? s1 : s0};
    int r[2];
    typename Epi::Pre pre[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        r[h] = b.begin + S[h] * 32 + lane;
        if (r[h] < b.end && (h == 0 || has1)) pre[h] = e.pre(r[h]);
    }
    int j[2][LEN];
    Acc a[2][LEN];
#pragma unroll
    for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int u = 0; u < LEN; ++u) {
            const int p = b.slice0 + S[h] * 32 * LEN + lane + 32 * u;
            const bool ok = h == 0 || has1;                   // warp-uniform
            j[h][u] = ok ? __ldg(L.idx + p) : 0;
            a[h][u] = ok ? Acc(__ldg(L.val + p)) : Acc(0);
        }
    Acc acc[2][NV];
#pragma unroll
    for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int q = 0; q < NV; ++q) acc[h][q] = Acc(0);
#pragma unroll
    for (int h = 0; h < 2; ++h)
        if (h == 0 || has1)
#pragma unroll
            for (int u = 0; u < LEN; ++u)
#pragma unroll
                for (int q = 0; q < NV; ++q) acc[h][q] += a[h][u] * g(q, j[h][u]);
    if (r[0] < b.end) e(r[0], b.kind, acc[0], pre[0]);
    if (has1 && r[1] < b.end) e(r[1], b.kind, acc[1], pre[1]);
}

// Dot products of nonzeros [s, t) with the warp (lane-strided, predicated).
template <int NV, class Acc, class V, class Gather>
__device__ __forceinline__ void warp_dot(int s, int t, const Layout<V>& L, const Gather& g, Acc (&acc)[NV]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int q = 0; q < NV; ++q) acc[q] = Acc(0);
    for (int k = s + lane; k < t; k += 32 * kUnroll) {
        int j[kUnroll];
        Acc a[kUnroll];
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
            const int kk = k + 32 * u;
            const bool ok = kk < t;
            j[u] = ok ? __ldg(L.idx + kk) : 0;
            a[u] = ok ? Acc(__ldg(L.val + kk)) : Acc(0);
        }
#pragma unroll
        for (int u = 0; u < kUnroll; ++u)
#pragma unroll
            for (int q = 0; q < NV; ++q) acc[q] += a[u] * g(q, j[u]);
    }
#pragma unroll
    for (int q = 0; q < NV; ++q) acc[q] = group_sum<32>(acc[q]);
}

// Dot products of two nonzero ranges [s0, t0) and [s1, t1) with the warp, their
// loads interleaved so both ranges' requests are in flight together.
template <int NV, class Acc, class V, class Gather>
__device__ __forceinline__ void warp_dot2(int s0, int t0, int s1, int t1, const Layout<V>& L, const Gather& g,
                                          Acc (&acc)[2][NV]) {
    constexpr int U = kUnroll / 2;
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int q = 0; q < NV; ++q) acc[h][q] = Acc(0);
    const int n0 = t0 - s0, n1 = t1 - s1, nmax = max(n0, n1);
    // software-pipelined like the SLAB loop: the next group's indices load with
    // this group's values and gathers
    int jn[2][U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
        const int kk = lane + 32 * u;
        jn[0][u] = kk < n0 ? __ldg(L.idx + s0 + kk) : 0;
        jn[1][u] = kk < n1 ? __ldg(L.idx + s1 + kk) : 0;
    }
    for (int k = lane; k < nmax; k += 32 * U) {
        int j[2][U];
        Acc a[2][U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int kk = k + 32 * u;
            j[0][u] = jn[0][u];
            j[1][u] = jn[1][u];
            a[0][u] = kk < n0 ? Acc(__ldg(L.val + s0 + kk)) : Acc(0);
            a[1][u] = kk < n1 ? Acc(__ldg(L.val + s1 + kk)) : Acc(0);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int kn = k + 32 * (U + u);
            jn[0][u] = kn < n0 ? __ldg(L.idx + s0 + kn) : 0;
            jn[1][u] = kn < n1 ? __ldg(L.idx + s1 + kn) : 0;
        }
#pragma unroll
        for (int h = 0; h < 2; ++h)
#pragma unroll
            for (int u = 0; u < U; ++u)
#pragma unroll
                for (int q = 0; q < NV; ++q) acc[h][q] += a[h][u] * g(q, j[h][u]);
    }
#pragma unroll
    for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int q = 0; q < NV; ++q) acc[h][q] = group_sum<32>(acc[h][q]);
}

// WARP: rows u0 and u1 of the bin (u1 may be past the bin: then it is skipped).
template <int NV, class Acc, class V, class Gather, class Epi>
__device__ __forceinline__ void visit_warp_row_pair(const Bin& b, int u0, int u1, const Layout<V>& L,
                                                    const Gather& g, Epi& e) {
    const bool has1 = u1 < b.units;
    const int r0 = b.begin + u0, r1 = b.begin + (has1 ? u1 : u0);
    const bool lead = (threadIdx.x & 31) == 0;
    typename Epi::Pre pre0, pre1;
    if (lead) {
        pre0 = e.pre(r0);
        if (has1) pre1 = e.pre(r1);
    }
    const int s0 = __ldg(L.ptr + r0), t0 = __ldg(L.ptr + r0 + 1);
    const int s1 = __ldg(L.ptr + r1), t1 = has1 ? __ldg(L.ptr + r1 + 1) : s1;
    Acc acc[2][NV];
    warp_dot2<NV, Acc>(s0, t0, s1, t1, L, g, acc);
    if (lead) {
        e(r0, b.kind, acc[0], pre0);
        if (has1) e(r1, b.kind, acc[1], pre1);
    }
}

// SEGMENT: the dot products of segments u0 and u1 (u1 may be past the bin),
// then each segment's share of its row.
template <int NV, class Acc, class V, class Epi>
__device__ __forceinline__ void finish_segment(const Bin& b, int gseg, int r, int kseg, int nseg,
                                               const Acc (&acc)[NV], const Layout<V>& L, Epi& e);

template <int NV, class Acc, class V, class Gather, class Epi>
__device__ __forceinline__ void visit_segment_pair(const Bin& b, int u0, int u1, const Layout<V>& L,
                                                   const Gather& g, Epi& e) {
    const bool has1 = u1 < b.units;
    const int gs0 = b.aux + u0, gs1 = b.aux + (has1 ? u1 : u0);
    const int4 a0 = __ldg(L.unit + 2 * gs0), a1 = __ldg(L.unit + 2 * gs1);
    const int k0 = __ldg(&L.unit[2 * gs0 + 1].x), k1 = __ldg(&L.unit[2 * gs1 + 1].x);
    Acc acc[2][NV];
    warp_dot2<NV, Acc>(a0.x, a0.y, a1.x, has1 ? a1.y : a1.x, L, g, acc);
    if ((threadIdx.x & 31) != 0) return;
    finish_segment<NV, Acc>(b, gs0, a0.z, k0, a0.w, acc[0], L, e);
    if (has1) finish_segment<NV, Acc>(b, gs1, a1.z, k1, a1.w, acc[1], L, e);
}

// One lane: publish a segment's partial; the row's last segment adds them all.
template <int NV, class Acc, class V, class Epi>
__device__ __forceinline__ void finish_segment(const Bin& b, int gseg, int r, int kseg, int nseg,
                                               const Acc (&acc)[NV], const Layout<V>& L, Epi& e) {
    Acc* part = reinterpret_cast<Acc*>(L.seg_part);
#pragma unroll
    for (int q = 0; q < NV; ++q) part[(size_t)gseg * NV + q] = acc[q];
    uint32_t* tk = L.seg_ticket + b.aux2 + (r - b.begin);
    if (ticket_release(tk) != (uint32_t)(nseg - 1)) return;
    if (b.part0) ticket_acquire(tk);
    else ticket_acquire_fence();
    *tk = 0u;
    typename Epi::Pre pre = e.pre(r);
    const int first = gseg - kseg;
    Acc tot[NV];
#pragma unroll
    for (int q = 0; q < NV; ++q) tot[q] = Acc(0);
    // the row's segment partials, finish_batch loads in flight, added in order
    constexpr int FB = finish_batch<NV, Acc>();
    for (int s0 = 0; s0 < nseg; s0 += FB) {
        Acc v[FB][NV];
#pragma unroll
        for (int w = 0; w < FB; ++w)
#pragma unroll
            for (int q = 0; q < NV; ++q)
                v[w][q] = s0 + w < nseg ? __ldcg(part + (size_t)(first + s0 + w) * NV + q) : Acc(0);
#pragma unroll
        for (int w = 0; w < FB; ++w)
#pragma unroll
            for (int q = 0; q < NV; ++q) tot[q] += v[w][q];
    }
    if constexpr (Epi::NP == 0) {
        e(r, b.kind, tot, pre);
    } else {
        using R = typename Epi::R;
        // Which warp finishes a row last varies between runs: the row's share of
        // the kernel's reductions goes to its own slot, summed in row order by
        // the kernel's last block, so every run adds the same numbers in the same order.
        Epi one = e;
        one.zero();
        one(r, b.kind, tot, pre);
        one.export_to(reinterpret_cast<R*>(L.seg_rowpart) + (size_t)(b.slot0 + (r - b.begin)) * Epi::NP);
    }
}

// In a kernel's last block: add the SEGMENT and SLAB rows' epilogue partials, in
// slot order.
template <int NP, class T, class V>
__device__ __forceinline__ void add_segment_rows(T (&tot)[NP], const Layout<V>& L, T* smem) {
    if (L.nsegrows == 0) {     // (block-uniform) the block sum of no slots is +0: add that alone
        if (threadIdx.x == 0)
#pragma unroll
            for (int p = 0; p < NP; ++p) tot[p] += T(0);
        return;
    }
    // B rows' loads are issued before their adds: B round trips overlap instead
    // of one L2 round trip per row (fixed order, so the sum stays deterministic)
    constexpr int B = NP <= 2 ? 8 : 2;
    const T* part = reinterpret_cast<const T*>(L.seg_rowpart);
    T s[NP];
#pragma unroll
    for (int p = 0; p < NP; ++p) s[p] = T(0);
    for (int k0 = threadIdx.x; k0 < L.nsegrows; k0 += kBlock * B) {
        T v[B][NP];
#pragma unroll
        for (int u = 0; u < B; ++u) {
            const int k = k0 + u * kBlock;
#pragma unroll
            for (int p = 0; p < NP; ++p) v[u][p] = k < L.nsegrows ? __ldcg(part + (size_t)k * NP + p) : T(0);
        }
#pragma unroll
        for (int u = 0; u < B; ++u)
#pragma unroll
            for (int p = 0; p < NP; ++p) s[p] += v[u][p];
    }
    block_sum<NP>(s, smem);
    if (threadIdx.x == 0)
#pragma unroll
        for (int p = 0; p < NP; ++p) tot[p] += s[p];
}

// In a kernel's last block: gather_partials followed by add_segment_rows, with
// the first round of both's loads issued together (one L2 round trip fewer on
// the serial tail of the pass); the same additions in the same order.  smem
// holds kWarps * 2 * NP values.
template <int NP, class T, class V>
__device__ __forceinline__ void gather_all_partials(T (&tot)[NP], const T* partials, int nblk,
                                                    const Layout<V>& L, T* smem) {
    constexpr int B = 4;                       // as gather_partials
    constexpr int BS = NP <= 2 ? 8 : 2;        // as add_segment_rows
    const T* part = reinterpret_cast<const T*>(L.seg_rowpart);
    T sv[BS][NP], bv[B][NP];
#pragma unroll
    for (int u = 0; u < BS; ++u) {
        const int k = threadIdx.x + u * kBlock;
#pragma unroll
        for (int p = 0; p < NP; ++p) sv[u][p] = k < L.nsegrows ? __ldcg(part + (size_t)k * NP + p) : T(0);
    }
#pragma unroll
    for (int u = 0; u < B; ++u) {
        const int b = threadIdx.x + u * kBlock;
#pragma unroll
        for (int p = 0; p < NP; ++p) bv[u][p] = b < nblk ? __ldcg(partials + (size_t)b * NP + p) : T(0);
    }
#pragma unroll
    for (int p = 0; p < NP; ++p) tot[p] = T(0);
#pragma unroll
    for (int u = 0; u < B; ++u)
#pragma unroll
        for (int p = 0; p < NP; ++p) tot[p] += bv[u][p];
    for (int b0 = threadIdx.x + kBlock * B; b0 < nblk; b0 += kBlock * B) {
        T v[B][NP];
#pragma unroll
        for (int u = 0; u < B; ++u) {
            const int b = b0 + u * kBlock;
#pragma unroll
            for (int p = 0; p < NP; ++p) v[u][p] = b < nblk ? __ldcg(partials + (size_t)b * NP + p) : T(0);
        }
#pragma unroll
        for (int u = 0; u < B; ++u)
#pragma unroll
            for (int p = 0; p < NP; ++p) tot[p] += v[u][p];
    }
    if (L.nsegrows == 0) {     // (block-uniform) as add_segment_rows: the slots' block sum is +0
        block_sum<NP>(tot, smem);
        if (threadIdx.x == 0)
#pragma unroll
            for (int p = 0; p < NP; ++p) tot[p] += T(0);
        return;
    }
    T sacc[NP];
#pragma unroll
    for (int p = 0; p < NP; ++p) sacc[p] = T(0);
#pragma unroll
    for (int u = 0; u < BS; ++u)
#pragma unroll
        for (int p = 0; p < NP; ++p) sacc[p] += sv[u][p];
    for (int k0 = threadIdx.x + kBlock * BS; k0 < L.nsegrows; k0 += kBlock * BS) {
        T v[BS][NP];
#pragma unroll
        for (int u = 0; u < BS; ++u) {
            const int k = k0 + u * kBlock;
#pragma unroll
            for (int p = 0; p < NP; ++p) v[u][p] = k < L.nsegrows ? __ldcg(part + (size_t)k * NP + p) : T(0);
        }
#pragma unroll
        for (int u = 0; u < BS; ++u)
#pragma unroll
            for (int p = 0; p < NP; ++p) sacc[p] += v[u][p];
    }
    // both block sums in one reduction (every value has its own fixed tree, so
    // these are the same sums as two reductions; one round of barriers fewer)
    T both[2 * NP];
#pragma unroll
    for (int p = 0; p < NP; ++p) {
        both[p] = tot[p];
        both[NP + p] = sacc[p];
    }
    block_sum<2 * NP>(both, smem);
    if (threadIdx.x == 0)
#pragma unroll
        for (int p = 0; p < NP; ++p) tot[p] = both[p] + both[NP + p];
}

// SLAB: unit u of the bin = steps [c S, min(L, (c+1) S)) of slice s (S =
// kSlabSteps, L = the slice's padded length); lane t accumulates row t of the
// slice.  A slice with more than one unit is finished by the unit that takes
// the slice's ticket last: it adds the units' partials in unit order.  The
// slice's epilogue partials go to the slice's own slot (units finish in
// varying order, slots are summed in order by the kernel's last block).
template <int NV, class Acc, class V, class Gather, class Epi>
__device__ __forceinline__ void visit_slab_unit(const Bin& b, int u, const Layout<V>& L, const Gather& g, Epi& e) {
    const int lane = threadIdx.x & 31;
    const int4 d = __ldg(L.unit + 2 * (b.aux + u));
    const int off = d.x, len = d.y, s = d.z, c = d.w;
    const int k0 = c * kSlabSteps, k1 = min(len, k0 + kSlabSteps);
    const int r = b.begin + 32 * s + lane;
    // the row's epilogue operands, loaded with the unit's entries (the slice's
    // last unit to finish uses them)
    typename Epi::Pre pre;
    if (r < b.end) pre = e.pre(r);
    Acc acc[NV];
#pragma unroll
    for (int q = 0; q < NV; ++q) acc[q] = Acc(0);
    // software-pipelined: the next step group's indices are loaded with this
    // group's values and gathers, so the index -> gather chain costs one round
    // trip per group instead of two
    int jn[kUnroll];
#pragma unroll
    for (int w = 0; w < kUnroll; ++w) jn[w] = k0 + w < k1 ? __ldg(L.idx + off + 32 * (k0 + w) + lane) : 0;
    for (int k = k0; k < k1; k += kUnroll) {
        int j[kUnroll];
        Acc a[kUnroll];
#pragma unroll
        for (int w = 0; w < kUnroll; ++w) {
            j[w] = jn[w];
            a[w] = k + w < k1 ? Acc(__ldg(L.val + off + 32 * (k + w) + lane)) : Acc(0);
        }
#pragma unroll
        for (int w = 0; w < kUnroll; ++w) {
            const int kn = k + kUnroll + w;
            jn[w] = kn < k1 ? __ldg(L.idx + off + 32 * kn + lane) : 0;
        }
#pragma unroll
        for (int w = 0; w < kUnroll; ++w)
#pragma unroll
            for (int q = 0; q < NV; ++q) acc[q] += a[w] * g(q, j[w]);
    }
    const int nunits = (len + kSlabSteps - 1) / kSlabSteps;
    if (nunits > 1) {
        Acc* part = reinterpret_cast<Acc*>(L.slab_part) + (size_t)(b.part0 + u) * 32 * NV;
#pragma unroll
        for (int q = 0; q < NV; ++q) part[lane * NV + q] = acc[q];
        __syncwarp();                      // the lanes' partials, released by lane 0's increment
        uint32_t t = 0;
        uint32_t* tk = L.seg_ticket + b.aux2 + s;
        if (lane == 0) t = ticket_release(tk);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t != (uint32_t)(nunits - 1)) return;
        if (lane == 0) {
            ticket_acquire(tk);
            *tk = 0u;
        }
        __syncwarp();                      // lane 0's acquire, for the other lanes' reads
        const Acc* first = reinterpret_cast<const Acc*>(L.slab_part) + (size_t)(b.part0 + u - c) * 32 * NV;
#pragma unroll
        for (int q = 0; q < NV; ++q) acc[q] = Acc(0);
        // the slice's unit partials, finish_batch loads in flight, added in unit order
        constexpr int FB = finish_batch<NV, Acc>();
        for (int w0 = 0; w0 < nunits; w0 += FB) {
            Acc v[FB][NV];
#pragma unroll
            for (int w = 0; w < FB; ++w)
#pragma unroll
                for (int q = 0; q < NV; ++q)
                    v[w][q] = w0 + w < nunits ? __ldcg(first + (size_t)(w0 + w) * 32 * NV + lane * NV + q) : Acc(0);
#pragma unroll
            for (int w = 0; w < FB; ++w)
#pragma unroll
                for (int q = 0; q < NV; ++q) acc[q] += v[w][q];
        }
    }
    if constexpr (Epi::NP == 0) {
        if (r < b.end) e(r, b.kind, acc, pre);
    } else {
        // the slice's 32 rows' epilogue partials, added over the warp in a fixed
        // butterfly order (lanes past the bin add zeros): one slot per slice
        using R = typename Epi::R;
        Epi one = e;
        one.zero();
        if (r < b.end) one(r, b.kind, acc, pre);
        R v[Epi::NP];
        one.export_to(v);
#pragma unroll
        for (int q = 0; q < Epi::NP; ++q) v[q] = group_sum<32>(v[q]);
        if (lane == 0) {
            R* slot = reinterpret_cast<R*>(L.seg_rowpart) + (size_t)(b.slot0 + s) * Epi::NP;
#pragma unroll
            for (int q = 0; q < Epi::NP; ++q) slot[q] = v[q];
        }
    }
}

// Dispatch: find this block's bin; each warp walks the bin's units with a
// grid stride.
template <int NV, class Acc, class V, class Gather, class Epi>
__device__ __forceinline__ void visit_bins(const BinTable& bt, int block, const Layout<V>& L,
                                           const Gather& g, Epi& e) {
    int bi = -1;
#pragma unroll
    for (int i = 0; i < kMaxBins; ++i)
        if (i < bt.nbins && block >= bt.bin[i].block_begin && block < bt.bin[i].block_begin + bt.bin[i].nblocks)
            bi = i;
    if (bi < 0) return;
    const Bin& b = bt.bin[bi];
    const int stride = b.nblocks * kWarps;
    const int w0 = (block - b.block_begin) * kWarps + (threadIdx.x >> 5);
    if (b.mode == BM_SLICED) {
        // rows of one or two nonzeros each (the columns of transportation and assignment
        // LPs): the exact-length loop (FP32 iterates; in the FP64 engine its extra code
        // spills at the step kernels' register budget)
        switch (sizeof(V) == 4 ? b.part0 : 0) {
        case 1:
            for (int u = w0; u < b.units; u += 2 * stride) visit_slice_pair_fixed<NV, 1, Acc>(b, u, u + stride, L, g, e);
            break;
        case 2:
            for (int u = w0; u < b.units; u += 2 * stride) visit_slice_pair_fixed<NV, 2, Acc>(b, u, u + stride, L, g, e);
            break;
        default:
            for (int u = w0; u < b.units; u += 2 * stride) visit_slice_pair<NV, Acc>(b, u, u + stride, L, g, e);
        }
    } else if (b.mode == BM_WARP) {
        for (int u = w0; u < b.units; u += 2 * stride) visit_warp_row_pair<NV, Acc>(b, u, u + stride, L, g, e);
    } else if (b.mode == BM_SEGMENT) {
        for (int u = w0; u < b.units; u += 2 * stride) visit_segment_pair<NV, Acc>(b, u, u + stride, L, g, e);
    } else {
        for (int u = w0; u < b.units; u += stride) visit_slab_unit<NV, Acc>(b, u, L, g, e);
    }
}

// Epilogue helper with nothing to prefetch.
struct NoPre {};

// ---- programmatic dependent launch of the iteration kernels ------------------
// A pass kernel is launched as the programmatic dependent of the one before it:
// its blocks may start while the previous pass's last blocks (and its serial
// tail) still run.  Before griddepcontrol.wait they only touch what the
// previous pass does not write (the matrix entries and the vectors of the
// warp's first unit, both state buffers where the pass picks one by the
// decision), so the first unit's loads hit L1 after the wait; every read that
// depends on the previous pass comes after it.
__device__ __forceinline__ void prefetch_l1(const void* p) { asm volatile("prefetch.global.L1 [%0];" ::"l"(p)); }
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void grid_dep_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// The entries of the warp's first unit in the bins of `block` (the units
// visit_bins gives it first), and touch(r) for the rows they finish.
template <class V, class Touch>
__device__ __forceinline__ void prefetch_first_unit(const BinTable& bt, int block, const Layout<V>& L,
                                                    const Touch& touch) {
    int bi = -1;
#pragma unroll
    for (int i = 0; i < kMaxBins; ++i)
        if (i < bt.nbins && block >= bt.bin[i].block_begin && block < bt.bin[i].block_begin + bt.bin[i].nblocks)
            bi = i;
    if (bi < 0) return;
    const Bin& b = bt.bin[bi];
    const int w0 = (block - b.block_begin) * kWarps + (threadIdx.x >> 5);
    if (w0 >= b.units) return;
    const int lane = threadIdx.x & 31;
    // (the first slice or unit and its first two steps only: with more, the touched
    // lines of five resident blocks outgrew L1 on LPs with longer columns)
    if (b.mode == BM_SLICED) {
        const int s = w0;
        int off, len;
        if (b.part0 > 0) {
            off = b.slice0 + s * 32 * b.part0;
            len = b.part0;
        } else {
            off = __ldg(L.soff + b.aux + s);
            len = (__ldg(L.soff + b.aux + s + 1) - off) >> 5;
        }
        for (int u = 0; u < len && u < 2; ++u) {
            prefetch_l1(L.idx + off + 32 * u + lane);
            prefetch_l1(L.val + off + 32 * u + lane);
        }
        const int r = b.begin + s * 32 + lane;
        if (r < b.end) touch(r);
    } else if (b.mode == BM_SLAB) {
        const int4 d = __ldg(L.unit + 2 * (b.aux + w0));
        const int k0 = d.w * kSlabSteps, k1 = min(d.y, k0 + kSlabSteps);
        for (int k = k0; k < k1 && k < k0 + 2; ++k) {
            prefetch_l1(L.idx + d.x + 32 * k + lane);
            prefetch_l1(L.val + d.x + 32 * k + lane);
        }
        const int r = b.begin + 32 * d.z + lane;
        if (r < b.end) touch(r);
    } else {
        int s0, t0, r = -1;
        if (b.mode == BM_WARP) {
            r = b.begin + w0;
            s0 = __ldg(L.ptr + r);
            t0 = __ldg(L.ptr + r + 1);
        } else {                                   // SEGMENT
            const int4 a0 = __ldg(L.unit + 2 * (b.aux + w0));
            s0 = a0.x;
            t0 = a0.y;
        }
        for (int k = s0 + lane; k < t0 && k < s0 + 64; k += 32) {
            prefetch_l1(L.idx + k);
            prefetch_l1(L.val + k);
        }
        if (r >= 0 && lane == 0) touch(r);
    }
}

}  // namespace sps
