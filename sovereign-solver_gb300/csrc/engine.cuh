// engine.cuh — device data layout and shared device helpers of the PDHG engine.
//
// Layout in HBM (all indices internal):
//   rows are renumbered so that each row bin (row type x length class) is one
//   contiguous range; columns are renumbered by column length class.  The
//   matrix is stored twice, as CSR (row pass: K x) and CSC (column pass: K^T y),
//   each as int32 offsets, int32 indices and V values (V = float or double).
//   Vectors are V arrays in internal order; scale factors and every reduction
//   are FP64.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace sps {

constexpr int kBlock = 256;          // threads per block of every pass kernel
constexpr int kWarps = kBlock / 32;
constexpr int kMaxBins = 16;

// One contiguous range of internal rows (or columns) with one schedule.
struct Bin {
    int32_t begin, end;      // [begin, end)
    int32_t lanes;           // 1,2,4,8,16,32 lanes per row, or 0 = whole block per row
    int32_t kind;            // row pass: 1 = '<=' rows, 0 = '=' rows; column pass: 0
    int32_t block_begin;     // first block of this bin in the launch
    int32_t nblocks;
};

struct BinTable {
    int32_t nbins;
    int32_t total_blocks;
    Bin bin[kMaxBins];
};

template <class V>
struct Compressed {          // CSR (ptr over rows) or CSC (ptr over columns)
    const int32_t* ptr;
    const int32_t* idx;
    const V* val;
};

// Control block, one per handle, in device memory.  Written only by single
// threads of "last blocks" or by block 0 thread 0, read by every kernel.
struct Ctl {
    int32_t done;            // 1 -> every iteration kernel returns at entry
    int32_t status;          // SPS_STATUS_* once done
    int32_t cur;             // adaptive: index of the accepted state buffers
    int32_t accepted;        // adaptive: last attempt accepted
    int32_t apply;           // pending action for the apply kernel (bit 0: load average, bit 1: reset window)
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

// Sum NP doubles over the block; result valid in thread 0.  Fixed order.
template <int NP>
__device__ __forceinline__ void block_sum(double (&v)[NP], double* smem /* kWarps*NP */) {
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
            double s = 0.0;
            for (int q = 0; q < kWarps; ++q) s += smem[q * NP + p];
            v[p] = s;
        }
    }
    __syncthreads();
}

// Write this block's NP partials, then report whether this block is the last
// one of the grid to finish (ticket counter; no waiting).
template <int NP>
__device__ __forceinline__ bool publish_partials(double (&v)[NP], double* partials, uint32_t* ticket,
                                                 double* smem, bool* am_last) {
    block_sum<NP>(v, smem);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int p = 0; p < NP; ++p) partials[(size_t)blockIdx.x * NP + p] = v[p];
        __threadfence();
        const uint32_t t = atomicAdd(ticket, 1u);
        *am_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    return *am_last;
}

// In the last block: sum the partials of all nblk blocks (fixed order).
template <int NP>
__device__ __forceinline__ void gather_partials(double (&tot)[NP], const double* partials, int nblk,
                                                double* smem) {
    __threadfence();
#pragma unroll
    for (int p = 0; p < NP; ++p) tot[p] = 0.0;
    for (int b = threadIdx.x; b < nblk; b += kBlock) {
#pragma unroll
        for (int p = 0; p < NP; ++p) tot[p] += __ldcg(partials + (size_t)b * NP + p);
    }
    block_sum<NP>(tot, smem);
}

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// ---------------------------------------------------------------------------
// Binned traversal.  The launch's blocks are split among bins; each bin's
// rows are visited with `lanes` lanes per row (lane-strided, coalesced index
// and value streams) or with the whole block per row.  For every row the
// functor gets the NV dot products of the row with NV gathered vectors:
//   g(q, j) -> value of vector q at column j (as Acc)
//   e(r, kind, acc[NV]) is called once per row by exactly one thread.

template <int NV, class Acc>
struct Dots { Acc v[NV]; };

template <int G, int NV, class Acc, class V, class Gather, class Epi>
__device__ __forceinline__ void visit_lanes(const Bin& b, int bib, const Compressed<V>& M,
                                            const Gather& g, Epi& e) {
    constexpr int per_warp = 32 / G;
    const int warp = threadIdx.x >> 5, wl = threadIdx.x & 31, lane = wl & (G - 1);
    const int stride = b.nblocks * kWarps * per_warp;
    for (int base = b.begin + (bib * kWarps + warp) * per_warp; base < b.end; base += stride) {
        const int r = base + wl / G;
        const bool valid = r < b.end;
        const int s = valid ? __ldg(M.ptr + r) : 0;
        const int t = valid ? __ldg(M.ptr + r + 1) : 0;
        Acc acc[NV];
#pragma unroll
        for (int q = 0; q < NV; ++q) acc[q] = Acc(0);
        int k = s + lane;
        for (; k + 3 * G < t; k += 4 * G) {
            int j[4];
            Acc a[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) { j[u] = __ldg(M.idx + k + u * G); a[u] = Acc(__ldg(M.val + k + u * G)); }
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int q = 0; q < NV; ++q) acc[q] += a[u] * g(q, j[u]);
        }
        for (; k < t; k += G) {
            const int j = __ldg(M.idx + k);
            const Acc a = Acc(__ldg(M.val + k));
#pragma unroll
            for (int q = 0; q < NV; ++q) acc[q] += a * g(q, j);
        }
#pragma unroll
        for (int q = 0; q < NV; ++q) acc[q] = group_sum<G>(acc[q]);
        if (valid && lane == 0) e(r, b.kind, acc);
    }
}

template <int NV, class Acc, class V, class Gather, class Epi>
__device__ __forceinline__ void visit_block(const Bin& b, int bib, const Compressed<V>& M,
                                            const Gather& g, Epi& e, Acc* red /* kWarps*NV */) {
    for (int r = b.begin + bib; r < b.end; r += b.nblocks) {
        const int s = __ldg(M.ptr + r), t = __ldg(M.ptr + r + 1);
        Acc acc[NV];
#pragma unroll
        for (int q = 0; q < NV; ++q) acc[q] = Acc(0);
        int k = s + threadIdx.x;
        for (; k + 3 * kBlock < t; k += 4 * kBlock) {
            int j[4];
            Acc a[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) { j[u] = __ldg(M.idx + k + u * kBlock); a[u] = Acc(__ldg(M.val + k + u * kBlock)); }
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int q = 0; q < NV; ++q) acc[q] += a[u] * g(q, j[u]);
        }
        for (; k < t; k += kBlock) {
            const int j = __ldg(M.idx + k);
            const Acc a = Acc(__ldg(M.val + k));
#pragma unroll
            for (int q = 0; q < NV; ++q) acc[q] += a * g(q, j);
        }
#pragma unroll
        for (int q = 0; q < NV; ++q) acc[q] = group_sum<32>(acc[q]);
        const int w = threadIdx.x >> 5;
        if ((threadIdx.x & 31) == 0) {
#pragma unroll
            for (int q = 0; q < NV; ++q) red[w * NV + q] = acc[q];
        }
        __syncthreads();
        if (threadIdx.x == 0) {
#pragma unroll
            for (int q = 0; q < NV; ++q) {
                Acc s2 = Acc(0);
                for (int u = 0; u < kWarps; ++u) s2 += red[u * NV + q];
                acc[q] = s2;
            }
            e(r, b.kind, acc);
        }
        __syncthreads();
    }
}

// Dispatch: find this block's bin and run its schedule.  Returns false if the
// block has no bin (launch grids can be padded).
template <int NV, class Acc, class V, class Gather, class Epi>
__device__ __forceinline__ void visit_bins(const BinTable& bt, int block, const Compressed<V>& M,
                                           const Gather& g, Epi& e, Acc* red) {
    int bi = -1;
    for (int i = 0; i < bt.nbins; ++i)
        if (block >= bt.bin[i].block_begin && block < bt.bin[i].block_begin + bt.bin[i].nblocks) bi = i;
    if (bi < 0) return;
    const Bin& b = bt.bin[bi];
    const int bib = block - b.block_begin;
    switch (b.lanes) {
        case 1:  visit_lanes<1, NV, Acc>(b, bib, M, g, e); break;
        case 2:  visit_lanes<2, NV, Acc>(b, bib, M, g, e); break;
        case 4:  visit_lanes<4, NV, Acc>(b, bib, M, g, e); break;
        case 8:  visit_lanes<8, NV, Acc>(b, bib, M, g, e); break;
        case 16: visit_lanes<16, NV, Acc>(b, bib, M, g, e); break;
        case 32: visit_lanes<32, NV, Acc>(b, bib, M, g, e); break;
        default: visit_block<NV, Acc>(b, bib, M, g, e, red); break;
    }
}

}  // namespace sps
