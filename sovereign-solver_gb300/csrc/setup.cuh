// setup.cuh — device kernels that build the engine's HBM layout from the
// caller's CSR: validation, column histogram, row/column renumbering,
// CSR -> CSC transpose (counting sort + per-column ordering by row), Ruiz and
// Pock-Chambolle scaling in FP64, conversion to the iterate precision, and the
// start/extract kernels of a solve.
#pragma once

#include "kernels.cuh"

namespace sps {

enum SetupError { SE_INDEX = 1, SE_VALUE = 2 };

// Check column indices and values of the staged (original-order) matrix and
// count nonzeros per column.
static __global__ void k_validate_count(const int32_t* __restrict__ idx, const double* __restrict__ val, int64_t nnz,
                                 int32_t n, int32_t* __restrict__ colcount, int32_t* __restrict__ err) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnz; k += (int64_t)gridDim.x * blockDim.x) {
        const int32_t j = idx[k];
        if (j < 0 || j >= n) { atomicOr(err, SE_INDEX); continue; }
        if (!isfinite(val[k])) atomicOr(err, SE_VALUE);
        atomicAdd(colcount + j, 1);
    }
}

// Internal CSR: internal row r copies original row perm_row[r]; column
// indices are renumbered.  One warp per row.
static __global__ void k_build_csr(const int32_t* __restrict__ optr, const int32_t* __restrict__ oidx,
                            const double* __restrict__ oval, const int32_t* __restrict__ perm_row,
                            const int32_t* __restrict__ inv_col, const int32_t* __restrict__ nptr,
                            int32_t* __restrict__ nidx, double* __restrict__ nval, int32_t m) {
    const int lane = threadIdx.x & 31;
    for (int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < m; r += (gridDim.x * blockDim.x) >> 5) {
        const int o = perm_row[r];
        const int s = optr[o], t = optr[o + 1], d = nptr[r];
        for (int k = s + lane; k < t; k += 32) {
            nidx[d + k - s] = inv_col[oidx[k]];
            nval[d + k - s] = oval[k];
        }
    }
}

// Scatter CSR entries into CSC slots (order inside a column fixed afterwards).
static __global__ void k_scatter_csc(const int32_t* __restrict__ rptr, const int32_t* __restrict__ ridx,
                              const double* __restrict__ rval, const int32_t* __restrict__ cptr,
                              int32_t* __restrict__ fill, int32_t* __restrict__ cidx, double* __restrict__ cval,
                              int32_t m) {
    const int lane = threadIdx.x & 31;
    for (int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < m; r += (gridDim.x * blockDim.x) >> 5) {
        for (int k = rptr[r] + lane; k < rptr[r + 1]; k += 32) {
            const int j = ridx[k];
            const int pos = cptr[j] + atomicAdd(fill + j, 1);
            cidx[pos] = r;
            cval[pos] = rval[k];
        }
    }
}

// Order each column's entries by row index (insertion sort, one thread per
// column) so the CSC, and every sum over it, is the same on every run.
// Columns longer than kSortMax are ordered on the host instead.
constexpr int kSortMax = 64;
static __global__ void k_sort_columns(const int32_t* __restrict__ cptr, int32_t* __restrict__ cidx,
                               double* __restrict__ cval, int32_t n) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const int s = cptr[j], t = cptr[j + 1];
        if (t - s > kSortMax) continue;
        for (int k = s + 1; k < t; ++k) {
            const int r = cidx[k];
            const double v = cval[k];
            int q = k - 1;
            while (q >= s && cidx[q] > r) { cidx[q + 1] = cidx[q]; cval[q + 1] = cval[q]; --q; }
            cidx[q + 1] = r;
            cval[q + 1] = v;
        }
    }
}

// Per-row (or per-column) max |s| and sum |s| of the scaled matrix
// s_ij = d_own[i] * v_ij * d_other[j].  G lanes per row (G = 1..32, chosen
// from the mean row length so short rows do not leave most of a warp idle).
template <int G>
static __global__ void k_abs_stats(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                                   const double* __restrict__ val, const double* __restrict__ d_own,
                                   const double* __restrict__ d_other, double* __restrict__ vmax,
                                   double* __restrict__ vsum, int32_t rows) {
    const int lane = threadIdx.x & (G - 1);
    const int64_t groups = ((int64_t)gridDim.x * blockDim.x) / G;
    for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / G; r < rows; r += groups) {
        double mx = 0.0, sm = 0.0;
        for (int k = ptr[r] + lane; k < ptr[r + 1]; k += G) {
            const double a = fabs(val[k] * d_other[idx[k]]);
            mx = fmax(mx, a);
            sm += a;
        }
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) {
            mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
            sm += __shfl_xor_sync(0xffffffffu, sm, o);
        }
        if (lane == 0) {
            vmax[r] = mx * d_own[r];
            vsum[r] = sm * d_own[r];
        }
    }
}

// Lanes per row for the statistics pass: the power of two at or above the mean
// row length, at most 32.
static inline int stats_lanes(int64_t nnz, int64_t rows) {
    const int64_t avg = rows > 0 ? (nnz + rows - 1) / rows : 1;
    int g = 1;
    while (g < 32 && g < avg) g <<= 1;
    return g;
}

static inline void launch_abs_stats(const int32_t* ptr, const int32_t* idx, const double* val, const double* d_own,
                                    const double* d_other, double* vmax, double* vsum, int32_t rows, int64_t nnz,
                                    int max_blocks, cudaStream_t st) {
    const int g = stats_lanes(nnz, rows);
    const int64_t threads = (int64_t)rows * g;
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((threads + 255) / 256, max_blocks));
    switch (g) {
        case 1: k_abs_stats<1><<<blocks, 256, 0, st>>>(ptr, idx, val, d_own, d_other, vmax, vsum, rows); break;
        case 2: k_abs_stats<2><<<blocks, 256, 0, st>>>(ptr, idx, val, d_own, d_other, vmax, vsum, rows); break;
        case 4: k_abs_stats<4><<<blocks, 256, 0, st>>>(ptr, idx, val, d_own, d_other, vmax, vsum, rows); break;
        case 8: k_abs_stats<8><<<blocks, 256, 0, st>>>(ptr, idx, val, d_own, d_other, vmax, vsum, rows); break;
        case 16: k_abs_stats<16><<<blocks, 256, 0, st>>>(ptr, idx, val, d_own, d_other, vmax, vsum, rows); break;
        default: k_abs_stats<32><<<blocks, 256, 0, st>>>(ptr, idx, val, d_own, d_other, vmax, vsum, rows); break;
    }
}

// d[i] /= sqrt(stat[i]) where stat > 0 (Ruiz: stat = max, Pock-Chambolle: stat = sum).
static __global__ void k_rescale(double* __restrict__ d, const double* __restrict__ stat, int32_t len) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < len; i += gridDim.x * blockDim.x)
        if (stat[i] > 0.0) d[i] /= sqrt(stat[i]);
}

// Final matrix values in the iterate precision: v * d_own[row] * d_other[col].
template <class V>
__global__ void k_finish_values(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                                const double* __restrict__ v64, const double* __restrict__ d_own,
                                const double* __restrict__ d_other, V* __restrict__ out, int32_t rows) {
    const int lane = threadIdx.x & 31;
    for (int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < rows; r += (gridDim.x * blockDim.x) >> 5) {
        const double dr = d_own[r];
        for (int k = ptr[r] + lane; k < ptr[r + 1]; k += 32) out[k] = V(v64[k] * dr * d_other[idx[k]]);
    }
}

// Final layout, SLICED bin: slot (slice, lane) of rows [begin, end) copies its
// row's entries to soff[slice] + 32 k + lane, zero-padding to the slice length.
template <class V>
__global__ void k_fill_sliced(const int32_t* __restrict__ tptr, const int32_t* __restrict__ tidx,
                              const V* __restrict__ tval, const int32_t* __restrict__ soff, int32_t begin,
                              int32_t end, int32_t first_slice, int32_t nslices, int32_t* __restrict__ oidx,
                              V* __restrict__ oval) {
    const int64_t slots = (int64_t)nslices * 32;
    for (int64_t sl = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; sl < slots; sl += (int64_t)gridDim.x * blockDim.x) {
        const int s = (int)(sl >> 5), lane = (int)(sl & 31);
        const int r = begin + (int)sl;
        const int rs = r < end ? tptr[r] : 0;
        const int len = r < end ? tptr[r + 1] - rs : 0;
        const int off = soff[first_slice + s];
        const int L = (soff[first_slice + s + 1] - off) >> 5;
        for (int k = 0; k < L; ++k) {
            oidx[off + 32 * k + lane] = k < len ? tidx[rs + k] : 0;
            oval[off + 32 * k + lane] = k < len ? tval[rs + k] : V(0);
        }
    }
}

// Final layout, WARP / SEGMENT bins: rows [begin, end) copied to their final offsets.
template <class V>
__global__ void k_fill_rows(const int32_t* __restrict__ tptr, const int32_t* __restrict__ tidx,
                            const V* __restrict__ tval, const int32_t* __restrict__ fptr, int32_t begin,
                            int32_t end, int32_t* __restrict__ oidx, V* __restrict__ oval) {
    const int lane = threadIdx.x & 31;
    for (int r = begin + ((blockIdx.x * blockDim.x + threadIdx.x) >> 5); r < end; r += (gridDim.x * blockDim.x) >> 5) {
        const int s = tptr[r], t = tptr[r + 1], d = fptr[r];
        for (int k = s + lane; k < t; k += 32) {
            oidx[d + k - s] = tidx[k];
            oval[d + k - s] = tval[k];
        }
    }
}

// Scaled vectors in internal order from FP64 inputs in the caller's order
// (gathered through the permutations on the device):
//   c~ = c*dc, l~ = l/dc, u~ = u/dc (columns);  b~ = b*dr (rows).
template <class V>
__global__ void k_scale_vectors(const double* __restrict__ c, const double* __restrict__ lb,
                                const double* __restrict__ ub, const double* __restrict__ b,
                                const int32_t* __restrict__ perm_col, const int32_t* __restrict__ perm_row,
                                const double* __restrict__ dc, const double* __restrict__ dr,
                                V* __restrict__ cs, V* __restrict__ los, V* __restrict__ his,
                                V* __restrict__ bs, int32_t n, int32_t m) {
    const int stride = gridDim.x * blockDim.x;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride) {
        const int o = perm_col[j];
        cs[j] = V(c[o] * dc[j]);
        if (los) {
            los[j] = V(lb[o] / dc[j]);
            his[j] = V(ub[o] / dc[j]);
        }
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride) bs[i] = V(b[perm_row[i]] * dr[i]);
}

// Reciprocal scale factors (FP64) for the adaptive checks, which multiply by them.
__global__ static void k_reciprocals(const double* __restrict__ dc, const double* __restrict__ dr,
                                     double* __restrict__ idc, double* __restrict__ idr, int32_t n, int32_t m) {
    const int stride = gridDim.x * blockDim.x;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride) idc[j] = 1.0 / dc[j];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride) idr[i] = 1.0 / dr[i];
}

// Reference diagonal steps (solver/lp/pdhg.py:139-147): 0.999 / max(sum|a|, 1e-4).
template <class V>
__global__ void k_diag_steps(const double* __restrict__ colsum, const double* __restrict__ rowsum,
                             V* __restrict__ tau, V* __restrict__ sigma, int32_t n, int32_t m) {
    const int stride = gridDim.x * blockDim.x;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride) tau[j] = V(0.999 / fmax(colsum[j], 1e-4));
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride) sigma[i] = V(0.999 / fmax(rowsum[i], 1e-4));
}

// FP64 sums over the scaled problem for the start-up constants:
//   out[0] = max |K~|, out[1] = ||c~||^2, out[2] = ||b~||^2.
template <class V>
__global__ void k_norms(const V* __restrict__ kval, int64_t nnz, const V* __restrict__ cs, int32_t n,
                        const V* __restrict__ bs, int32_t m, double* __restrict__ out /* 3 per block */) {
    double mx = 0.0, sc = 0.0, sb = 0.0;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnz; k += stride) mx = fmax(mx, fabs(double(kval[k])));
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += stride) sc += double(cs[j]) * double(cs[j]);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += stride) sb += double(bs[i]) * double(bs[i]);
    for (int o = 16; o > 0; o >>= 1) {
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        sc += __shfl_xor_sync(0xffffffffu, sc, o);
        sb += __shfl_xor_sync(0xffffffffu, sb, o);
    }
    __shared__ double s[3][32];
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) { s[0][w] = mx; s[1][w] = sc; s[2][w] = sb; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 1; q < (int)(blockDim.x >> 5); ++q) { mx = fmax(mx, s[0][q]); sc += s[1][q]; sb += s[2][q]; }
        out[blockIdx.x * 3 + 0] = mx;
        out[blockIdx.x * 3 + 1] = sc;
        out[blockIdx.x * 3 + 2] = sb;
    }
}

// Start of an adaptive solve: x0 = proj(warm x / dc), y0 = proj(warm y / dr),
// sums zero, last-restart point = start point, device deadline.
template <class V>
__global__ void k_ad_start(Args<V> a, const double* __restrict__ wx, const double* __restrict__ wy,
                           const int32_t* __restrict__ perm_col, const int32_t* __restrict__ perm_row,
                           const int8_t* __restrict__ rkind, uint64_t time_limit_ns) {
    const int stride = gridDim.x * blockDim.x;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < a.n; j += stride) {
        const double x0 = wx ? wx[perm_col[j]] / a.dc[j] : 0.0;
        const V xv = clampv(V(x0), lo_at(a, j), hi_at(a, j));
        a.X[0][j] = xv;
        a.xl[j] = xv;
        a.xs[j] = V(0);
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.m; i += stride) {
        double y0 = wy ? wy[perm_row[i]] / a.dr[i] : 0.0;
        if (rkind[i]) y0 = fmin(y0, 0.0);
        a.Y[0][i] = V(y0);
        a.yl[i] = V(y0);
        a.ys[i] = V(0);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0)
        a.ctl->deadline_ns = time_limit_ns ? global_ns() + time_limit_ns : 0;
}

template <class V>
__global__ void k_rf_start(Args<V> a, uint64_t time_limit_ns) {
    const int stride = gridDim.x * blockDim.x;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < a.n; j += stride) { a.X[0][j] = V(0); a.xs[j] = V(0); }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.m; i += stride) { a.Y[0][i] = V(0); a.ys[i] = V(0); }
    if (blockIdx.x == 0 && threadIdx.x == 0)
        a.ctl->deadline_ns = time_limit_ns ? global_ns() + time_limit_ns : 0;
}

// Returned point in the device problem's original numbering, unscaled, FP64.
template <class V>
__global__ void k_extract(const V* __restrict__ x, const V* __restrict__ y, const double* __restrict__ dc,
                          const double* __restrict__ dr, const int32_t* __restrict__ perm_col,
                          const int32_t* __restrict__ perm_row, double* __restrict__ xo,
                          double* __restrict__ yo, int32_t n, int32_t m) {
    const int stride = gridDim.x * blockDim.x;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride) xo[perm_col[j]] = double(x[j]) * dc[j];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride) yo[perm_row[i]] = double(y[i]) * dr[i];
}

// Adaptive mode's solution in the caller's space, on the device: x in the
// caller's column order, unscaled and clipped to the caller's bounds (as
// FP64 arrays, or the uniform scalars lo_u / hi_u when lb and ub are null;
// infinite bounds clip at +-1e30), y unscaled in the caller's row order, and
// c^T x: per-block partials in part, summed in block order by the last block
// (ticket) into *obj.
template <class V>
__global__ void k_extract_user(const V* __restrict__ x, const V* __restrict__ y, const double* __restrict__ dc,
                               const double* __restrict__ dr, const int32_t* __restrict__ perm_col,
                               const int32_t* __restrict__ perm_row, const double* __restrict__ c,
                               const double* __restrict__ lb, const double* __restrict__ ub, double lo_u,
                               double hi_u, double* __restrict__ xo, double* __restrict__ yo, int32_t n, int32_t m,
                               double* __restrict__ part, uint32_t* ticket, double* obj) {
    __shared__ double sm[256 / 32];
    __shared__ bool last;
    const int stride = gridDim.x * blockDim.x;
    double acc = 0.0;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride) {
        const int o = perm_col[j];
        double lo = lb ? lb[o] : lo_u, hi = ub ? ub[o] : hi_u;
        lo = isfinite(lo) ? lo : -1e30;
        hi = isfinite(hi) ? hi : 1e30;
        const double v = fmin(fmax(double(x[j]) * dc[j], lo), hi);
        xo[o] = v;
        acc += c[o] * v;
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride) yo[perm_row[i]] = double(y[i]) * dr[i];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) b += sm[w];
        part[blockIdx.x] = b;
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    __threadfence();
    double t = 0.0;
    for (int b = 0; b < (int)gridDim.x; ++b) t += __ldcg(part + b);
    *obj = t;
    *ticket = 0u;
}

}  // namespace sps
