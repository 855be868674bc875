// kkt_noalloc.cu — relative KKT error of a given point, computed without
// allocating any device memory (sps_kkt_noalloc in include/sps_pdhg.h).
//
// Who needs it: callers that hold the LP and the point in device memory they
// own and cannot call cudaMalloc at that moment — code running inside another
// framework's memory pool or a fixed device-memory budget, and latency-critical
// loops where a cudaMalloc/cudaFree would synchronise the device.  It is the
// same FP64 check that sps_solve runs on its own (allocated) workspace, as a
// variant whose scratch is a file-scope device array.
//
// Scratch: kScratchDoubles doubles in g_noalloc_scratch (about 2.1 MB), held
// by every GPU that loads the library until the process exits:
//   [0, kMaxCols)                          K^T y accumulator (cleared each call)
//   [kMaxCols, + 2 * kMaxBlocks * kParts)  per-block partial sums of the two passes
//   last slot                              ticket of the column pass (cleared each call)
// Limits: n <= kMaxCols (262144) columns; any number of rows.
// Every call shares the array: two calls that overlap on the GPU (different
// streams, or different host threads without ordering) race and return
// garbage; order them on one stream.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "../../include/sps_pdhg.h"

namespace sps {
void set_create_error(const std::string& msg);   // defined in api.cu (message for sps_last_error(NULL))
}

namespace {

constexpr int kThreads = 256;
constexpr int kMaxBlocks = 1024;
constexpr int kParts = 4;
constexpr int kMaxCols = 1 << 18;
constexpr int kPartBase = kMaxCols;
constexpr int kTicketSlot = kMaxCols + 2 * kMaxBlocks * kParts;
constexpr int kScratchDoubles = kTicketSlot + 32;

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

// Device address of g_noalloc_scratch, looked up once per device.
std::mutex g_mu;
double* g_addr[64] = {};

int scratch_address(int dev, double** out) {
    if (dev < 0 || dev >= 64) return SPS_ERR_CUDA;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) {
            cudaGetLastError();
            sps::set_create_error(std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") + cudaGetErrorString(e));
            return SPS_ERR_CUDA;
        }
        g_addr[dev] = static_cast<double*>(p);
    }
    *out = g_addr[dev];
    return SPS_OK;
}

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block sum of kParts values into part[blockIdx.x * kParts + q].
__device__ __forceinline__ void store_block_partials(double (&v)[kParts], double* part) {
    __shared__ double sm[kThreads / 32][kParts];
    for (int q = 0; q < kParts; ++q) v[q] = warp_sum(v[q]);
    if ((threadIdx.x & 31) == 0)
        for (int q = 0; q < kParts; ++q) sm[threadIdx.x >> 5][q] = v[q];
    __syncthreads();
    if (threadIdx.x == 0)
        for (int q = 0; q < kParts; ++q) {
            double s = 0.0;
            for (int w = 0; w < kThreads / 32; ++w) s += sm[w][q];
            part[blockIdx.x * kParts + q] = s;
        }
}

// Row pass, one warp per row: residual of K x against the rhs (<= rows count
// only violations), rhs^T y, ||rhs||^2, sign violations of y on <= rows, and
// the scatter of K^T y into the accumulator.
__global__ void __launch_bounds__(kThreads) na_rows(sps_device_lp lp, const double* __restrict__ x,
                                                     const double* __restrict__ y, double* __restrict__ s) {
    double v[kParts] = {0.0, 0.0, 0.0, 0.0};
    const int m = lp.m_ub + lp.m_eq;
    const int lane = threadIdx.x & 31;
    double* aty = s;
    for (int i = (blockIdx.x * kThreads + threadIdx.x) >> 5; i < m; i += (gridDim.x * kThreads) >> 5) {
        const double yi = y[i];
        double acc = 0.0;
        for (int k = lp.indptr[i] + lane; k < lp.indptr[i + 1]; k += 32) {
            const double a = lp.values[k];
            const int j = lp.indices[k];
            acc += a * x[j];
            atomicAdd(aty + j, a * yi);
        }
        acc = warp_sum(acc);
        if (lane == 0) {
            const double b = lp.rhs[i];
            double res = acc - b;
            double sign = 0.0;
            if (i < lp.m_ub) {
                res = fmax(res, 0.0);
                sign = fmax(yi, 0.0);
            }
            v[0] += res * res;
            v[1] += b * yi;
            v[2] += b * b;
            v[3] += sign * sign;
        }
    }
    store_block_partials(v, s + kPartBase);
}

// Column pass, one thread per column, and the final reduction in the last block.
// out: rel_kkt, rel_primal, rel_dual, rel_gap, primal objective, dual objective.
__global__ void __launch_bounds__(kThreads) na_cols(sps_device_lp lp, const double* __restrict__ x,
                                                     double* __restrict__ s, int row_blocks,
                                                     double* __restrict__ out) {
    double v[kParts] = {0.0, 0.0, 0.0, 0.0};
    const double* aty = s;
    for (int j = blockIdx.x * kThreads + threadIdx.x; j < lp.n; j += gridDim.x * kThreads) {
        const double cj = lp.c[j], lo = lp.lb[j], hi = lp.ub[j];
        const bool hl = isfinite(lo), hh = isfinite(hi);
        const double r = cj - aty[j];
        const double lam = (hl && hh) ? r : hl ? fmax(r, 0.0) : hh ? fmin(r, 0.0) : 0.0;
        const double d = r - lam;
        v[0] += d * d;
        v[1] += cj * x[j];
        v[2] += (hl ? lo * fmax(lam, 0.0) : 0.0) + (hh ? hi * fmin(lam, 0.0) : 0.0);
        v[3] += cj * cj;
    }
    store_block_partials(v, s + kPartBase + kMaxBlocks * kParts);
    __shared__ bool last;
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned int* ticket = reinterpret_cast<unsigned int*>(s + kTicketSlot);
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    __threadfence();
    double R[kParts] = {0, 0, 0, 0}, Cc[kParts] = {0, 0, 0, 0};
    for (int b = 0; b < row_blocks; ++b)
        for (int q = 0; q < kParts; ++q) R[q] += __ldcg(s + kPartBase + b * kParts + q);
    for (int b = 0; b < (int)gridDim.x; ++b)
        for (int q = 0; q < kParts; ++q) Cc[q] += __ldcg(s + kPartBase + kMaxBlocks * kParts + b * kParts + q);
    const double rp = sqrt(R[0]) / (1.0 + sqrt(R[2]));
    const double rd = sqrt(Cc[0] + R[3]) / (1.0 + sqrt(Cc[3]));
    const double po = Cc[1], dob = R[1] + Cc[2];
    const double gap = fabs(po - dob) / (1.0 + fabs(po) + fabs(dob));
    out[0] = fmax(rp, fmax(rd, gap));
    out[1] = rp;
    out[2] = rd;
    out[3] = gap;
    out[4] = po;
    out[5] = dob;
    *reinterpret_cast<unsigned int*>(s + kTicketSlot) = 0u;
}

}  // namespace

extern "C" int sps_kkt_noalloc(const sps_device_lp* lp, const double* x, const double* y, double* out,
                               void* stream) {
    if (!lp || !x || !y || !out) {
        sps::set_create_error("sps_kkt_noalloc: null argument");
        return SPS_ERR_INVALID;
    }
    const int m = lp->m_ub + lp->m_eq;
    if (lp->n < 0 || lp->m_ub < 0 || lp->m_eq < 0) {
        sps::set_create_error("sps_kkt_noalloc: negative dimension");
        return SPS_ERR_INVALID;
    }
    if (lp->n > kMaxCols) {
        sps::set_create_error("sps_kkt_noalloc: n = " + std::to_string(lp->n) +
                              " exceeds the no-allocation limit of 262144 columns");
        return SPS_ERR_INVALID;
    }
    if ((m > 0 && (!lp->indptr || !lp->rhs)) || (lp->n > 0 && (!lp->c || !lp->lb || !lp->ub))) {
        sps::set_create_error("sps_kkt_noalloc: null device array");
        return SPS_ERR_INVALID;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        sps::set_create_error("sps_kkt_noalloc: no current CUDA device");
        return SPS_ERR_CUDA;
    }
    double* s = nullptr;
    if (int rc = scratch_address(dev, &s)) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // clear what must start at zero: the K^T y accumulator and the ticket
    cudaError_t e = cudaMemsetAsync(s, 0, sizeof(double) * (size_t)lp->n, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(s + kTicketSlot, 0, sizeof(double), st);
    const int row_blocks = (int)std::min<int64_t>(kMaxBlocks, std::max<int64_t>(1, ((int64_t)m * 32 + kThreads - 1) / kThreads));
    const int col_blocks = (int)std::min<int64_t>(kMaxBlocks, std::max<int64_t>(1, ((int64_t)lp->n + kThreads - 1) / kThreads));
    if (e == cudaSuccess) {
        na_rows<<<row_blocks, kThreads, 0, st>>>(*lp, x, y, s);
        na_cols<<<col_blocks, kThreads, 0, st>>>(*lp, x, s, row_blocks, out);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
        sps::set_create_error(std::string("sps_kkt_noalloc: ") + cudaGetErrorString(e));
        return SPS_ERR_CUDA;
    }
    return SPS_OK;
}
