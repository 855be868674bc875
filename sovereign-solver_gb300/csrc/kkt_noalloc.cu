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
// Order-independent K^T y.  The caller gives K in CSR only, so K^T y is a
// scatter of the products a_ij * y_i into the columns.  Floating-point atomic
// adds would make the sum depend on the order the hardware runs them in.
// Instead every product is cut into three integer digits on grids fixed for
// the whole call (units U, U 2^-b, U 2^-2b, U a power of two above the largest
// |a_ij y_i|, b chosen so that no column sum of one digit can exceed 2^51), and
// the digits are added with 64-bit integer atomics.  Integer sums do not depend
// on order, so the result is bitwise reproducible; it carries about 3b bits
// below the largest product (b = 51 - ceil(log2(nnz + 1)), e.g. 117 bits for
// 1e4 nonzeros, 60 bits for 2^31), as good as or better than an FP64 sum.
//
// Scratch: g_noalloc_scratch, kScratchWords 8-byte words (about 6.3 MB), held
// by every GPU that loads the library until the process exits:
//   [0, 3 kMaxCols)                        three digit accumulators per column
//   [kPartBase, + 2 kMaxBlocks kParts)     per-block partial sums of the two passes
//   kMaxSlot                               largest |a_ij y_i| (bits), cleared each call
//   kTicketSlot                            ticket of the column pass, cleared each call
// Limits: n <= kMaxCols (262144) columns; any number of rows.
// Every call shares the array: two calls that overlap on the GPU (different
// streams, or different host threads without ordering) race and return
// garbage; order them on one stream.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <mutex>
#include <string>

#include <cuda.h>
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
constexpr int kDigits = 3;
constexpr int kPartBase = kDigits * kMaxCols;
constexpr int kMaxSlot = kPartBase + 2 * kMaxBlocks * kParts;
constexpr int kTicketSlot = kMaxSlot + 1;
constexpr int kScratchWords = kTicketSlot + 31;

static __device__ __align__(256) double g_noalloc_scratch[kScratchWords];

// ---- device address of g_noalloc_scratch, looked up once per CUDA context.
// The key is the context's unique id (cuCtxGetId), so a context created after
// cudaDeviceReset, or a caller's own non-primary context, gets its own lookup
// instead of a stale address.  The driver functions come through the runtime's
// entry-point query, so the library needs no link against libcuda.
using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

std::mutex g_mu;
constexpr int kCacheSlots = 64;
unsigned long long g_ctx_id[kCacheSlots] = {};
double* g_addr[kCacheSlots] = {};
int g_used = 0;
CtxGetCurrentFn g_get_current = nullptr;
CtxGetIdFn g_get_id = nullptr;
bool g_fns_tried = false;

// Id of the calling thread's current context; false when none is current or the
// driver query is unavailable.
bool current_ctx_id(unsigned long long* id) {
    if (!g_fns_tried) {
        g_fns_tried = true;
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_get_current = reinterpret_cast<CtxGetCurrentFn>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_get_id = reinterpret_cast<CtxGetIdFn>(f);
        cudaGetLastError();
    }
    if (!g_get_current || !g_get_id) return false;
    CUcontext ctx = nullptr;
    if (g_get_current(&ctx) != CUDA_SUCCESS || !ctx) return false;
    return g_get_id(ctx, id) == CUDA_SUCCESS;
}

int scratch_address(double** out) {
    std::lock_guard<std::mutex> lk(g_mu);
    unsigned long long id = 0;
    bool have_id = current_ctx_id(&id);
    if (have_id)
        for (int i = 0; i < g_used; ++i)
            if (g_ctx_id[i] == id) {
                *out = g_addr[i];
                return SPS_OK;
            }
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
        cudaGetLastError();
        sps::set_create_error(std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") + cudaGetErrorString(e));
        return SPS_ERR_CUDA;
    }
    if (!have_id) have_id = current_ctx_id(&id);   // the lookup above made the primary context current
    if (have_id && g_used < kCacheSlots) {
        g_ctx_id[g_used] = id;
        g_addr[g_used] = static_cast<double*>(p);
        ++g_used;
    }
    *out = static_cast<double*>(p);
    return SPS_OK;
}

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block sum of kParts values into part[blockIdx.x * kParts + q] (fixed order).
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

// Grid of the digits: e0 = exponent with max|a_ij y_i| < 2^e0, b bits per digit.
struct Grid {
    int e0, b;
    bool finite;
};

__device__ __forceinline__ Grid grid_of(const sps_device_lp& lp, const double* s) {
    const int m = lp.m_ub + lp.m_eq;
    const long long nnz = m > 0 ? (long long)max(lp.indptr[m], 0) : 0ll;
    const unsigned long long bits = *reinterpret_cast<const unsigned long long*>(s + kMaxSlot);
    Grid g;
    g.finite = bits < 0x7FF0000000000000ull;
    const int ex = (int)(bits >> 52);                 // biased exponent of the largest |product|
    g.e0 = (ex == 0 ? -1022 : ex - 1022);             // 2^(e0-1) <= max < 2^e0 (subnormals: 2^-1022)
    int lg = 0;
    while ((1ll << lg) <= nnz && lg < 62) ++lg;       // ceil(log2(nnz + 1))
    g.b = max(8, 51 - lg);
    return g;
}

// Pass 1, one warp per row: largest |a_ij y_i| (as bits: non-negative doubles
// order like their bit patterns, so an integer max is order-independent).
__global__ void __launch_bounds__(kThreads) na_max(sps_device_lp lp, const double* __restrict__ y,
                                                     double* __restrict__ s) {
    const int m = lp.m_ub + lp.m_eq;
    const int lane = threadIdx.x & 31;
    unsigned long long mx = 0ull;
    for (int i = (blockIdx.x * kThreads + threadIdx.x) >> 5; i < m; i += (gridDim.x * kThreads) >> 5) {
        const double yi = y[i];
        for (int k = lp.indptr[i] + lane; k < lp.indptr[i + 1]; k += 32) {
            const double p = fabs(lp.values[k] * yi);
            const unsigned long long pb = isnan(p) ? 0x7FF8000000000000ull : __double_as_longlong(p);
            mx = max(mx, pb);
        }
    }
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, (unsigned long long)__shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0 && mx) atomicMax(reinterpret_cast<unsigned long long*>(s + kMaxSlot), mx);
}

// Pass 2, one warp per row: residual of K x against the rhs (<= rows count
// only violations), rhs^T y, ||rhs||^2, sign violations of y on <= rows, and
// the digits of every product a_ij y_i added into column j's accumulators.
__global__ void __launch_bounds__(kThreads) na_rows(sps_device_lp lp, const double* __restrict__ x,
                                                     const double* __restrict__ y, double* __restrict__ s) {
    double v[kParts] = {0.0, 0.0, 0.0, 0.0};
    const int m = lp.m_ub + lp.m_eq;
    const int lane = threadIdx.x & 31;
    const Grid g = grid_of(lp, s);
    unsigned long long* acc = reinterpret_cast<unsigned long long*>(s);
    for (int i = (blockIdx.x * kThreads + threadIdx.x) >> 5; i < m; i += (gridDim.x * kThreads) >> 5) {
        const double yi = y[i];
        double sum = 0.0;
        for (int k = lp.indptr[i] + lane; k < lp.indptr[i + 1]; k += 32) {
            const double a = lp.values[k];
            const int j = lp.indices[k];
            sum += a * x[j];
            if (!g.finite) continue;
            // digits of p on the grids 2^(e0-b), 2^(e0-2b), 2^(e0-3b): each scaling by a
            // power of two and each remainder is exact, so only the last digit rounds
            double r = a * yi;
            for (int d = 0; d < kDigits; ++d) {
                const int e = g.e0 - (d + 1) * g.b;
                const long long q = __double2ll_rn(scalbn(r, -e));
                if (q) atomicAdd(acc + (size_t)d * kMaxCols + j, (unsigned long long)q);
                r -= scalbn((double)q, e);
            }
        }
        sum = warp_sum(sum);
        if (lane == 0) {
            const double b = lp.rhs[i];
            double res = sum - b;
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

// Pass 3, one thread per column, and the final reduction in the last block.
// out: rel_kkt, rel_primal, rel_dual, rel_gap, primal objective, dual objective.
__global__ void __launch_bounds__(kThreads) na_cols(sps_device_lp lp, const double* __restrict__ x,
                                                     double* __restrict__ s, int row_blocks,
                                                     double* __restrict__ out) {
    double v[kParts] = {0.0, 0.0, 0.0, 0.0};
    const Grid g = grid_of(lp, s);
    const long long* acc = reinterpret_cast<const long long*>(s);
    for (int j = blockIdx.x * kThreads + threadIdx.x; j < lp.n; j += gridDim.x * kThreads) {
        const double cj = lp.c[j], lo = lp.lb[j], hi = lp.ub[j];
        const bool hl = isfinite(lo), hh = isfinite(hi);
        double aty = 0.0;      // coarse digit first: two roundings in a fixed order
        for (int d = 0; d < kDigits; ++d) aty += scalbn((double)acc[(size_t)d * kMaxCols + j], g.e0 - (d + 1) * g.b);
        if (!g.finite) aty = NAN;
        const double r = cj - aty;
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
    // rows need all four matrix/rhs arrays, even when they hold no nonzeros
    if ((m > 0 && (!lp->indptr || !lp->indices || !lp->values || !lp->rhs)) ||
        (lp->n > 0 && (!lp->c || !lp->lb || !lp->ub))) {
        sps::set_create_error("sps_kkt_noalloc: null device array");
        return SPS_ERR_INVALID;
    }
    double* s = nullptr;
    if (int rc = scratch_address(&s)) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // clear what must start at zero: the digit accumulators, the max and the ticket
    cudaError_t e = cudaSuccess;
    for (int d = 0; d < kDigits && e == cudaSuccess && lp->n > 0; ++d)
        e = cudaMemsetAsync(s + (size_t)d * kMaxCols, 0, sizeof(double) * (size_t)lp->n, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(s + kMaxSlot, 0, 2 * sizeof(double), st);
    const int row_blocks = (int)std::min<int64_t>(kMaxBlocks, std::max<int64_t>(1, ((int64_t)m * 32 + kThreads - 1) / kThreads));
    const int col_blocks = (int)std::min<int64_t>(kMaxBlocks, std::max<int64_t>(1, ((int64_t)lp->n + kThreads - 1) / kThreads));
    if (e == cudaSuccess) {
        na_max<<<row_blocks, kThreads, 0, st>>>(*lp, y, s);
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
