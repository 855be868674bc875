// gnn.cu — the learned warm start's network (sps_gnn_* in include/sps_gnn.h):
// forward, hand-written backward, loss and Adam, all as CUDA kernels.
//
// Activations are kept per instance and node, row-major with the hidden width
// innermost ([instance][node][H], FP32), so every per-node kernel runs over the
// flattened node list of the whole batch and the weight gradients are sums
// over it.  Aggregations are CSR SpMMs (warp per destination row, float2 per
// lane); the dense node update is a register-tiled FP32 contraction of
// 128-node tiles with both weight matrices staged in shared memory (BF16
// weights widened to FP32), its backward a 32-node-tile kernel.  Every
// reduction (weight gradients, losses, pooling) writes per-block partials that
// a second kernel sums in block order: training is bitwise reproducible.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/sps_gnn.h"
#include "gnn_internal.cuh"
#include "nvtx.cuh"

namespace {

constexpr int kT = 256;          // threads per block
constexpr int kTile = 32;        // nodes per tile in the dense kernels
constexpr int kMaxF = 8;         // input feature width limit

__device__ __forceinline__ float relu(float v) { return v > 0.f ? v : 0.f; }

// ---- input layer: h = relu(W f + b), W is H x F ------------------------------------
template <int H>
__global__ void __launch_bounds__(kT) k_input(const float* __restrict__ f, int64_t nodes, int F,
                                              const __nv_bfloat16* __restrict__ W, const float* __restrict__ bias,
                                              float* __restrict__ h) {
    const int64_t total = nodes * H;
    for (int64_t t = blockIdx.x * (int64_t)kT + threadIdx.x; t < total; t += (int64_t)gridDim.x * kT) {
        const int64_t v = t / H;
        const int o = int(t % H);
        float acc = bias[o];
        for (int q = 0; q < F; ++q) acc += __bfloat162float(W[o * F + q]) * f[v * F + q];
        h[t] = relu(acc);
    }
}

// ---- aggregation: out[s, r] (+)= sum_k val[k] * in[s, idx[k]] ----------------------
// One warp per destination row of one instance; lane l owns features 2l, 2l+1
// (H = 64) or l (H = 32).
template <int H>
__global__ void __launch_bounds__(kT) k_agg(const int32_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                                            const float* __restrict__ val, const float* __restrict__ in,
                                            float* __restrict__ out, int n_dst, int n_src, int batch, int accumulate) {
    const int lane = threadIdx.x & 31;
    const int64_t rows = (int64_t)n_dst * batch;
    for (int64_t w = (blockIdx.x * (int64_t)kT + threadIdx.x) >> 5; w < rows; w += ((int64_t)gridDim.x * kT) >> 5) {
        const int64_t s = w / n_dst;
        const int r = int(w % n_dst);
        const float* src = in + s * (int64_t)n_src * H;
        const int b = ptr[r], e = ptr[r + 1];
        if (H == 64) {
            float2 acc = make_float2(0.f, 0.f);
            int k = b;
            for (; k + 4 <= e; k += 4) {
                float2 v[4];
                float a[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    a[u] = __ldg(val + k + u);
                    v[u] = __ldg(reinterpret_cast<const float2*>(src + (int64_t)__ldg(idx + k + u) * H) + lane);
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) { acc.x += a[u] * v[u].x; acc.y += a[u] * v[u].y; }
            }
            for (; k < e; ++k) {
                const float a = __ldg(val + k);
                const float2 v = __ldg(reinterpret_cast<const float2*>(src + (int64_t)__ldg(idx + k) * H) + lane);
                acc.x += a * v.x;
                acc.y += a * v.y;
            }
            float2* o = reinterpret_cast<float2*>(out + w * H) + lane;
            if (accumulate) { const float2 p = *o; acc.x += p.x; acc.y += p.y; }
            *o = acc;
        } else {
            float acc = 0.f;
            for (int k = b; k < e; ++k) acc += __ldg(val + k) * __ldg(src + (int64_t)__ldg(idx + k) * H + lane);
            float* o = out + w * H + lane;
            if (accumulate) acc += *o;
            *o = acc;
        }
    }
}

// ---- dense node update: out = relu(U h + M a + b) ---------------------------------
// A register-tiled FP32 contraction of the tile's [h | a] (kUpdNodes x 2H) with
// W^T = [U | M]^T (2H x H).  The block stages W^T (BF16 widened to FP32) once
// and, per tile, the nodes' h and a rows as they lie in memory (16-byte loads
// and stores).  Thread t owns nodes ng + 32 i (i < 4, ng = t / 8) and outputs
// 4 og + 32 j + c (og = t % 8, c < 4, j < H / 32): per four input features it
// reads four 16-byte node vectors and 2 H / 8 16-byte weight vectors from
// shared memory for 32 (H = 64) FMAs per feature, so the FMA pipe, not
// shared memory, sets the pace.  Each output is bias + sum over k of W[o][k] x[k]
// in k order (h's features, then a's), one fmaf per k.
constexpr int kUpdNodes = 128;                 // nodes per tile

template <int H>
__host__ __device__ constexpr int upd_stride() { return 2 * H + 4; }   // padded tile row: 4 consecutive rows hit distinct banks

template <int H>
__global__ void __launch_bounds__(kT, 2) k_update(const float* __restrict__ h, const float* __restrict__ a,
                                                  const __nv_bfloat16* __restrict__ U,
                                                  const __nv_bfloat16* __restrict__ M,
                                                  const float* __restrict__ bias, float* __restrict__ out,
                                                  int64_t nodes) {
    static_assert(H % 32 == 0 && kT == 256, "thread layout: 8 output groups x 32 node groups");
    constexpr int K2 = 2 * H, S = upd_stride<H>(), J = H / 32;
    extern __shared__ float sm[];
    float* Wt = sm;                           // [k][o], k < H from U, k >= H from M
    float* X = Wt + K2 * H;                   // [node][S]: h (k < H) then a
    for (int t = threadIdx.x; t < K2 * H; t += kT) {
        const int o = t / K2, k = t % K2;
        Wt[k * H + o] = __bfloat162float(k < H ? U[o * H + k] : M[o * H + (k - H)]);
    }
    const int og = threadIdx.x & 7, ng = threadIdx.x >> 3;
    float4 bo[J];
#pragma unroll
    for (int j = 0; j < J; ++j) {
        const float* b = bias + 4 * og + 32 * j;    // the parameter block's offsets need not be 16-byte aligned
        bo[j] = make_float4(b[0], b[1], b[2], b[3]);
    }
    const int64_t tiles = (nodes + kUpdNodes - 1) / kUpdNodes;
    for (int64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const int64_t base = tile * kUpdNodes;
        __syncthreads();
        for (int t = threadIdx.x; t < kUpdNodes * (K2 / 4); t += kT) {
            const int nd = t / (K2 / 4), q = t % (K2 / 4);
            const int64_t v = base + nd;
            float4 val = make_float4(0.f, 0.f, 0.f, 0.f);
            if (v < nodes)
                val = q < H / 4 ? *reinterpret_cast<const float4*>(h + v * H + 4 * q)
                                : *reinterpret_cast<const float4*>(a + v * H + 4 * (q - H / 4));
            *reinterpret_cast<float4*>(X + nd * S + 4 * q) = val;
        }
        __syncthreads();
        float4 acc[4][J];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < J; ++j) acc[i][j] = bo[j];
#pragma unroll 2
        for (int k = 0; k < K2; k += 4) {
            float4 xv[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) xv[i] = *reinterpret_cast<const float4*>(X + (ng + 32 * i) * S + k);
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
                float4 w[J];
#pragma unroll
                for (int j = 0; j < J; ++j)
                    w[j] = *reinterpret_cast<const float4*>(Wt + (k + kk) * H + 4 * og + 32 * j);
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const float x = kk == 0 ? xv[i].x : kk == 1 ? xv[i].y : kk == 2 ? xv[i].z : xv[i].w;
#pragma unroll
                    for (int j = 0; j < J; ++j) {
                        acc[i][j].x = fmaf(w[j].x, x, acc[i][j].x);
                        acc[i][j].y = fmaf(w[j].y, x, acc[i][j].y);
                        acc[i][j].z = fmaf(w[j].z, x, acc[i][j].z);
                        acc[i][j].w = fmaf(w[j].w, x, acc[i][j].w);
                    }
                }
            }
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int64_t v = base + ng + 32 * i;
            if (v >= nodes) continue;
#pragma unroll
            for (int j = 0; j < J; ++j) {
                const float4 r = make_float4(relu(acc[i][j].x), relu(acc[i][j].y), relu(acc[i][j].z),
                                             relu(acc[i][j].w));
                *reinterpret_cast<float4*>(out + v * H + 4 * og + 32 * j) = r;
            }
        }
    }
}

// ---- dense node update on the tensor cores (H = 64) -------------------------------
// The same update as k_update, out = relu([h | a] W^T + b) with W = [U | M]
// (64 x 128), as tcgen05 MMAs: M = 128 nodes per tile (one TMEM lane each), N =
// 64 outputs (64 TMEM columns of FP32 accumulators), K = 128 in four 32-float
// chunks of 128-byte rows (K-major, 128-byte swizzle: 16-byte piece q of row r
// sits at piece q ^ (r & 7) of the row; 8-row groups 1024 bytes apart), eight
// K = 8 steps per chunk.  The activations are split as x = big + small, both
// TF32 (round to nearest), and both parts are multiplied (the BF16 weights are
// exact in TF32): the products are exact and the sum is accumulated in FP32,
// so the result agrees with the FP32 update to FP32 rounding, not TF32's.
// All 256 threads stage a chunk (global -> split -> swizzled shared memory,
// two buffers); thread 0 issues the chunk's MMAs and commits them to the
// buffer's mbarrier, which the stagers wait on before they overwrite it; the
// eight warps read the accumulators back (tcgen05.ld, warp w: lanes of quarter
// w % 4, columns 32 (w / 4) ..) for the bias and ReLU.  Every wait is bounded;
// a block that gives up sets *err, stops, and still frees its TMEM.
namespace tc {
constexpr int kRows = 128;                    // nodes per tile: the MMA's M and the TMEM lanes
constexpr int kABytes = kRows * 128;          // one 32-float chunk of the activations (16 KB)
constexpr int kBBytes = 64 * 128;             // one 32-float chunk of the weights (8 KB)
constexpr uint32_t kTmemCols = 64;
constexpr int kSmemBytes = 4 * kBBytes + 4 * kABytes + 64 + 1024;   // + barriers, TMEM slot, alignment
constexpr int kWaitPolls = 1 << 20;
// instruction descriptor: D F32, A and B TF32, both K-major, N = 64, M = 128
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ float tf32_rna(float x) {
    uint32_t u;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(u) : "f"(x));
    return __uint_as_float(u);
}

// K-major operand, 128-byte swizzle, 8-row groups 1024 bytes apart
__device__ __forceinline__ uint64_t desc_sw128(uint32_t addr) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (int i = 0; i < kWaitPolls; ++i) {
        uint32_t done;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(done) : "r"(bar), "r"(parity) : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void mma_tf32(uint32_t d, uint64_t a, uint64_t b, uint32_t accumulate) {
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
                 ::"r"(d), "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate) : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                 "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
                 "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                   "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                   "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
                   "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
                   "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}
}  // namespace tc

__global__ void __launch_bounds__(kT, 2) k_update_tc(const float* __restrict__ h, const float* __restrict__ a,
                                                     const __nv_bfloat16* __restrict__ U,
                                                     const __nv_bfloat16* __restrict__ M,
                                                     const float* __restrict__ bias, float* __restrict__ out,
                                                     int64_t nodes, int32_t* __restrict__ err) {
    constexpr int H = 64;
    extern __shared__ __align__(16) unsigned char tc_smem[];
    unsigned char* base = tc_smem + ((1024 - (tc::smem_u32(tc_smem) & 1023)) & 1023);
    unsigned char* Bs = base;                              // 4 chunks of W, 64 rows of 128 bytes
    unsigned char* As = base + 4 * tc::kBBytes;            // buffer b: big at As + 2 b kABytes, small after it
    uint64_t* bars = reinterpret_cast<uint64_t*>(As + 4 * tc::kABytes);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    // the weights, K-major: row o of chunk c holds W[o][32 c .. 32 c + 31]
    for (int t = threadIdx.x; t < 4 * H * 8; t += kT) {
        const int c = t / (H * 8), o = (t / 8) % H, q = t % 8;
        float w[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int k = 32 * c + 4 * q + e;
            w[e] = __bfloat162float(k < H ? U[o * H + k] : M[o * H + (k - H)]);
        }
        *reinterpret_cast<float4*>(Bs + c * tc::kBBytes + o * 128 + ((q ^ (o & 7)) << 4)) =
            make_float4(w[0], w[1], w[2], w[3]);
    }
    if (threadIdx.x == 0) {
        tc::mbar_init(tc::smem_u32(&bars[0]), 1);
        tc::mbar_init(tc::smem_u32(&bars[1]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     ::"r"(tc::smem_u32(tmem_slot)), "r"(tc::kTmemCols) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // W, written by threads, read by the MMA
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = *tmem_slot;
    const int col0 = 32 * (warp >> 2);                     // this warp's accumulator columns
    const uint32_t tq = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)col0;
    uint32_t parity[2] = {0u, 0u};
    bool ok = true;
    const int64_t tiles = (nodes + tc::kRows - 1) / tc::kRows;
    for (int64_t tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
        const int64_t base_node = tile * tc::kRows;
        for (int c = 0; c < 4; ++c) {
            const int buf = c & 1;
            if (c >= 2) {                                  // the MMAs that read this buffer (chunk c - 2)
                if (!tc::mbar_wait(tc::smem_u32(&bars[buf]), parity[buf])) ok = false;
                parity[buf] ^= 1u;
            }
            unsigned char* big = As + 2 * buf * tc::kABytes;
            unsigned char* small = big + tc::kABytes;
            const float* src = c < 2 ? h + 32 * c : a + 32 * (c - 2);
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int pc = threadIdx.x + kT * i, row = pc >> 3, q = pc & 7;
                const int64_t v = base_node + row;
                float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
                if (v < nodes) x = __ldg(reinterpret_cast<const float4*>(src + v * H + 4 * q));
                const float4 hi = make_float4(tc::tf32_rna(x.x), tc::tf32_rna(x.y), tc::tf32_rna(x.z), tc::tf32_rna(x.w));
                const float4 lo = make_float4(tc::tf32_rna(x.x - hi.x), tc::tf32_rna(x.y - hi.y),
                                              tc::tf32_rna(x.z - hi.z), tc::tf32_rna(x.w - hi.w));
                const int off = row * 128 + ((q ^ (row & 7)) << 4);
                *reinterpret_cast<float4*>(big + off) = hi;
                *reinterpret_cast<float4*>(small + off) = lo;
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            tc::fence_before();
            __syncthreads();
            tc::fence_after();
            if (threadIdx.x == 0) {
                const uint32_t ab = tc::smem_u32(big), as = tc::smem_u32(small);
                const uint32_t bb = tc::smem_u32(Bs + c * tc::kBBytes);
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) {
                    const uint64_t bd = tc::desc_sw128(bb + 32 * kk);
                    tc::mma_tf32(tmem, tc::desc_sw128(ab + 32 * kk), bd, (c | kk) != 0 ? 1u : 0u);
                    tc::mma_tf32(tmem, tc::desc_sw128(as + 32 * kk), bd, 1u);
                }
                tc::mma_commit(tc::smem_u32(&bars[buf]));
            }
        }
#pragma unroll
        for (int b = 0; b < 2; ++b) {                      // chunks 2 and 3: the tile's last MMAs
            if (!tc::mbar_wait(tc::smem_u32(&bars[b]), parity[b])) ok = false;
            parity[b] ^= 1u;
        }
        tc::fence_after();
        uint32_t r[32];
        tc::tmem_ld32(tq, r);
        const int64_t v = base_node + 32 * (warp & 3) + lane;
        if (v < nodes && ok) {
            float* o = out + v * H + col0;
#pragma unroll
            for (int j = 0; j < 32; j += 4) {
                const float4 y = make_float4(relu(__uint_as_float(r[j]) + bias[col0 + j]),
                                             relu(__uint_as_float(r[j + 1]) + bias[col0 + j + 1]),
                                             relu(__uint_as_float(r[j + 2]) + bias[col0 + j + 2]),
                                             relu(__uint_as_float(r[j + 3]) + bias[col0 + j + 3]));
                *reinterpret_cast<float4*>(o + j) = y;
            }
        }
        tc::fence_before();
        ok = __syncthreads_and(ok) != 0;                    // TMEM read before the next tile's MMAs
        tc::fence_after();
    }
    if (!ok && threadIdx.x == 0) atomicExch(err, 1);
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(tc::kTmemCols) : "memory");
}

// ---- heads: out[v] = w . h[v] + b (warp per node) ----------------------------------
template <int H>
__global__ void __launch_bounds__(kT) k_head(const float* __restrict__ h, const __nv_bfloat16* __restrict__ w,
                                             const float* __restrict__ b, float* __restrict__ out, int64_t nodes) {
    const int lane = threadIdx.x & 31;
    float w0 = __bfloat162float(w[lane]), w1 = H == 64 ? __bfloat162float(w[lane + 32]) : 0.f;
    for (int64_t v = (blockIdx.x * (int64_t)kT + threadIdx.x) >> 5; v < nodes; v += ((int64_t)gridDim.x * kT) >> 5) {
        float s = h[v * H + lane] * w0;
        if (H == 64) s += h[v * H + lane + 32] * w1;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) out[v] = s + b[0];
    }
}

// ---- per-instance column sums of h over nodes (pooling), block partials ------------
// part[(s * nb + blk) * H + f] over node chunks of instance s (grid.y = instance).
template <int H>
__global__ void __launch_bounds__(kT) k_colsum_part(const float* __restrict__ h, int n, float* __restrict__ part) {
    const int s = blockIdx.y, f = threadIdx.x % H, lanes = kT / H, sub = threadIdx.x / H;
    __shared__ float red[kT];
    float acc = 0.f;
    for (int64_t v = blockIdx.x * (int64_t)lanes + sub; v < n; v += (int64_t)gridDim.x * lanes)
        acc += h[((int64_t)s * n + v) * H + f];
    red[threadIdx.x] = acc;
    __syncthreads();
    if (sub == 0) {
        for (int q = 1; q < lanes; ++q) acc += red[q * H + f];
        part[((int64_t)s * gridDim.x + blockIdx.x) * H + f] = acc;
    }
}

// pool[s][0:H] = mean over constraints, pool[s][H:2H] = mean over variables;
// log_omega[s] = wo . pool + bo
template <int H>
__global__ void k_pool_finish(const float* __restrict__ pc, int nbc, const float* __restrict__ pv, int nbv, int m,
                              int n, const __nv_bfloat16* __restrict__ wo, const float* __restrict__ bo,
                              float* __restrict__ pool, float* __restrict__ lw) {
    const int s = blockIdx.x, f = threadIdx.x;
    __shared__ float red[2 * H];
    if (f < 2 * H) {
        float acc = 0.f;
        if (f < H) { for (int b = 0; b < nbc; ++b) acc += pc[((int64_t)s * nbc + b) * H + f]; acc /= float(m); }
        else { for (int b = 0; b < nbv; ++b) acc += pv[((int64_t)s * nbv + b) * H + f - H]; acc /= float(n); }
        pool[s * 2 * H + f] = acc;
        red[f] = acc * __bfloat162float(wo[f]);
    }
    __syncthreads();
    if (f == 0) {
        float t = 0.f;
        for (int q = 0; q < 2 * H; ++q) t += red[q];
        lw[s] = t + bo[0];
    }
}

// ---- loss and output gradients --------------------------------------------------------
// d = out - target; dout = coef * d; block partial of sum d^2 (per block, in order)
__global__ void __launch_bounds__(kT) k_sq_loss(const float* __restrict__ out, const float* __restrict__ tgt,
                                                int64_t count, float coef, float* __restrict__ dout,
                                                double* __restrict__ part) {
    __shared__ double red[kT];
    double acc = 0.0;
    for (int64_t t = blockIdx.x * (int64_t)kT + threadIdx.x; t < count; t += (int64_t)gridDim.x * kT) {
        const float d = out[t] - tgt[t];
        dout[t] = coef * d;
        acc += double(d) * double(d);
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = kT / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// ---- head backward: dh[v] = dout[v] w + dlw[s] wo_part / N; partials of dw, db -------
// part[blk][0:H] = sum dout h, part[blk][H] = sum dout (H+1 per block)
template <int H>
__global__ void __launch_bounds__(kT) k_head_back(const float* __restrict__ h, const float* __restrict__ dout,
                                                  const __nv_bfloat16* __restrict__ w, const float* __restrict__ dlw,
                                                  const __nv_bfloat16* __restrict__ wo_part, int n, int batch,
                                                  float* __restrict__ dh, float* __restrict__ part) {
    const int f = threadIdx.x % H, lanes = kT / H, sub = threadIdx.x / H;
    const float wf = __bfloat162float(w[f]), wof = __bfloat162float(wo_part[f]) / float(n);
    const int64_t nodes = (int64_t)n * batch;
    float gw = 0.f, gb = 0.f;
    for (int64_t v = blockIdx.x * (int64_t)lanes + sub; v < nodes; v += (int64_t)gridDim.x * lanes) {
        const float d = dout[v];
        dh[v * H + f] = d * wf + dlw[v / n] * wof;
        gw += d * h[v * H + f];
        if (f == 0) gb += d;
    }
    __shared__ float red[kT];
    __shared__ float redb[kT / 32 + 1];
    red[threadIdx.x] = gw;
    if (f == 0) redb[sub] = gb;
    __syncthreads();
    if (sub == 0) {
        for (int q = 1; q < lanes; ++q) gw += red[q * H + f];
        part[(int64_t)blockIdx.x * (H + 1) + f] = gw;
        if (f == 0) {
            for (int q = 1; q < lanes; ++q) gb += redb[q];
            part[(int64_t)blockIdx.x * (H + 1) + H] = gb;
        }
    }
}

// ---- dense node update backward ------------------------------------------------------
// z = U h + M a + b, out = relu(z), dz = dout * (out > 0):
//   dh (=/+=) U^T dz, da = M^T dz, partials of dU = sum dz h^T, dM = sum dz a^T, db = sum dz.
// Thread t: node t / 8 and input features (t % 8) + 8 i for dh / da; weight-gradient
// entries o = t / 4, k = (t % 4) + 4 i (16 of dU and 16 of dM per thread for H = 64).
template <int H>
__global__ void __launch_bounds__(kT) k_update_back(const float* __restrict__ dout, const float* __restrict__ out,
                                                    const float* __restrict__ h, const float* __restrict__ a,
                                                    const __nv_bfloat16* __restrict__ U,
                                                    const __nv_bfloat16* __restrict__ M, float* __restrict__ dh,
                                                    int dh_accumulate, float* __restrict__ da,
                                                    float* __restrict__ part, int64_t nodes) {
    constexpr int OP = H / 8;
    constexpr int ZS = H + 1;
    constexpr int WO = kT / 4 >= H ? 1 : H / (kT / 4);         // weight rows per thread
    constexpr int WK = H / 4;                                  // weight columns per thread
    extern __shared__ float sm[];
    float* Us = sm;                 // [o][k]
    float* Ms = Us + H * H;
    float* Z = Ms + H * H;          // dz tile [kTile][ZS]
    float* Hs = Z + kTile * ZS;     // h tile
    float* As = Hs + kTile * ZS;    // a tile
    for (int t = threadIdx.x; t < H * H; t += kT) {
        Us[t] = __bfloat162float(U[t]);
        Ms[t] = __bfloat162float(M[t]);
    }
    const int node = threadIdx.x >> 3, g = threadIdx.x & 7;
    const int wo0 = threadIdx.x >> 2, wk0 = threadIdx.x & 3;   // weight-gradient ownership
    float gU[WO][WK], gM[WO][WK], gb[WO];
#pragma unroll
    for (int r = 0; r < WO; ++r) {
        gb[r] = 0.f;
#pragma unroll
        for (int i = 0; i < WK; ++i) { gU[r][i] = 0.f; gM[r][i] = 0.f; }
    }
    const int64_t tiles = (nodes + kTile - 1) / kTile;
    for (int64_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const int64_t base = tile * kTile;
        __syncthreads();
        for (int t = threadIdx.x; t < kTile * H; t += kT) {
            const int nd = t / H, k = t % H;
            const int64_t v = base + nd;
            const bool ok = v < nodes;
            Z[nd * ZS + k] = ok && out[v * H + k] > 0.f ? dout[v * H + k] : 0.f;
            Hs[nd * ZS + k] = ok ? h[v * H + k] : 0.f;
            As[nd * ZS + k] = ok ? a[v * H + k] : 0.f;
        }
        __syncthreads();
        // input gradients of this thread's node
        float gh[OP], ga[OP];
#pragma unroll
        for (int i = 0; i < OP; ++i) { gh[i] = 0.f; ga[i] = 0.f; }
        const float* z = Z + node * ZS;
        for (int o = 0; o < H; ++o) {
            const float zo = z[o];
#pragma unroll
            for (int i = 0; i < OP; ++i) {
                gh[i] += Us[o * H + g + 8 * i] * zo;
                ga[i] += Ms[o * H + g + 8 * i] * zo;
            }
        }
        const int64_t v = base + node;
        if (v < nodes) {
#pragma unroll
            for (int i = 0; i < OP; ++i) {
                const int64_t q = v * H + g + 8 * i;
                dh[q] = dh_accumulate ? dh[q] + gh[i] : gh[i];
                da[q] = ga[i];
            }
        }
        // weight gradients over the tile
        for (int nd = 0; nd < kTile; ++nd) {
#pragma unroll
            for (int r = 0; r < WO; ++r) {
                const int o = wo0 + r * (kT / 4);
                if (o >= H) continue;
                const float zo = Z[nd * ZS + o];
                if (wk0 == 0) gb[r] += zo;
#pragma unroll
                for (int i = 0; i < WK; ++i) {
                    const int k = wk0 + 4 * i;
                    gU[r][i] += zo * Hs[nd * ZS + k];
                    gM[r][i] += zo * As[nd * ZS + k];
                }
            }
        }
    }
    // block partial: [dU (H*H) | dM (H*H) | db (H)]
    float* P = part + (int64_t)blockIdx.x * (2 * H * H + H);
#pragma unroll
    for (int r = 0; r < WO; ++r) {
        const int o = wo0 + r * (kT / 4);
        if (o >= H) continue;
#pragma unroll
        for (int i = 0; i < WK; ++i) {
            const int k = wk0 + 4 * i;
            P[o * H + k] = gU[r][i];
            P[H * H + o * H + k] = gM[r][i];
        }
        if (wk0 == 0) P[2 * H * H + o] = gb[r];
    }
}

// input layer backward: dz = dout * (h > 0); partials of dW (H x F) and db (H)
template <int H>
__global__ void __launch_bounds__(kT) k_input_back(const float* __restrict__ dout, const float* __restrict__ h,
                                                   const float* __restrict__ f, int F, int64_t nodes,
                                                   float* __restrict__ part) {
    const int o = threadIdx.x % H, lanes = kT / H, sub = threadIdx.x / H;
    float gw[kMaxF], gb = 0.f;
    for (int q = 0; q < kMaxF; ++q) gw[q] = 0.f;
    for (int64_t v = blockIdx.x * (int64_t)lanes + sub; v < nodes; v += (int64_t)gridDim.x * lanes) {
        const float z = h[v * H + o] > 0.f ? dout[v * H + o] : 0.f;
        gb += z;
        for (int q = 0; q < F; ++q) gw[q] += z * f[v * F + q];
    }
    __shared__ float red[kT * (kMaxF + 1)];
    for (int q = 0; q < F; ++q) red[q * kT + threadIdx.x] = gw[q];
    red[kMaxF * kT + threadIdx.x] = gb;
    __syncthreads();
    if (sub == 0) {
        float* P = part + (int64_t)blockIdx.x * (H * F + H);
        for (int q = 0; q < F; ++q) {
            float s = 0.f;
            for (int l = 0; l < lanes; ++l) s += red[q * kT + l * H + o];
            P[o * F + q] = s;
        }
        float s = 0.f;
        for (int l = 0; l < lanes; ++l) s += red[kMaxF * kT + l * H + o];
        P[H * F + o] = s;
    }
}

// grad[p] += scale * sum_b part[b][p] (blocks in order)
__global__ void k_sum_parts(const float* __restrict__ part, int nb, int width, float scale, float* __restrict__ grad) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < width; p += gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int b = 0; b < nb; ++b) s += part[(int64_t)b * width + p];
        grad[p] += scale * s;
    }
}

// log-omega head gradients: dwo += sum_s dlw[s] pool[s], dbo += sum_s dlw[s]
template <int H>
__global__ void k_omega_back(const float* __restrict__ dlw, const float* __restrict__ pool, int batch,
                             float* __restrict__ gwo, float* __restrict__ gbo) {
    const int f = threadIdx.x;
    if (f < 2 * H) {
        float s = 0.f;
        for (int b = 0; b < batch; ++b) s += dlw[b] * pool[b * 2 * H + f];
        gwo[f] += s;
    }
    if (f == 0) {
        float s = 0.f;
        for (int b = 0; b < batch; ++b) s += dlw[b];
        gbo[0] += s;
    }
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m1,
                       float* __restrict__ m2, __nv_bfloat16* __restrict__ pb, int64_t count, float lr, float b1,
                       float b2, float eps, float c1, float c2) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < count; t += (int64_t)gridDim.x * blockDim.x) {
        const float gt = g[t];
        const float a = b1 * m1[t] + (1.f - b1) * gt;
        const float b = b2 * m2[t] + (1.f - b2) * gt * gt;
        m1[t] = a;
        m2[t] = b;
        const float v = p[t] - lr * (a / c1) / (sqrtf(b / c2) + eps);
        p[t] = v;
        pb[t] = __float2bfloat16_rn(v);
    }
}

__global__ void k_to_bf16(const float* __restrict__ p, __nv_bfloat16* __restrict__ pb, int64_t count) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < count; t += (int64_t)gridDim.x * blockDim.x)
        pb[t] = __float2bfloat16_rn(p[t]);
}

// ---- LP features (lp_features): constraint side, one warp per (instance, row) --------
// cmin = min of c over the row's columns (0 for an empty row); fc = [b, kind, cmin, 1]
__global__ void __launch_bounds__(kT) k_lp_con_features(const int32_t* __restrict__ ptr,
                                                         const int32_t* __restrict__ idx,
                                                         const int8_t* __restrict__ kind,
                                                         const float* __restrict__ c, const float* __restrict__ b,
                                                         int n, int m, int batch, float* __restrict__ fc,
                                                         float* __restrict__ cmin) {
    const int lane = threadIdx.x & 31;
    const int64_t rows = (int64_t)m * batch;
    for (int64_t w = (blockIdx.x * (int64_t)kT + threadIdx.x) >> 5; w < rows; w += ((int64_t)gridDim.x * kT) >> 5) {
        const int64_t s = w / m;
        const int r = int(w % m);
        const float* cs = c + s * (int64_t)n;
        float v = INFINITY;
        for (int k = ptr[r] + lane; k < ptr[r + 1]; k += 32) v = fminf(v, cs[idx[k]]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (lane == 0) {
            const float cm = ptr[r + 1] > ptr[r] ? v : 0.f;
            cmin[w] = cm;
            fc[w * 4 + 0] = b[w];
            fc[w * 4 + 1] = float(kind[r]);
            fc[w * 4 + 2] = cm;
            fc[w * 4 + 3] = 1.f;
        }
    }
}

// variable side, one thread per (instance, column): fv = [c, mean gap over '<=' rows,
// mean gap over '=' rows, 1] with gap = c - cmin(row)
__global__ void __launch_bounds__(kT) k_lp_var_features(const int32_t* __restrict__ ptr,
                                                        const int32_t* __restrict__ idx,
                                                        const int8_t* __restrict__ kind,
                                                        const float* __restrict__ c, const float* __restrict__ cmin,
                                                        int n, int m, int batch, float* __restrict__ fv) {
    const int64_t total = (int64_t)n * batch;
    for (int64_t t = blockIdx.x * (int64_t)kT + threadIdx.x; t < total; t += (int64_t)gridDim.x * kT) {
        const int64_t s = t / n;
        const int j = int(t % n);
        const float cj = c[t];
        float sle = 0.f, seq = 0.f;
        int nle = 0, neq = 0;
        for (int k = ptr[j]; k < ptr[j + 1]; ++k) {
            const int r = idx[k];
            const float d = cj - cmin[s * m + r];
            if (kind[r]) { sle += d; ++nle; } else { seq += d; ++neq; }
        }
        fv[t * 4 + 0] = cj;
        fv[t * 4 + 1] = sle / float(nle > 0 ? nle : 1);
        fv[t * 4 + 2] = seq / float(neq > 0 ? neq : 1);
        fv[t * 4 + 3] = 1.f;
    }
}

}  // namespace

// ===========================================================================
// Host object
// ===========================================================================
struct sps_gnn {
    sps_gnn_graph g{};
    sps_gnn_options opt{};
    int H = 64, L = 3, Fv = 1, Fc = 1, n = 0, m = 0, B = 1;
    int lpf = 0;                 // lp_features: inputs are scaled c and b, expanded on the device
    float *craw = nullptr, *braw = nullptr, *cmin = nullptr;
    int8_t* kind = nullptr;
    int64_t nnz = 0, np = 0;
    cudaStream_t st = nullptr;
    std::vector<void*> dev;
    std::string err;
    // graph: CSR by constraint (a_c and a_v values), CSR by variable (a_v and a_c values)
    int32_t *cptr, *cidx, *vptr, *vidx;
    float *ac_c, *av_c, *av_v, *ac_v;
    // parameters
    float *P, *G, *M1, *M2;
    __nv_bfloat16* PB;
    int64_t step = 0;
    // offsets into the parameter vector
    int64_t oWv, obv, oWc, obc, oL0, per_layer, oWx, obx, oWy, oby, oWo, obo;
    // activations (max batch)
    float *fv, *fc, *xt, *yt, *lt;
    std::vector<float*> HV, HC, AV, AC;
    float *dHV, *dHC, *dHV2, *dHC2, *dA;
    float *x0, *y0, *lw, *pool, *dx0, *dy0, *dlw;
    int32_t* d_err = nullptr;    // set by a tensor-core update that gave up waiting (internal error)
    float *part;              // weight-gradient block partials
    double* lpart;            // loss partials
    float *pcp, *pvp;         // pooling partials
    int nb_dense = 0, nb_pool_c = 0, nb_pool_v = 0, nb_loss = 0;
    int64_t part_floats = 0;

    ~sps_gnn() {
        for (void* p : dev) cudaFree(p);
        if (st) cudaStreamDestroy(st);
    }
    template <class T>
    cudaError_t alloc(T** p, size_t count) {
        void* q = nullptr;
        const cudaError_t e = cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T));
        if (e == cudaSuccess) dev.push_back(q);
        *p = static_cast<T*>(q);
        return e;
    }
    int fail(int code, const std::string& msg) {
        err = msg;
        return code;
    }
    int64_t layer_off(int l) const { return oL0 + per_layer * l; }
};

namespace {

thread_local std::string g_gnn_create_error;

#define GNN_CK(call)                                                                         \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess)                                                               \
            return g->fail(e_ == cudaErrorMemoryAllocation ? -3 : -2,                        \
                           std::string(#call) + ": " + cudaGetErrorString(e_));              \
    } while (0)

template <int H>
size_t update_smem() { return sizeof(float) * (2 * H * H + kUpdNodes * upd_stride<H>()); }
template <int H>
size_t update_back_smem() { return sizeof(float) * (2 * H * H + 3 * kTile * (H + 1)); }

template <int H>
int set_smem_attrs() {
    if (cudaFuncSetAttribute(k_update<H>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)update_smem<H>()) !=
        cudaSuccess)
        return -2;
    if (H == 64 &&
        cudaFuncSetAttribute(k_update_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, tc::kSmemBytes) != cudaSuccess)
        return -2;
    if (cudaFuncSetAttribute(k_update_back<H>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)update_back_smem<H>()) != cudaSuccess)
        return -2;
    return 0;
}

int grid_for(int64_t work, int per_block) {
    const int64_t b = (work + per_block - 1) / per_block;
    return (int)std::max<int64_t>(1, std::min<int64_t>(b, 152 * 8));
}

// The dense node update: on the tensor cores for H = 64, the register-tiled
// FP32 kernel for H = 32.
template <int H>
void dense_update(sps_gnn* g, const float* h, const float* a, const __nv_bfloat16* U, const __nv_bfloat16* M,
                  const float* b, float* out, int64_t nodes) {
    if constexpr (H == 64)
        k_update_tc<<<g->nb_dense, kT, tc::kSmemBytes, g->st>>>(h, a, U, M, b, out, nodes, g->d_err);
    else
        k_update<H><<<g->nb_dense, kT, update_smem<H>(), g->st>>>(h, a, U, M, b, out, nodes);
}

// After the stream is synchronised: a tensor-core update that gave up waiting
// for its MMAs left its flag (the outputs of that forward are not valid).
int device_error(sps_gnn* g) {
    int32_t e = 0;
    if (!g->d_err) return 0;
    if (cudaMemcpyAsync(&e, g->d_err, sizeof(e), cudaMemcpyDeviceToHost, g->st) != cudaSuccess ||
        cudaStreamSynchronize(g->st) != cudaSuccess)
        return g->fail(-2, "reading the network's error flag failed");
    return e ? g->fail(-2, "internal error: a tensor-core node update stopped waiting for its MMAs") : 0;
}

// Forward pass over `batch` instances whose features are already on the device.
template <int H>
int forward(sps_gnn* g, int batch) {
    const int n = g->n, m = g->m, L = g->L;
    const int64_t NV = (int64_t)n * batch, NC = (int64_t)m * batch;
    const __nv_bfloat16* W = g->PB;
    const float* P = g->P;
    cudaStream_t st = g->st;
    k_input<H><<<grid_for(NV * H, kT), kT, 0, st>>>(g->fv, NV, g->Fv, W + g->oWv, P + g->obv, g->HV[0]);
    k_input<H><<<grid_for(NC * H, kT), kT, 0, st>>>(g->fc, NC, g->Fc, W + g->oWc, P + g->obc, g->HC[0]);
    for (int l = 0; l < L; ++l) {
        const int64_t o = g->layer_off(l);
        const int64_t oUc = o, oMc = o + H * H, obc = o + 2 * H * H;
        const int64_t oUv = obc + H, oMv = oUv + H * H, obv = oMv + H * H;
        k_agg<H><<<grid_for(NC * 32, kT), kT, 0, st>>>(g->cptr, g->cidx, g->ac_c, g->HV[l], g->AC[l], m, n, batch, 0);
        dense_update<H>(g, g->HC[l], g->AC[l], W + oUc, W + oMc, P + obc, g->HC[l + 1], NC);
        k_agg<H><<<grid_for(NV * 32, kT), kT, 0, st>>>(g->vptr, g->vidx, g->av_v, g->HC[l + 1], g->AV[l], n, m, batch,
                                                       0);
        dense_update<H>(g, g->HV[l], g->AV[l], W + oUv, W + oMv, P + obv, g->HV[l + 1], NV);
    }
    k_head<H><<<grid_for(NV * 32, kT), kT, 0, st>>>(g->HV[L], W + g->oWx, P + g->obx, g->x0, NV);
    k_head<H><<<grid_for(NC * 32, kT), kT, 0, st>>>(g->HC[L], W + g->oWy, P + g->oby, g->y0, NC);
    k_colsum_part<H><<<dim3(g->nb_pool_c, batch), kT, 0, st>>>(g->HC[L], m, g->pcp);
    k_colsum_part<H><<<dim3(g->nb_pool_v, batch), kT, 0, st>>>(g->HV[L], n, g->pvp);
    k_pool_finish<H><<<batch, 2 * H, 0, st>>>(g->pcp, g->nb_pool_c, g->pvp, g->nb_pool_v, m, n, W + g->oWo,
                                              P + g->obo, g->pool, g->lw);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? 0 : g->fail(-2, std::string("forward: ") + cudaGetErrorString(e));
}

// Loss (host value) and gradient into g->G (zeroed here) for `batch` instances
// whose features and targets are on the device.
template <int H>
int backward(sps_gnn* g, int batch, double* loss) {
    const int n = g->n, m = g->m, L = g->L;
    const int64_t NV = (int64_t)n * batch, NC = (int64_t)m * batch;
    const __nv_bfloat16* W = g->PB;
    cudaStream_t st = g->st;
    const float ax = g->opt.loss_x, ay = g->opt.loss_y, ao = g->opt.loss_omega;
    GNN_CK(cudaMemsetAsync(g->G, 0, sizeof(float) * g->np, st));
    // output gradients: loss = (1/B) sum_s [ax/n |x0-xt|^2 + ay/m |y0-yt|^2 + ao (lw-lt)^2]
    const int nbl = g->nb_loss;
    k_sq_loss<<<nbl, kT, 0, st>>>(g->x0, g->xt, NV, 2.f * ax / (float(n) * batch), g->dx0, g->lpart);
    k_sq_loss<<<nbl, kT, 0, st>>>(g->y0, g->yt, NC, 2.f * ay / (float(m) * batch), g->dy0, g->lpart + nbl);
    k_sq_loss<<<1, kT, 0, st>>>(g->lw, g->lt, batch, 2.f * ao / float(batch), g->dlw, g->lpart + 2 * nbl);
    // heads
    const int nbh = g->nb_dense;
    k_head_back<H><<<nbh, kT, 0, st>>>(g->HV[L], g->dx0, W + g->oWx, g->dlw, W + g->oWo + H, n, batch, g->dHV,
                                       g->part);
    k_sum_parts<<<4, 256, 0, st>>>(g->part, nbh, H + 1, 1.f, g->G + g->oWx);
    k_head_back<H><<<nbh, kT, 0, st>>>(g->HC[L], g->dy0, W + g->oWy, g->dlw, W + g->oWo, m, batch, g->dHC, g->part);
    k_sum_parts<<<4, 256, 0, st>>>(g->part, nbh, H + 1, 1.f, g->G + g->oWy);
    k_omega_back<H><<<1, 2 * H, 0, st>>>(g->dlw, g->pool, batch, g->G + g->oWo, g->G + g->obo);
    // layers, last to first.  dHV / dHC hold the gradient of HV[l+1] / HC[l+1].
    float *dhv = g->dHV, *dhc = g->dHC, *dhv_next = g->dHV2, *dhc_next = g->dHC2;
    const int width = 2 * H * H + H;
    for (int l = L - 1; l >= 0; --l) {
        const int64_t o = g->layer_off(l);
        const int64_t oUc = o, oMc = o + H * H;
        const int64_t oUv = oMc + H * H + H, oMv = oUv + H * H;
        // variable update: HV[l+1] = relu(Uv HV[l] + Mv AV[l] + bv)
        k_update_back<H><<<nbh, kT, update_back_smem<H>(), st>>>(dhv, g->HV[l + 1], g->HV[l], g->AV[l], W + oUv,
                                                                 W + oMv, dhv_next, 0, g->dA, g->part, NV);
        k_sum_parts<<<32, 256, 0, st>>>(g->part, nbh, width, 1.f, g->G + oUv);
        // AV[l] = agg_v(HC[l+1]): dHC[l+1] += agg over constraints with a_v values
        k_agg<H><<<grid_for(NC * 32, kT), kT, 0, st>>>(g->cptr, g->cidx, g->av_c, g->dA, dhc, m, n, batch, 1);
        // constraint update: HC[l+1] = relu(Uc HC[l] + Mc AC[l] + bc)
        k_update_back<H><<<nbh, kT, update_back_smem<H>(), st>>>(dhc, g->HC[l + 1], g->HC[l], g->AC[l], W + oUc,
                                                                 W + oMc, dhc_next, 0, g->dA, g->part, NC);
        k_sum_parts<<<32, 256, 0, st>>>(g->part, nbh, width, 1.f, g->G + oUc);
        // AC[l] = agg_c(HV[l]): dHV[l] += agg over variables with a_c values
        k_agg<H><<<grid_for(NV * 32, kT), kT, 0, st>>>(g->vptr, g->vidx, g->ac_v, g->dA, dhv_next, n, m, batch, 1);
        std::swap(dhv, dhv_next);
        std::swap(dhc, dhc_next);
    }
    // input layers
    k_input_back<H><<<nbh, kT, 0, st>>>(dhv, g->HV[0], g->fv, g->Fv, NV, g->part);
    k_sum_parts<<<4, 256, 0, st>>>(g->part, nbh, H * g->Fv + H, 1.f, g->G + g->oWv);
    k_input_back<H><<<nbh, kT, 0, st>>>(dhc, g->HC[0], g->fc, g->Fc, NC, g->part);
    k_sum_parts<<<4, 256, 0, st>>>(g->part, nbh, H * g->Fc + H, 1.f, g->G + g->oWc);
    GNN_CK(cudaGetLastError());
    if (loss) {
        std::vector<double> lp(2 * nbl + 1);
        GNN_CK(cudaMemcpyAsync(lp.data(), g->lpart, sizeof(double) * lp.size(), cudaMemcpyDeviceToHost, st));
        GNN_CK(cudaStreamSynchronize(st));
        double sx = 0, sy = 0;
        for (int b = 0; b < nbl; ++b) { sx += lp[b]; sy += lp[nbl + b]; }
        *loss = (ax * sx / n + ay * sy / m + ao * lp[2 * nbl]) / batch;
    }
    return 0;
}

int upload_inputs(sps_gnn* g, int batch, const float* vf, const float* cf, const float* xt, const float* yt,
                  const float* lt) {
    cudaStream_t st = g->st;
    const size_t nv = (size_t)g->n * batch, nc = (size_t)g->m * batch;
    if (g->lpf) {
        GNN_CK(cudaMemcpyAsync(g->craw, vf, sizeof(float) * nv, cudaMemcpyHostToDevice, st));
        GNN_CK(cudaMemcpyAsync(g->braw, cf, sizeof(float) * nc, cudaMemcpyHostToDevice, st));
        k_lp_con_features<<<grid_for((int64_t)nc * 32, kT), kT, 0, st>>>(g->cptr, g->cidx, g->kind, g->craw, g->braw,
                                                                       g->n, g->m, batch, g->fc, g->cmin);
        k_lp_var_features<<<grid_for((int64_t)nv, kT), kT, 0, st>>>(g->vptr, g->vidx, g->kind, g->craw, g->cmin,
                                                                  g->n, g->m, batch, g->fv);
        GNN_CK(cudaGetLastError());
    } else {
        GNN_CK(cudaMemcpyAsync(g->fv, vf, sizeof(float) * nv * g->Fv, cudaMemcpyHostToDevice, st));
        GNN_CK(cudaMemcpyAsync(g->fc, cf, sizeof(float) * nc * g->Fc, cudaMemcpyHostToDevice, st));
    }
    if (xt) GNN_CK(cudaMemcpyAsync(g->xt, xt, sizeof(float) * nv, cudaMemcpyHostToDevice, st));
    if (yt) GNN_CK(cudaMemcpyAsync(g->yt, yt, sizeof(float) * nc, cudaMemcpyHostToDevice, st));
    if (lt) GNN_CK(cudaMemcpyAsync(g->lt, lt, sizeof(float) * batch, cudaMemcpyHostToDevice, st));
    return 0;
}

int check_batch(sps_gnn* g, int32_t batch, const float* vf, const float* cf) {
    if (batch < 1 || batch > g->B) return g->fail(-1, "batch must be in [1, max_batch]");
    if (!vf || !cf) return g->fail(-1, "null features");
    return 0;
}

// Scaled-uniform initialisation (fan-in), deterministic in the seed.
void init_params(std::vector<float>& p, const sps_gnn* g) {
    uint64_t s = g->opt.seed * 6364136223846793005ULL + 1442695040888963407ULL;
    auto uni = [&]() {
        s ^= s >> 12; s ^= s << 25; s ^= s >> 27;
        return double((s * 2685821657736338717ULL) >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
    };
    const int H = g->H;
    auto fill = [&](int64_t off, int64_t count, double fan_in) {
        const double a = std::sqrt(3.0 / std::max(1.0, fan_in));
        for (int64_t t = 0; t < count; ++t) p[off + t] = float(a * uni());
    };
    std::fill(p.begin(), p.end(), 0.f);
    fill(g->oWv, (int64_t)H * g->Fv, g->Fv);
    fill(g->oWc, (int64_t)H * g->Fc, g->Fc);
    for (int l = 0; l < g->L; ++l) {
        const int64_t o = g->layer_off(l);
        fill(o, 2LL * H * H, 2.0 * H);                       // Uc, Mc
        fill(o + 2LL * H * H + H, 2LL * H * H, 2.0 * H);     // Uv, Mv
    }
    fill(g->oWx, H, H);
    fill(g->oWy, H, H);
    fill(g->oWo, 2 * H, 2.0 * H);
}

template <int H>
int run_loss_grad(sps_gnn* g, int batch, double* loss) {
    if (int rc = forward<H>(g, batch)) return rc;
    return backward<H>(g, batch, loss);
}

}  // namespace

namespace sps {
namespace gnn {

int device_io(sps_gnn* g, DeviceIO* io) {
    if (!g || !io) return -1;
    io->n = g->n;
    io->m = g->m;
    io->max_batch = g->B;
    io->lp_features = g->lpf;
    io->device = g->opt.device;
    io->stream = g->st;
    io->c_in = g->craw;
    io->b_in = g->braw;
    io->x0 = g->x0;
    io->y0 = g->y0;
    io->log_omega = g->lw;
    return 0;
}

int check_device_error(sps_gnn* g) { return g ? device_error(g) : -1; }

int forward_in_place(sps_gnn* g, int batch) {
    if (!g || !g->lpf || batch < 1 || batch > g->B) return g ? g->fail(-1, "forward_in_place needs lp_features") : -1;
    k_lp_con_features<<<grid_for((int64_t)g->m * batch * 32, kT), kT, 0, g->st>>>(
        g->cptr, g->cidx, g->kind, g->craw, g->braw, g->n, g->m, batch, g->fc, g->cmin);
    k_lp_var_features<<<grid_for((int64_t)g->n * batch, kT), kT, 0, g->st>>>(g->vptr, g->vidx, g->kind, g->craw,
                                                                          g->cmin, g->n, g->m, batch, g->fv);
    if (cudaGetLastError() != cudaSuccess) return g->fail(-2, "feature kernels failed to launch");
    return g->H == 64 ? forward<64>(g, batch) : forward<32>(g, batch);
}

}  // namespace gnn
}  // namespace sps

extern "C" {

int sps_gnn_options_init(sps_gnn_options* o) {
    if (!o) return -1;
    std::memset(o, 0, sizeof(*o));
    o->hidden = 64;
    o->layers = 3;
    o->seed = 0;
    o->lr = 1e-3f;
    o->beta1 = 0.9f;
    o->beta2 = 0.999f;
    o->eps = 1e-8f;
    o->loss_x = 1.f;
    o->loss_y = 1.f;
    o->loss_omega = 0.1f;
    o->max_batch = 8;
    o->device = 0;
    return 0;
}

int sps_gnn_create(const sps_gnn_graph* gr, const sps_gnn_options* opt_in, sps_gnn** out) {
    g_gnn_create_error.clear();
    if (!gr || !out) { g_gnn_create_error = "null graph or output"; return -1; }
    *out = nullptr;
    sps_gnn_options opt;
    if (opt_in) opt = *opt_in; else sps_gnn_options_init(&opt);
    if (opt.hidden != 32 && opt.hidden != 64) { g_gnn_create_error = "hidden must be 32 or 64"; return -1; }
    if (opt.layers < 1 || opt.layers > 8 || opt.max_batch < 1) { g_gnn_create_error = "layers in 1..8, max_batch >= 1"; return -1; }
    if (gr->n_var < 1 || gr->n_con < 1 || gr->f_var < 1 || gr->f_var > kMaxF || gr->f_con < 1 || gr->f_con > kMaxF ||
        !gr->con_ptr) {
        g_gnn_create_error = "graph needs n_var, n_con >= 1, feature widths in 1..8 and con_ptr";
        return -1;
    }
    const int m = gr->n_con, n = gr->n_var;
    if (gr->con_ptr[0] != 0) { g_gnn_create_error = "con_ptr[0] != 0"; return -1; }
    for (int i = 0; i < m; ++i)
        if (gr->con_ptr[i + 1] < gr->con_ptr[i]) { g_gnn_create_error = "con_ptr not monotone"; return -1; }
    const int64_t nnz = gr->con_ptr[m];
    if (nnz > 0 && (!gr->con_idx || !gr->con_val)) { g_gnn_create_error = "null con_idx / con_val"; return -1; }
    for (int64_t k = 0; k < nnz; ++k)
        if (gr->con_idx[k] < 0 || gr->con_idx[k] >= n || !std::isfinite(gr->con_val[k])) {
            g_gnn_create_error = "edge " + std::to_string(k) + ": variable out of range or non-finite value";
            return -1;
        }
    if (opt.lp_features && (gr->f_var != 1 || gr->f_con != 1)) {
        g_gnn_create_error = "lp_features takes one input per variable (c) and per row (b): f_var = f_con = 1";
        return -1;
    }
    auto g = new sps_gnn();
    g->g = *gr;
    g->opt = opt;
    g->lpf = opt.lp_features ? 1 : 0;
    g->H = opt.hidden; g->L = opt.layers;
    g->Fv = g->lpf ? 4 : gr->f_var;
    g->Fc = g->lpf ? 4 : gr->f_con;
    g->n = n; g->m = m; g->B = opt.max_batch; g->nnz = nnz;
    const int H = g->H;
    // parameter offsets
    int64_t o = 0;
    g->oWv = o; o += (int64_t)H * g->Fv; g->obv = o; o += H;
    g->oWc = o; o += (int64_t)H * g->Fc; g->obc = o; o += H;
    g->oL0 = o; g->per_layer = 4LL * H * H + 2 * H; o += g->per_layer * g->L;
    g->oWx = o; o += H; g->obx = o; o += 1;
    g->oWy = o; o += H; g->oby = o; o += 1;
    g->oWo = o; o += 2 * H; g->obo = o; o += 1;
    g->np = o;
    // host graph: degrees, normalised values, CSR by variable
    std::vector<int32_t> degc(m), degv(n, 0), vptr(n + 1, 0), vidx(nnz);
    std::vector<float> ac_c(nnz), av_c(nnz), av_v(nnz), ac_v(nnz);
    std::vector<int8_t> kd(m, 0);
    for (int i = 0; i < m; ++i) degc[i] = gr->con_ptr[i + 1] - gr->con_ptr[i];
    for (int64_t k = 0; k < nnz; ++k) degv[gr->con_idx[k]]++;
    for (int j = 0; j < n; ++j) vptr[j + 1] = vptr[j] + degv[j];
    std::vector<int32_t> fill(vptr.begin(), vptr.end() - 1);
    for (int i = 0; i < m; ++i)
        for (int32_t k = gr->con_ptr[i]; k < gr->con_ptr[i + 1]; ++k) {
            const int j = gr->con_idx[k];
            const float a = gr->con_val[k];
            ac_c[k] = a / float(degc[i]);
            av_c[k] = a / float(degv[j]);
            const int32_t q = fill[j]++;
            vidx[q] = i;
            av_v[q] = av_c[k];
            ac_v[q] = ac_c[k];
        }
    int rc = 0;
    {
        sps_gnn* gg = g;
        auto setup = [&]() -> int {
            sps_gnn* g = gg;
            GNN_CK(cudaSetDevice(opt.device));
            GNN_CK(cudaStreamCreateWithFlags(&g->st, cudaStreamNonBlocking));
            if (H == 64) { if (set_smem_attrs<64>()) return g->fail(-2, "shared-memory attribute"); }
            else if (set_smem_attrs<32>()) return g->fail(-2, "shared-memory attribute");
            GNN_CK(g->alloc(&g->cptr, m + 1)); GNN_CK(g->alloc(&g->cidx, nnz));
            GNN_CK(g->alloc(&g->vptr, n + 1)); GNN_CK(g->alloc(&g->vidx, nnz));
            GNN_CK(g->alloc(&g->ac_c, nnz)); GNN_CK(g->alloc(&g->av_c, nnz));
            GNN_CK(g->alloc(&g->av_v, nnz)); GNN_CK(g->alloc(&g->ac_v, nnz));
            auto up = [&](void* d, const void* s, size_t b) {
                return b ? cudaMemcpyAsync(d, s, b, cudaMemcpyHostToDevice, g->st) : cudaSuccess;
            };
            GNN_CK(up(g->cptr, gr->con_ptr, 4 * (size_t)(m + 1))); GNN_CK(up(g->cidx, gr->con_idx, 4 * (size_t)nnz));
            GNN_CK(up(g->vptr, vptr.data(), 4 * (size_t)(n + 1))); GNN_CK(up(g->vidx, vidx.data(), 4 * (size_t)nnz));
            GNN_CK(up(g->ac_c, ac_c.data(), 4 * (size_t)nnz)); GNN_CK(up(g->av_c, av_c.data(), 4 * (size_t)nnz));
            GNN_CK(up(g->av_v, av_v.data(), 4 * (size_t)nnz)); GNN_CK(up(g->ac_v, ac_v.data(), 4 * (size_t)nnz));
            GNN_CK(g->alloc(&g->P, g->np)); GNN_CK(g->alloc(&g->G, g->np));
            GNN_CK(g->alloc(&g->M1, g->np)); GNN_CK(g->alloc(&g->M2, g->np));
            GNN_CK(g->alloc(&g->PB, g->np));
            const int64_t B = g->B, NV = (int64_t)n * B, NC = (int64_t)m * B;
            GNN_CK(g->alloc(&g->fv, NV * g->Fv)); GNN_CK(g->alloc(&g->fc, NC * g->Fc));
            if (g->lpf) {
                GNN_CK(g->alloc(&g->craw, NV)); GNN_CK(g->alloc(&g->braw, NC)); GNN_CK(g->alloc(&g->cmin, NC));
                GNN_CK(g->alloc(&g->kind, m));
                if (gr->con_kind)
                    for (int i = 0; i < m; ++i) kd[i] = gr->con_kind[i] ? 1 : 0;
                GNN_CK(up(g->kind, kd.data(), (size_t)m));
            }
            GNN_CK(g->alloc(&g->xt, NV)); GNN_CK(g->alloc(&g->yt, NC)); GNN_CK(g->alloc(&g->lt, B));
            g->HV.resize(g->L + 1); g->HC.resize(g->L + 1); g->AV.resize(g->L); g->AC.resize(g->L);
            for (int l = 0; l <= g->L; ++l) { GNN_CK(g->alloc(&g->HV[l], NV * H)); GNN_CK(g->alloc(&g->HC[l], NC * H)); }
            for (int l = 0; l < g->L; ++l) { GNN_CK(g->alloc(&g->AV[l], NV * H)); GNN_CK(g->alloc(&g->AC[l], NC * H)); }
            GNN_CK(g->alloc(&g->dHV, NV * H)); GNN_CK(g->alloc(&g->dHV2, NV * H));
            GNN_CK(g->alloc(&g->dHC, NC * H)); GNN_CK(g->alloc(&g->dHC2, NC * H));
            GNN_CK(g->alloc(&g->dA, std::max(NV, NC) * H));
            GNN_CK(g->alloc(&g->x0, NV)); GNN_CK(g->alloc(&g->y0, NC)); GNN_CK(g->alloc(&g->lw, B));
            GNN_CK(g->alloc(&g->dx0, NV)); GNN_CK(g->alloc(&g->dy0, NC)); GNN_CK(g->alloc(&g->dlw, B));
            GNN_CK(g->alloc(&g->pool, 2 * H * B));
            GNN_CK(g->alloc(&g->d_err, 1));
            GNN_CK(cudaMemsetAsync(g->d_err, 0, sizeof(int32_t), g->st));
            g->nb_dense = 152 * 2;
            g->nb_loss = 152 * 2;
            g->nb_pool_c = std::max(1, std::min(64, (m + 31) / 32));
            g->nb_pool_v = std::max(1, std::min(152, (n + 31) / 32));
            g->part_floats = (int64_t)g->nb_dense * (2 * H * H + H);
            GNN_CK(g->alloc(&g->part, g->part_floats));
            GNN_CK(g->alloc(&g->lpart, 2 * g->nb_loss + 1));
            GNN_CK(g->alloc(&g->pcp, (int64_t)g->nb_pool_c * H * B));
            GNN_CK(g->alloc(&g->pvp, (int64_t)g->nb_pool_v * H * B));
            std::vector<float> p(g->np);
            init_params(p, g);
            GNN_CK(up(g->P, p.data(), sizeof(float) * g->np));
            GNN_CK(cudaMemsetAsync(g->M1, 0, sizeof(float) * g->np, g->st));
            GNN_CK(cudaMemsetAsync(g->M2, 0, sizeof(float) * g->np, g->st));
            k_to_bf16<<<grid_for(g->np, 256), 256, 0, g->st>>>(g->P, g->PB, g->np);
            GNN_CK(cudaGetLastError());
            GNN_CK(cudaStreamSynchronize(g->st));
            return 0;
        };
        rc = setup();
    }
    if (rc) {
        g_gnn_create_error = g->err;
        delete g;
        return rc;
    }
    *out = g;
    return 0;
}

int sps_gnn_predict(sps_gnn* g, int32_t batch, const float* vf, const float* cf, float* x0, float* y0, float* lw) {
    sps::NvtxRange nvtx_range("sps_gnn_predict");
    if (!g) return -1;
    if (int rc = check_batch(g, batch, vf, cf)) return rc;
    GNN_CK(cudaSetDevice(g->opt.device));
    if (int rc = upload_inputs(g, batch, vf, cf, nullptr, nullptr, nullptr)) return rc;
    const int rc = g->H == 64 ? forward<64>(g, batch) : forward<32>(g, batch);
    if (rc) return rc;
    const size_t nv = (size_t)g->n * batch, nc = (size_t)g->m * batch;
    if (x0) GNN_CK(cudaMemcpyAsync(x0, g->x0, sizeof(float) * nv, cudaMemcpyDeviceToHost, g->st));
    if (y0) GNN_CK(cudaMemcpyAsync(y0, g->y0, sizeof(float) * nc, cudaMemcpyDeviceToHost, g->st));
    if (lw) GNN_CK(cudaMemcpyAsync(lw, g->lw, sizeof(float) * batch, cudaMemcpyDeviceToHost, g->st));
    GNN_CK(cudaStreamSynchronize(g->st));
    return device_error(g);
}

int sps_gnn_loss_grad(sps_gnn* g, int32_t batch, const float* vf, const float* cf, const float* xt, const float* yt,
                      const float* lt, double* loss, float* grad) {
    if (!g) return -1;
    if (int rc = check_batch(g, batch, vf, cf)) return rc;
    if (!xt || !yt || !lt) return g->fail(-1, "null targets");
    GNN_CK(cudaSetDevice(g->opt.device));
    if (int rc = upload_inputs(g, batch, vf, cf, xt, yt, lt)) return rc;
    const int rc = g->H == 64 ? run_loss_grad<64>(g, batch, loss) : run_loss_grad<32>(g, batch, loss);
    if (rc) return rc;
    if (grad) {
        GNN_CK(cudaMemcpyAsync(grad, g->G, sizeof(float) * g->np, cudaMemcpyDeviceToHost, g->st));
        GNN_CK(cudaStreamSynchronize(g->st));
    }
    return device_error(g);
}

int sps_gnn_train_step(sps_gnn* g, int32_t batch, const float* vf, const float* cf, const float* xt, const float* yt,
                       const float* lt, double* loss) {
    sps::NvtxRange nvtx_range("sps_gnn_train_step");
    if (!g) return -1;
    if (int rc = check_batch(g, batch, vf, cf)) return rc;
    if (!xt || !yt || !lt) return g->fail(-1, "null targets");
    GNN_CK(cudaSetDevice(g->opt.device));
    if (int rc = upload_inputs(g, batch, vf, cf, xt, yt, lt)) return rc;
    const int rc = g->H == 64 ? run_loss_grad<64>(g, batch, loss) : run_loss_grad<32>(g, batch, loss);
    if (rc) return rc;
    g->step += 1;
    const float c1 = 1.f - std::pow(g->opt.beta1, float(g->step)), c2 = 1.f - std::pow(g->opt.beta2, float(g->step));
    k_adam<<<grid_for(g->np, 256), 256, 0, g->st>>>(g->P, g->G, g->M1, g->M2, g->PB, g->np, g->opt.lr,
                                                    g->opt.beta1, g->opt.beta2, g->opt.eps, c1, c2);
    GNN_CK(cudaGetLastError());
    return device_error(g);     // (synchronises the stream)
}

int64_t sps_gnn_num_params(const sps_gnn* g) { return g ? g->np : -1; }

int sps_gnn_get_params(sps_gnn* g, float* out) {
    if (!g || !out) return -1;
    GNN_CK(cudaSetDevice(g->opt.device));
    GNN_CK(cudaMemcpyAsync(out, g->P, sizeof(float) * g->np, cudaMemcpyDeviceToHost, g->st));
    GNN_CK(cudaStreamSynchronize(g->st));
    return 0;
}

int sps_gnn_set_params(sps_gnn* g, const float* in) {
    if (!g || !in) return -1;
    for (int64_t t = 0; t < g->np; ++t)
        if (!std::isfinite(in[t])) return g->fail(-1, "non-finite parameter");
    GNN_CK(cudaSetDevice(g->opt.device));
    GNN_CK(cudaMemcpyAsync(g->P, in, sizeof(float) * g->np, cudaMemcpyHostToDevice, g->st));
    GNN_CK(cudaMemsetAsync(g->M1, 0, sizeof(float) * g->np, g->st));
    GNN_CK(cudaMemsetAsync(g->M2, 0, sizeof(float) * g->np, g->st));
    k_to_bf16<<<grid_for(g->np, 256), 256, 0, g->st>>>(g->P, g->PB, g->np);
    GNN_CK(cudaGetLastError());
    GNN_CK(cudaStreamSynchronize(g->st));
    g->step = 0;
    return 0;
}

const char* sps_gnn_last_error(const sps_gnn* g) { return g ? g->err.c_str() : g_gnn_create_error.c_str(); }

void sps_gnn_destroy(sps_gnn* g) { delete g; }

}  // extern "C"
