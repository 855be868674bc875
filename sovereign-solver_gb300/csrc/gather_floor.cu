// gather_floor.cu — benchmark support: the floor of a sparse matrix pass whose
// column indices are random (sps_time_gather_floor in include/sps_pdhg.h).
//
// A row pass of K x streams the indices and values of K (8 bytes per
// nonzero) and gathers x at the indices.  When the indices are random over a
// vector that fits in L2, every gathered 4-byte element costs a 32-byte L1
// sector and the pass is bound by the L1/L2 sector rate, not by HBM.  This
// kernel measures that floor with nothing else in the way: each thread reads
// four consecutive nonzeros as one 16-byte index load and one 16-byte value
// load (the best streaming form), gathers x at the four indices and adds the
// products; one value per block is written so the work cannot be dropped.
// The same kernel over indices that walk x in order gives the streaming
// ceiling of the same bytes.  Both take the engine's own dtypes (int32
// indices, FP32 values and x).
#include <algorithm>
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/sps_pdhg.h"

namespace sps {
void set_create_error(const std::string& msg);   // defined in api.cu
}

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ uint32_t mix32(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return (uint32_t)(z ^ (z >> 31));
}

// idx[k] uniform over [0, vec_len) (random) or k mod vec_len (in order); val and x ones.
__global__ void gf_fill(int32_t* __restrict__ idx, float* __restrict__ val, float* __restrict__ x, int64_t nnz,
                        int32_t vec_len, int random) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnz; k += stride) {
        idx[k] = random ? (int32_t)(mix32((uint64_t)k) % (uint32_t)vec_len) : (int32_t)(k % vec_len);
        val[k] = 1.0f;
    }
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < vec_len; j += stride) x[j] = 1.0f;
}

__global__ void __launch_bounds__(kThreads) gf_pass(const int4* __restrict__ idx, const float4* __restrict__ val,
                                                    const float* __restrict__ x, int64_t quads,
                                                    float* __restrict__ out) {
    float acc = 0.0f;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < quads; q += stride) {
        const int4 j = __ldg(idx + q);
        const float4 a = __ldg(val + q);
        acc += a.x * __ldg(x + j.x) + a.y * __ldg(x + j.y) + a.z * __ldg(x + j.z) + a.w * __ldg(x + j.w);
    }
    __shared__ float sm[kThreads / 32];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        float s = 0.0f;
        for (int w = 0; w < kThreads / 32; ++w) s += sm[w];
        out[blockIdx.x] = s;
    }
}

}  // namespace

#define GF_CK(call)                                                                                  \
    do {                                                                                             \
        const cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess) {                                                                     \
            sps::set_create_error(std::string("sps_time_gather_floor: ") + cudaGetErrorString(e_)); \
            rc = e_ == cudaErrorMemoryAllocation ? SPS_ERR_OOM : SPS_ERR_CUDA;                       \
            goto done;                                                                               \
        }                                                                                            \
    } while (0)

extern "C" int sps_time_gather_floor(int64_t nnz, int32_t vec_len, int32_t reps, int32_t device, double* out) {
    if (!out || nnz <= 0 || vec_len <= 0 || reps <= 0 || nnz > ((int64_t)1 << 32)) {
        sps::set_create_error("sps_time_gather_floor: need 0 < nnz <= 2^32, vec_len > 0, reps > 0 and an output");
        return SPS_ERR_INVALID;
    }
    int rc = SPS_OK;
    const int64_t quads = (nnz + 3) / 4, padded = quads * 4;
    int32_t* idx = nullptr;
    float *val = nullptr, *x = nullptr, *sink = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int sms = 0, per_sm = 0, blocks = 0;
    GF_CK(cudaSetDevice(device));
    GF_CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    GF_CK(cudaEventCreate(&e0));
    GF_CK(cudaEventCreate(&e1));
    GF_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    GF_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gf_pass, kThreads, 0));
    blocks = std::max(1, sms * std::max(per_sm, 1));            // one resident wave
    GF_CK(cudaMallocAsync(&idx, sizeof(int32_t) * padded, st));
    GF_CK(cudaMallocAsync(&val, sizeof(float) * padded, st));
    GF_CK(cudaMallocAsync(&x, sizeof(float) * vec_len, st));
    GF_CK(cudaMallocAsync(&sink, sizeof(float) * blocks, st));
    for (int random = 1; random >= 0; --random) {
        gf_fill<<<sms * 8, kThreads, 0, st>>>(idx, val, x, padded, vec_len, random);
        gf_pass<<<blocks, kThreads, 0, st>>>(reinterpret_cast<const int4*>(idx), reinterpret_cast<const float4*>(val),
                                            x, quads, sink);   // warm-up
        GF_CK(cudaGetLastError());
        double total = 0.0;
        for (int r = 0; r < reps; ++r) {
            GF_CK(cudaEventRecord(e0, st));
            gf_pass<<<blocks, kThreads, 0, st>>>(reinterpret_cast<const int4*>(idx),
                                                reinterpret_cast<const float4*>(val), x, quads, sink);
            GF_CK(cudaEventRecord(e1, st));
            GF_CK(cudaEventSynchronize(e1));
            float ms = 0.0f;
            GF_CK(cudaEventElapsedTime(&ms, e0, e1));
            total += ms;
        }
        out[random ? 0 : 1] = total / reps;
    }
done:
    if (idx) cudaFreeAsync(idx, st);
    if (val) cudaFreeAsync(val, st);
    if (x) cudaFreeAsync(x, st);
    if (sink) cudaFreeAsync(sink, st);
    if (st) {
        cudaStreamSynchronize(st);
        cudaStreamDestroy(st);
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    return rc;
}
