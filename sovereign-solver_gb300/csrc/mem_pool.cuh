// mem_pool.cuh — device memory of the single-LP engines.
//
// One stream-ordered memory pool per CUDA context that keeps up to
// kPoolKeepBytes of freed memory mapped for the next allocation.  The device's
// default pool has a release threshold of 0: at every synchronisation it
// returned to the system what sps_destroy and the set-up's own temporaries had
// freed, so each sps_create mapped its arena and temporaries afresh (a few
// hundred MB for a 4M-nonzero LP).  The pool is looked up by the context's
// unique id (cuCtxGetId, through the runtime's driver entry-point query, so the
// library needs no link against libcuda): a context created after
// cudaDeviceReset, or a caller's own context, gets a pool of its own.  Where
// the id cannot be read or a pool cannot be made, the engines allocate from the
// default pool as before.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

namespace sps {

constexpr uint64_t kPoolKeepBytes = uint64_t(8) << 30;   // freed memory kept mapped, per context

// The pool for allocations on `device` (which must be the current device), or
// null: then use cudaMallocAsync.
inline cudaMemPool_t engine_pool(int device) {
    using GetCurrentFn = CUresult (*)(CUcontext*);
    using GetIdFn = CUresult (*)(CUcontext, unsigned long long*);
    constexpr int kSlots = 64;
    static std::mutex mu;
    static bool tried = false;
    static GetCurrentFn get_current = nullptr;
    static GetIdFn get_id = nullptr;
    static unsigned long long ids[kSlots];
    static cudaMemPool_t pools[kSlots];
    static int used = 0;
    std::lock_guard<std::mutex> lk(mu);
    if (!tried) {
        tried = true;
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<GetCurrentFn>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<GetIdFn>(f);
        cudaGetLastError();
    }
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS)
        return nullptr;
    for (int i = 0; i < used; ++i)
        if (ids[i] == id) return pools[i];
    if (used == kSlots) return nullptr;
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    cudaMemPool_t p = nullptr;
    if (cudaMemPoolCreate(&p, &props) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    uint64_t keep = kPoolKeepBytes;
    if (cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep) != cudaSuccess) {
        cudaGetLastError();
        cudaMemPoolDestroy(p);
        return nullptr;
    }
    ids[used] = id;
    pools[used] = p;
    ++used;
    return p;
}

}  // namespace sps
