// nvtx.cuh — a named NVTX range around each entry point that does device work,
// so a profiler (ncu --nvtx, Nsight Systems) attributes time to sps_create,
// sps_solve, sps_batch_solve and the other calls.  NVTX v3 is header-only;
// with no profiler attached a range is two cheap function calls.
#pragma once

#include <nvtx3/nvToolsExt.h>

namespace sps {

struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

}  // namespace sps
