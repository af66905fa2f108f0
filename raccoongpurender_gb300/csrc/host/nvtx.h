// nvtx.h — NVTX ranges over the C-ABI entry points, so that a timeline
// profiler (Nsight Systems, or ncu's NVTX filtering) shows which library call
// each kernel belongs to.  NVTX 3 is header-only and costs nothing when no
// profiler is attached.
#pragma once
#include <nvtx3/nvToolsExt.h>

namespace rgr {
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};
}  // namespace rgr

#define RGR_NVTX_RANGE(name) ::rgr::NvtxRange rgr_nvtx_range_(name)
