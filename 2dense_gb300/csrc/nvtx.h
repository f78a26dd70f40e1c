// nvtx.h — NVTX ranges around the host entry points (steps, stages, uploads, saves, the
// adjoint's passes), visible in Nsight timelines; header-only NVTX3, inert without a tool.
#pragma once
#include <nvtx3/nvToolsExt.h>

namespace dense {
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};
}  // namespace dense
