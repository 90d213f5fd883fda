// NVTX ranges around the host-side phases of a render (scene build, render request, wave,
// bounce, serving round), so that a profiler's timeline groups the launches by phase. NVTX is
// header-only: without a profiler attached a range costs a test of a null function pointer.
#pragma once
#include <nvtx3/nvToolsExt.h>

namespace yg
{
struct NvtxRange
{
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};
} // namespace yg
