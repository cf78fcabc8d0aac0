// Named ranges for profilers (Nsight Systems / Nsight Compute ranges) around
// the phases of a step: NVTX v3, header-only. Without a profiler attached a
// range costs a call that returns at once.
#pragma once

#include <nvtx3/nvToolsExt.h>

namespace pfs {

struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

}  // namespace pfs
