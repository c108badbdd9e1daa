// NVTX ranges around the host-side stages (grid generation, AO store,
// density, functional, V_xc, mixed builds, response), so that an NVTX-aware
// profiler attributes the launches to the reference's stages.  Header-only
// NVTX 3: without a tool attached every call is a no-op.
#pragma once

#include <nvtx3/nvToolsExt.h>

namespace cgb {

struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

}  // namespace cgb
