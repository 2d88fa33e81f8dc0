// Tracing: NVTX host ranges in the "vipp_gb300" domain around every C-ABI
// entry point that queues GPU work and around each kernel class's launches
// (tree, operators, p2m_m2m, m2l, l2l_l2p, p2p, rk4, soften), so that a
// profiler's timeline, or ncu --nvtx --nvtx-include, can select them. NVTX3 is
// header-only and loads a tool only when one is attached
// (NVTX_INJECTION64_PATH); without one a range costs a few nanoseconds.
// Inside a captured step graph the class ranges mark the capture, not the
// replays.
#pragma once

#include <nvtx3/nvToolsExt.h>

namespace gb {

inline nvtxDomainHandle_t nvtx_domain() {
    static const nvtxDomainHandle_t d = nvtxDomainCreateA("vipp_gb300");
    return d;
}

inline void nvtx_push(const char *name) {
    nvtxEventAttributes_t a = {};
    a.version = NVTX_VERSION;
    a.size = NVTX_EVENT_ATTRIB_STRUCT_SIZE;
    a.messageType = NVTX_MESSAGE_TYPE_ASCII;
    a.message.ascii = name;
    nvtxDomainRangePushEx(nvtx_domain(), &a);
}

inline void nvtx_pop() { nvtxDomainRangePop(nvtx_domain()); }

struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtx_push(name); }
    ~NvtxRange() { nvtx_pop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

}  // namespace gb
