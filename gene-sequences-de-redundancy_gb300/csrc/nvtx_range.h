// nvtx_range.h -- NVTX ranges over the stages of a job (visible on the
// profilers' timelines; no cost without a profiler attached).  NVTX 3 is
// header-only, so nothing is linked.
#pragma once
#if __has_include(<nvtx3/nvToolsExt.h>)
#include <nvtx3/nvToolsExt.h>
#define GSDR_NVTX 1
#else
#define GSDR_NVTX 0  // a toolkit without the NVTX headers: the ranges do nothing
#endif

namespace gsdr {

// An NVTX range over a scope; end() closes it early, and an early return
// closes it on the way out.
struct NvtxRange {
    explicit NvtxRange(const char* name) {
#if GSDR_NVTX
        nvtxRangePushA(name);
#else
        (void)name;
#endif
    }
    ~NvtxRange() { end(); }
    void end() {
#if GSDR_NVTX
        if (open_) nvtxRangePop();
#endif
        open_ = false;
    }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;

  private:
    bool open_ = true;
};

}  // namespace gsdr
