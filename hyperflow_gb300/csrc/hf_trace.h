// NVTX ranges around the C ABI's step entry points and kernel phases, for timeline profilers
// (nsys, ncu's NVTX filters).  NVTX v3 is header-only: without an attached tool each range costs
// a branch on an unset function pointer, so the ranges stay on in every build.
#pragma once

#include <nvtx3/nvToolsExt.h>

namespace hf {

// one named range for the lifetime of the object (push at construction, pop at destruction)
class TraceRange {
  public:
    explicit TraceRange(const char* name) { nvtxRangePushA(name); }
    ~TraceRange() { nvtxRangePop(); }
    TraceRange(const TraceRange&) = delete;
    TraceRange& operator=(const TraceRange&) = delete;
};

}  // namespace hf
