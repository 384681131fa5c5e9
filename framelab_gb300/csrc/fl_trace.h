// fl_trace.h -- NVTX ranges around the C-ABI entry points, so a profiler's
// timeline shows each library call (plan creation, projections, solves) as a
// named range over its kernels. NVTX v3 is header-only; without a profiler
// attached a range costs two calls into an empty stub.
#pragma once
#include <nvtx3/nvToolsExt.h>

struct FlRange {
    explicit FlRange(const char* name) { nvtxRangePushA(name); }
    ~FlRange() { nvtxRangePop(); }
    FlRange(const FlRange&) = delete;
    FlRange& operator=(const FlRange&) = delete;
};
#define FL_RANGE(name) FlRange fl_range_guard_(name)
