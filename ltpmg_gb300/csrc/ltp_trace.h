// ltp_trace.h -- NVTX ranges around the library's host-side steps (batch
// loads and launches, pipeline submissions, the serving loops' batch
// closing and completion), for Nsight Systems timelines.  NVTX v3 is
// header-only; with no tool attached a range costs a branch.
#pragma once
#include <nvtx3/nvToolsExt.h>

namespace ltp {

struct TraceRange {
    explicit TraceRange(const char *name) { nvtxRangePushA(name); }
    ~TraceRange() { nvtxRangePop(); }
    TraceRange(const TraceRange &) = delete;
    TraceRange &operator=(const TraceRange &) = delete;
};

}  // namespace ltp
