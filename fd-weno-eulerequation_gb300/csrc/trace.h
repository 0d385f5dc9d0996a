// Named NVTX ranges around the C ABI's entry points, so a profiler timeline
// (ncu --nvtx, nsys) shows which call a kernel belongs to.  NVTX v3 is
// header-only; without an attached tool each range costs a call that
// returns at once.
#pragma once

#include <nvtx3/nvToolsExt.h>

namespace wenofd {

struct TraceRange {
  explicit TraceRange(const char *name) { nvtxRangePushA(name); }
  ~TraceRange() { nvtxRangePop(); }
  TraceRange(const TraceRange &) = delete;
  TraceRange &operator=(const TraceRange &) = delete;
};

}  // namespace wenofd

#define WENOFD_TRACE(name) ::wenofd::TraceRange wenofd_trace_range_(name)
