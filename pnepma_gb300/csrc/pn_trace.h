// pn_trace.h -- NVTX ranges around the library's entry points: one range per solve, sweep, batch
// call and material call, named after the entry point, so Nsight timelines show where host calls
// begin and end.  NVTX v3 is header-only; without a tool attached every call returns at once.
#pragma once

#include <nvtx3/nvToolsExt.h>

namespace pn {

class TraceRange {
 public:
  explicit TraceRange(const char* name) { nvtxRangePushA(name); }
  ~TraceRange() { nvtxRangePop(); }
  TraceRange(const TraceRange&) = delete;
  TraceRange& operator=(const TraceRange&) = delete;
};

}  // namespace pn
