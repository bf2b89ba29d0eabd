// vox_trace.h — NVTX ranges around the C ABI's calls, so that a profiler timeline
// (Nsight Systems, ncu's range filters) shows which API call issued which launches.
// NVTX 3 is header-only; with no tool attached a range costs a null-pointer check.
#pragma once

#include <nvtx3/nvToolsExt.h>

namespace vox {

class TraceRange {
 public:
  explicit TraceRange(const char* name) { nvtxRangePushA(name); }
  ~TraceRange() { nvtxRangePop(); }
  TraceRange(const TraceRange&) = delete;
  TraceRange& operator=(const TraceRange&) = delete;
};

}  // namespace vox
