// NVTX ranges around the runtime's entry points (header-only NVTX v3: without a profiler
// attached the calls return at once).  Nsight Compute and Nsight Systems show them, so a
// capture can be filtered to one world step, batch step or serving iteration.
#pragma once

#include <nvtx3/nvToolsExt.h>

namespace se::rt {

struct TraceRange {
  explicit TraceRange(const char* name) { nvtxRangePushA(name); }
  ~TraceRange() { nvtxRangePop(); }
  TraceRange(const TraceRange&) = delete;
  TraceRange& operator=(const TraceRange&) = delete;
};

}  // namespace se::rt
