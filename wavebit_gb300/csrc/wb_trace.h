// NVTX ranges around the library's entry points and stages, for profilers that read them (ncu
// --nvtx filters, timeline tools). NVTX3 is header-only: without a tool attached every call is
// a no-op, so the ranges stay in release builds.
#pragma once
#include <nvtx3/nvToolsExt.h>

namespace wb {
struct TraceRange {
  explicit TraceRange(const char* name) { nvtxRangePushA(name); }
  ~TraceRange() { nvtxRangePop(); }
  TraceRange(const TraceRange&) = delete;
  TraceRange& operator=(const TraceRange&) = delete;
};
}  // namespace wb
