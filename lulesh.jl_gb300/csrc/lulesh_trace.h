// NVTX ranges around the reference-facing calls and the step's phases, for
// timeline and kernel-profiling tools (Nsight Systems; Nsight Compute's
// --nvtx --nvtx-include filters select the kernels a call launched). NVTX v3
// is header-only: with no tool attached a range costs a few nanoseconds, so
// the ranges are always on. Phase ranges are named after the reference
// functions the kernels launched inside them replace. Launches recorded into
// a CUDA graph are marked once, when the graph is captured.
#pragma once

#include <nvtx3/nvToolsExt.h>

namespace lulesh {

class TraceRange {
 public:
  explicit TraceRange(const char* name) { nvtxRangePushA(name); }
  ~TraceRange() { nvtxRangePop(); }
  TraceRange(const TraceRange&) = delete;
  TraceRange& operator=(const TraceRange&) = delete;
};

}  // namespace lulesh
