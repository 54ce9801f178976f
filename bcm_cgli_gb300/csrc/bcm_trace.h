// NVTX ranges around the C entry points, so a timeline from nsys, or an
// ncu capture filtered with --nvtx, shows which library call issued which
// kernels.  The calls cost a few nanoseconds and do nothing unless a tool
// is attached (NVTX v3 is header-only).
#pragma once

#include <nvtx3/nvToolsExt.h>

namespace bcmg {

class TraceRange {
 public:
  explicit TraceRange(const char *name) { nvtxRangePushA(name); }
  ~TraceRange() { nvtxRangePop(); }
  TraceRange(const TraceRange &) = delete;
  TraceRange &operator=(const TraceRange &) = delete;
};

}  // namespace bcmg
