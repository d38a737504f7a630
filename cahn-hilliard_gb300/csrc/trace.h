// trace.h — NVTX ranges around the C ABI's entry points.
//
// Every entry point that queues or waits for device work opens a range named
// after itself ("chgb_step", "chgb_observables", ...), so a profiler timeline
// (Nsight Systems) or a range-filtered ncu capture (`ncu --nvtx
// --nvtx-include "chgb_step/"`) shows which call launched which kernels.  NVTX
// v3 is header-only: with no tool attached a range costs a few nanoseconds of
// host time.  Build with -DCHGB_NO_NVTX to compile the ranges out.
#pragma once

#ifndef CHGB_NO_NVTX
#include <nvtx3/nvToolsExt.h>

namespace chgb {
struct TraceRange {
    explicit TraceRange(const char *name) { nvtxRangePushA(name); }
    ~TraceRange() { nvtxRangePop(); }
    TraceRange(const TraceRange &) = delete;
    TraceRange &operator=(const TraceRange &) = delete;
};
}  // namespace chgb
#define CHGB_TRACE(name) ::chgb::TraceRange chgb_trace_range_(name)
#else
#define CHGB_TRACE(name) ((void) 0)
#endif
