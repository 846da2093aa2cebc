// NVTX ranges around the host entry points: a profiler's timeline shows each
// query's kernels and copies under the entry point's name.  NVTX v3 is
// header-only; with no tool attached a range costs a branch on a null hook.
#pragma once

#include <nvtx3/nvToolsExt.h>

namespace pwt {

struct Range {
	explicit Range(const char *name) { nvtxRangePushA(name); }
	~Range() { nvtxRangePop(); }
	Range(const Range &) = delete;
	Range &operator=(const Range &) = delete;
};

} // namespace pwt

#define PW_TRACE(name) pwt::Range pw_trace_range_(name)
