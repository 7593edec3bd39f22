// Launch accounting and optional per-kernel CUDA-event timing.
//
// Every kernel launch of the library goes through NRGB_LAUNCH_SCOPE, which
// counts it and, when timing is enabled (nrgb_profile_enable), brackets it
// with events recorded on the launching stream.  Summaries are read with
// nrgb_profile_summary after the work has completed.
#pragma once

#include <cuda_runtime.h>

namespace nrgb {

void count_launch();
// Returns a slot (or -1 when timing is off); pass it to prof_end.
int prof_begin(const char* name, cudaStream_t st);
void prof_end(int slot, cudaStream_t st);

struct LaunchScope {
  int slot;
  cudaStream_t st;
  LaunchScope(const char* name, cudaStream_t s) : slot(prof_begin(name, s)), st(s) { count_launch(); }
  ~LaunchScope() { prof_end(slot, st); }
};

}  // namespace nrgb

#define NRGB_CAT2(a, b) a##b
#define NRGB_CAT(a, b) NRGB_CAT2(a, b)
#define NRGB_LAUNCH_SCOPE(name, stream) ::nrgb::LaunchScope NRGB_CAT(nrgb_scope_, __LINE__)(name, stream)
