// Tracing of the C-ABI: an NVTX range per call (visible in Nsight Systems /
// Compute timelines; NVTX v3 is header-only and costs nothing without a
// profiler attached) and, with the environment variable NIFTYREC_LOG=1, one
// JSON line per call on stderr: the entry point, host time of the call and
// the path it took (1 fused gantry kernels, 2 general kernels).
#pragma once

#include <nvtx3/nvToolsExt.h>

#include <chrono>

namespace nrgb {

bool log_enabled();  // NIFTYREC_LOG set to a value other than "0" (read once)
void log_call(const char* name, double host_ms);

class ApiScope {
 public:
  explicit ApiScope(const char* name) : name_(name), log_(log_enabled()) {
    nvtxRangePushA(name);
    if (log_) t0_ = std::chrono::steady_clock::now();
  }
  ~ApiScope() {
    nvtxRangePop();
    if (log_)
      log_call(name_, std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0_).count());
  }
  ApiScope(const ApiScope&) = delete;
  ApiScope& operator=(const ApiScope&) = delete;

 private:
  const char* name_;
  bool log_;
  std::chrono::steady_clock::time_point t0_;
};

}  // namespace nrgb

#define NRGB_API(name) ::nrgb::ApiScope nrgb_api_scope_(name)
