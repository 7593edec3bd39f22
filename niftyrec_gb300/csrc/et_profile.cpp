#include "et_profile.h"

#include <atomic>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "et_array_interface.h"

namespace nrgb {

namespace {

std::atomic<long long> g_launches{0};
std::atomic<bool> g_timing{false};
std::mutex g_mu;
std::string g_only;  // time only launches of this name (empty: all)

struct Entry {
  const char* name;
  cudaEvent_t a, b;
};
std::vector<Entry> g_entries;
std::vector<cudaEvent_t> g_free;

cudaEvent_t get_event() {
  if (!g_free.empty()) {
    cudaEvent_t e = g_free.back();
    g_free.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

}  // namespace

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

int prof_begin(const char* name, cudaStream_t st) {
  if (!g_timing.load(std::memory_order_relaxed)) return -1;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_only.empty() && g_only != name) return -1;
  Entry e{name, get_event(), get_event()};
  cudaEventRecord(e.a, st);
  g_entries.push_back(e);
  return static_cast<int>(g_entries.size()) - 1;
}

void prof_end(int slot, cudaStream_t st) {
  if (slot < 0) return;
  std::lock_guard<std::mutex> lk(g_mu);
  if (slot < static_cast<int>(g_entries.size())) cudaEventRecord(g_entries[slot].b, st);
}

}  // namespace nrgb

extern "C" {

// Count of kernel launches issued by this library since load.
long long nrgb_launch_count(void) { return nrgb::g_launches.load(); }

// Enable (1) or disable (0) per-kernel event timing; either clears the record.
int nrgb_profile_enable(int on) {
  std::lock_guard<std::mutex> lk(nrgb::g_mu);
  for (auto& e : nrgb::g_entries) {
    nrgb::g_free.push_back(e.a);
    nrgb::g_free.push_back(e.b);
  }
  nrgb::g_entries.clear();
  nrgb::g_timing.store(on != 0);
  return 0;
}

// Restrict the event timing to launches named `name` (null or "": all).
int nrgb_profile_only(const char* name) {
  std::lock_guard<std::mutex> lk(nrgb::g_mu);
  nrgb::g_only = name ? name : "";
  return 0;
}

// Writes "name launches total_ms\n" per kernel name into buf (NUL-terminated).
// Synchronises on the recorded events.  Returns the bytes needed.
int nrgb_profile_summary(char* buf, int len) {
  std::lock_guard<std::mutex> lk(nrgb::g_mu);
  std::map<std::string, std::pair<int, double>> agg;
  for (auto& e : nrgb::g_entries) {
    cudaEventSynchronize(e.b);
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, e.a, e.b) != cudaSuccess) {
      cudaGetLastError();
      ms = 0.0f;
    }
    auto& v = agg[e.name];
    v.first += 1;
    v.second += ms;
  }
  std::string out;
  char line[256];
  for (auto& kv : agg) {
    std::snprintf(line, sizeof(line), "%s %d %.6f\n", kv.first.c_str(), kv.second.first, kv.second.second);
    out += line;
  }
  if (buf && len > 0) {
    std::strncpy(buf, out.c_str(), static_cast<size_t>(len) - 1);
    buf[len - 1] = '\0';
  }
  return static_cast<int>(out.size()) + 1;
}

}  // extern "C"
