// Optional per-kernel timing of the library's own launches.
//
// While enabled (yell_profile_start .. yell_profile_stop) every launch made
// by the launchers is bracketed by a pair of CUDA events recorded on the
// launching stream; totals per kernel name are read back after stop.  When
// disabled the scope objects cost one relaxed atomic load.
//
// Every launch scope and every batch / serving step is also an NVTX range
// (header-only NVTX 3: a no-op unless a tool such as ncu or nsys is attached),
// so a timeline shows the library's launches by name inside its steps.
#pragma once
#include <atomic>
#include <cstdint>
#include <string>
#include <vector>
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

namespace yell_gb300 {

extern std::atomic<bool> g_profiling;

struct ProfileRecord {
  const char* name;
  cudaEvent_t start, stop;
};

void profile_push(const char* name, cudaEvent_t start, cudaEvent_t stop);
cudaEvent_t profile_event();  // from a pool; valid until the next profile_start

int profile_start();
int profile_stop();
int profile_count();
int profile_get(int i, std::string* name, uint64_t* launches, double* total_ms);

// An NVTX range for the lifetime of the object.
class TraceRange {
 public:
  explicit TraceRange(const char* name) { nvtxRangePushA(name); }
  ~TraceRange() { nvtxRangePop(); }
  TraceRange(const TraceRange&) = delete;
  TraceRange& operator=(const TraceRange&) = delete;
};

// Brackets one kernel launch on `st` when profiling is on (and always with an
// NVTX range of the kernel's name).
class LaunchScope {
 public:
  LaunchScope(const char* name, cudaStream_t st) : name_(name), st_(st), range_(name) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (g_profiling.load(std::memory_order_relaxed) &&
        cudaStreamIsCapturing(st_, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusNone) {
      start_ = profile_event();
      stop_ = profile_event();
      if (start_ && stop_) cudaEventRecord(start_, st_);
    }
  }
  ~LaunchScope() {
    if (start_ && stop_) {
      cudaEventRecord(stop_, st_);
      profile_push(name_, start_, stop_);
    }
  }

 private:
  const char* name_;
  cudaStream_t st_;
  TraceRange range_;
  cudaEvent_t start_ = nullptr, stop_ = nullptr;
};

}  // namespace yell_gb300
