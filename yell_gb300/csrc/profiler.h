// Optional per-kernel timing of the library's own launches.
//
// While enabled (yell_profile_start .. yell_profile_stop) every launch made
// by the launchers is bracketed by a pair of CUDA events recorded on the
// launching stream; totals per kernel name are read back after stop.  When
// disabled the scope objects cost one relaxed atomic load.
#pragma once
#include <atomic>
#include <cstdint>
#include <string>
#include <vector>
#include <cuda_runtime.h>

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

// Brackets one kernel launch on `st` when profiling is on.
class LaunchScope {
 public:
  LaunchScope(const char* name, cudaStream_t st) : name_(name), st_(st) {
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
  cudaEvent_t start_ = nullptr, stop_ = nullptr;
};

}  // namespace yell_gb300
