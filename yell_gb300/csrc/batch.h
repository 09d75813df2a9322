// Batch executor: runs a list of polymuls of uneven (N, L) as one launch
// sequence per degree bucket (internal; used by yell_dev_polymul_batch and by
// the server).
#pragma once
#include <array>
#include <cstdint>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "kernels.h"
#include "runtime.h"
#include "yell_gb300.h"

namespace yell_gb300 {

class BatchExecutor {
 public:
  static constexpr int kDegrees = (int)(kMaxLogN - kMinLogN + 1);

  int init();
  ~BatchExecutor();

  // Runs descs[0..n) on stream s.  Entry i's two-pass scratch is
  // desc_scratch[i] (an L*N-word device buffer) when desc_scratch is given,
  // else the executor's own grow-on-demand scratch.  With use_graph the
  // launch sequence is captured once per batch shape and replayed.  The
  // caller has made sure every entry's tables are resident (ensure_tables).
  // With fork, buckets run on per-degree side streams joined back into s;
  // without, they run one after another on s (cheaper to issue for small
  // batches whose concurrency comes from several slots in flight).
  int run(DeviceContext* ctx, const yell_polymul_desc* descs, uint64_t* const* desc_scratch,
          uint32_t n, cudaStream_t s, bool use_graph, bool fork = true);

  // The same batch as one launch of the persistent queue kernel: the work
  // items of every bucket in one device queue (batch_queue.h).  Asynchronous
  // on s; a dependency wait that exceeds timeout_ns records YELL_ERR_TIMEOUT
  // in the status word read by queue_status().
  // With phased, the same items run as three stream-ordered launches, one
  // per phase (batch_phases.cu), and nothing waits on the device.
  int run_queue(DeviceContext* ctx, const yell_polymul_desc* descs, uint32_t n, cudaStream_t s,
                uint64_t timeout_ns, bool phased = false);
  // Waits for s and returns (and clears) the queue kernel's status word.
  int queue_status(cudaStream_t s, uint32_t* status);
  // A queue whose row steps depend on column passes that are never queued:
  // every wait runs out after timeout_ns (the bounded-wait check).
  int queue_wait_check(DeviceContext* ctx, cudaStream_t s, uint64_t timeout_ns, uint32_t* status);

  // Grows the list buffers to hold `limbs` limbs now (so later runs do not
  // reallocate, which would synchronise the device).
  int reserve_limbs(size_t limbs);

  // Kernel launches made by the last run() (replays included).
  uint64_t last_launches() const { return last_launches_; }

 private:
  struct Bucket {
    uint32_t log_n = 0;
    uint32_t limbs = 0;
    size_t c_off = 0, a_off = 0, b_off = 0, s_off = 0, cm_off = 0;
    size_t scratch_off = 0;
    const DevMod* mods = nullptr;
  };
  struct CachedGraph {
    cudaGraphExec_t exec = nullptr;
    uint64_t launches = 0;
  };

  int reserve_lists(size_t bytes);
  int reserve_scratch(size_t words);
  int reserve_queue_ctl(size_t words);
  void drop_graphs();
  cudaError_t launch_buckets(const std::vector<Bucket>& buckets, cudaStream_t s, bool scratch_lists,
                             bool fork);

  uint8_t* d_lists_ = nullptr;
  uint8_t* h_lists_ = nullptr;
  size_t lists_bytes_ = 0;
  uint64_t* d_scratch_ = nullptr;
  size_t scratch_words_ = 0;
  uint32_t* d_queue_ctl_ = nullptr;  // [0] status, [1] ticket counter, [2..] per-limb counters
  size_t queue_ctl_words_ = 0;
  bool queue_attrs_ = false;
  bool phase_attrs_ = false;
  uint64_t generation_ = 0;
  std::array<cudaStream_t, kDegrees> side_{};
  std::array<cudaEvent_t, kDegrees> join_{};
  cudaEvent_t fork_ = nullptr, staged_ = nullptr;
  std::map<std::string, CachedGraph> graphs_;
  uint64_t last_launches_ = 0;
};

}  // namespace yell_gb300
