// Persistent batch kernel: one launch for a whole batch of polymuls of uneven
// (N, L), driven by a device work queue (internal).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

namespace yell_gb300 {

// Work item kinds.  Whole-limb degrees (N <= 2^12) are one item per CTA tile;
// degrees 2^13 .. 2^20 run the two-pass polymul as three items per tile: the
// forward column pass of a and b, the fused row step, the inverse column pass.
enum QueueItemKind : uint32_t { kItemWhole = 0, kItemColFwd = 1, kItemRows = 2, kItemColInv = 3 };

// One degree bucket: limb lists as in the batch executor; `s` the per-limb
// scratch list (two-pass degrees); counter_off the bucket's first per-limb
// completion counter (two per limb: column passes done, row steps done).
struct QueueBucket {
  LimbSet c;
  ConstLimbSet a, b;
  LimbSet s;
  const DevMod* mods;
  uint32_t log_n;
  uint32_t counter_off;
};

// Item t of the queue: bucket index << 8 | kind, and the tile (block) index.
struct QueueItem {
  uint32_t bucket_kind;
  uint32_t bid;
};

struct QueueLaunch {
  const QueueBucket* buckets;  // 8-byte aligned; copied to shared memory at the kernel's start
  const QueueItem* items;
  uint32_t n_items;
  uint32_t n_buckets;  // at most kQueueMaxBuckets
  uint32_t* next;      // ticket dispenser, zero before the launch
  uint32_t* done;      // per-limb completion counters, zero before the launch
  uint32_t* status;    // first error of a bounded wait (YELL_ERR_TIMEOUT), sticky
  uint64_t timeout_ns; // bound of each dependency wait
  uint32_t grid;
};

// Degrees served by the queue kernel (the column stages of its two-pass
// degrees are fixed by queue_k1).
constexpr uint32_t kQueueMinLogN = 3, kQueueMaxLogN = 20, kQueueFirstTwoPass = 13;
constexpr uint32_t kQueueTileLog = 12;  // tile words of every item (2^11 at N = 8)
constexpr uint32_t kQueueMaxBuckets = kQueueMaxLogN - kQueueMinLogN + 1;  // one bucket per degree

// Column stages of the queue's two-pass items: rows of at most 512 words
// (one warp's) from 2^16 up, so the row step needs only warp barriers.
__host__ __device__ constexpr int queue_k1(int log_n) { return log_n == 13 ? 6 : (log_n <= 15 ? 7 : log_n - 9); }

// Dynamic shared memory of the queue kernel (two 4096-word tiles).
size_t queue_smem_bytes();
cudaError_t queue_set_attributes();
cudaError_t launch_batch_queue(const QueueLaunch& q, cudaStream_t s);

// The same items as three launches in queue order (batch_phases.cu):
// counts[0] forward column passes and whole-limb tiles, counts[1] row steps,
// counts[2] inverse column passes.  The buckets are read on the host and
// passed by value; `items` is the device copy of the queue.
cudaError_t phases_set_attributes();
cudaError_t launch_batch_phases(const QueueBucket* host_buckets, uint32_t n_buckets, const QueueItem* items,
                                const uint32_t counts[3], cudaStream_t s);

}  // namespace yell_gb300
