// The persistent batch kernel.  A grid of resident CTAs takes tickets from a
// device counter in queue order; the host writes the queue so that every item
// comes after the items it depends on (all forward column passes, then the
// whole-limb items, then the row steps, then the inverse column passes).
// Whoever holds the smallest unfinished ticket has all its dependencies done,
// so the queue always makes progress.  A dependency wait (a row step waits
// for the column passes of its limb, an inverse column pass for the row
// steps) is bounded in time and in iterations: on expiry it records
// YELL_ERR_TIMEOUT in a status word the host reads, and proceeds.
//
// Item bodies are the polymul kernels' own bodies (ntt_kernels.cuh) called
// with the item's tile index; words written by other CTAs of this launch are
// read through L2 (ld.global.cg), never the non-coherent path; a finished
// item publishes its stores with a fence before bumping its limb's counter.
#include "batch_queue.h"

#include "ntt_kernels.cuh"
#include "yell_gb300.h"

namespace yell_gb300 {
namespace {

constexpr int kQueueThreads = 256;
static_assert(kQueueTileLog == (uint32_t)kTileLog, "queue tiles are the two-pass tiles");

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait until *p >= need (one thread).  Gives up when the global
// timer has advanced timeout_ns, or the SM clock 3 * timeout_ns cycles (a
// second bound that does not rely on the global timer), or after 2^24 polls,
// recording YELL_ERR_TIMEOUT.
__device__ void wait_count(const uint32_t* p, uint32_t need, uint32_t* status, uint64_t timeout_ns) {
  const uint64_t t0 = global_ns();
  const long long c0 = clock64();
  const long long cycles = (long long)(3 * timeout_ns);
  uint32_t sleep_ns = 32;
  for (uint32_t polls = 0;; ++polls) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    if (v >= need) return;
    if (global_ns() - t0 > timeout_ns || clock64() - c0 > cycles || polls >= (1u << 24)) {
      atomicCAS(status, 0u, (uint32_t)YELL_ERR_TIMEOUT);
      return;
    }
    __nanosleep(sleep_ns);
    if (sleep_ns < 1024) sleep_ns <<= 1;
  }
}

template <int LOGN>
__device__ __forceinline__ void run_item(uint32_t kind, const QueueBucket& B, uint32_t bid) {
  if constexpr (LOGN < (int)kQueueFirstTwoPass) {
    using C = TileCfg<(LOGN >= 4 ? kTileLog : kTileLog - 1), LOGN, 0, (LOGN >= 4 ? 4 : 3)>;
    static_assert(C::THREADS == kQueueThreads, "whole-limb tile of the queue kernel");
    polymul_whole_body<C>(B.c, B.a, B.b, B.mods, bid);
  } else {
    constexpr int K1 = queue_k1(LOGN), LOGB = LOGN - K1;
    using CC = ColCfg<LOGN, K1>;
    using RC = RowCfg<LOGN, K1>;
    static_assert(CC::THREADS == kQueueThreads && RC::THREADS == kQueueThreads, "two-pass tiles of the queue kernel");
    if (kind == kItemColFwd) col_pass2_body<CC, LOGB>(B.a, B.b, B.c, B.s, B.mods, bid);
    else if (kind == kItemRows) polymul_rows_body<RC, K1, true>(B.c, as_const(B.s), B.mods, bid);
    else col_pass_body<CC, LOGB, true, true>(as_const(B.c), B.c, B.mods, bid);
  }
}

// Tickets of one CTA: slot cur is the item being run, slot cur + 1 the next
// one (its item already read), slot cur + 2 the one after it (ticket taken).
struct TicketRing {
  uint32_t ticket[3];
  QueueItem item[3];
};

__device__ __forceinline__ uint32_t ring_next(uint32_t s) { return s == 2 ? 0u : s + 1u; }

// One function per degree, not inlined: each body gets its own register
// allocation within the kernel's 128 registers.  Inlined into one switch, the
// bodies shared one allocation and the kernel spilled 448 bytes per thread;
// separately each spills at most 16.  The bucket stays in shared memory.
// Thread 0 starts the two queue reads of later items here, before the body:
// the next item's descriptor and the ticket after it.  Both complete while
// the body runs and are stored when it returns, so neither round trip (nor
// one across the call) is waited for.
template <int LOGN>
__device__ __noinline__ void run_item_of(uint32_t kind, const QueueBucket* s_buckets, uint32_t bucket, uint32_t bid,
                                         const QueueLaunch* q, TicketRing* ring, uint32_t cur) {
  const uint32_t s1 = ring_next(cur), s2 = ring_next(s1);
  uint32_t t2 = 0;
  QueueItem it1{0, 0};
  if (threadIdx.x == 0) {
    const uint32_t t1 = ring->ticket[s1];
    if (t1 < q->n_items) it1 = q->items[t1];
    t2 = atomicAdd(q->next, 1u);
  }
  run_item<LOGN>(kind, s_buckets[bucket], bid);
  if (threadIdx.x == 0) {
    ring->item[s1] = it1;
    ring->ticket[s2] = t2;  // slot s2 was read before the previous item's barrier
  }
}

__device__ __forceinline__ void dispatch(uint32_t kind, const QueueBucket* s_buckets, uint32_t bucket, uint32_t log_n,
                                         uint32_t bid, const QueueLaunch* q, TicketRing* ring, uint32_t cur) {
  switch (log_n) {
    case 3: run_item_of<3>(kind, s_buckets, bucket, bid, q, ring, cur); break;
    case 4: run_item_of<4>(kind, s_buckets, bucket, bid, q, ring, cur); break;
    case 5: run_item_of<5>(kind, s_buckets, bucket, bid, q, ring, cur); break;
    case 6: run_item_of<6>(kind, s_buckets, bucket, bid, q, ring, cur); break;
    case 7: run_item_of<7>(kind, s_buckets, bucket, bid, q, ring, cur); break;
    case 8: run_item_of<8>(kind, s_buckets, bucket, bid, q, ring, cur); break;
    case 9: run_item_of<9>(kind, s_buckets, bucket, bid, q, ring, cur); break;
    case 10: run_item_of<10>(kind, s_buckets, bucket, bid, q, ring, cur); break;
    case 11: run_item_of<11>(kind, s_buckets, bucket, bid, q, ring, cur); break;
    case 12: run_item_of<12>(kind, s_buckets, bucket, bid, q, ring, cur); break;
    case 13: run_item_of<13>(kind, s_buckets, bucket, bid, q, ring, cur); break;
    case 14: run_item_of<14>(kind, s_buckets, bucket, bid, q, ring, cur); break;
    case 15: run_item_of<15>(kind, s_buckets, bucket, bid, q, ring, cur); break;
    case 16: run_item_of<16>(kind, s_buckets, bucket, bid, q, ring, cur); break;
    case 17: run_item_of<17>(kind, s_buckets, bucket, bid, q, ring, cur); break;
    case 18: run_item_of<18>(kind, s_buckets, bucket, bid, q, ring, cur); break;
    case 19: run_item_of<19>(kind, s_buckets, bucket, bid, q, ring, cur); break;
    case 20: run_item_of<20>(kind, s_buckets, bucket, bid, q, ring, cur); break;
    default: break;
  }
}

// Each CTA holds two tickets beyond the item it runs (their atomics and the
// next item's descriptor read are hidden behind the item).  Still
// deadlock-free: the smallest ticket taken and not finished is always some
// CTA's current item (a CTA's prefetched tickets are larger than its current
// one), and it depends only on smaller tickets, which are all finished.
__global__ void __launch_bounds__(kQueueThreads, 2) k_batch_queue(QueueLaunch q) {
  __shared__ TicketRing ring;
  __shared__ __align__(16) QueueBucket s_buckets[kQueueMaxBuckets];
  static_assert(sizeof(QueueBucket) % 8 == 0, "buckets are copied as 8-byte words");
  {
    const uint2* src = reinterpret_cast<const uint2*>(q.buckets);
    uint2* dst = reinterpret_cast<uint2*>(s_buckets);
    const uint32_t words = min(q.n_buckets, kQueueMaxBuckets) * (uint32_t)(sizeof(QueueBucket) / 8);
    for (uint32_t i = threadIdx.x; i < words; i += blockDim.x) dst[i] = src[i];
  }
  if (threadIdx.x == 0) {
    const uint32_t t0 = atomicAdd(q.next, 1u);
    ring.ticket[0] = t0;
    ring.item[0] = t0 < q.n_items ? q.items[t0] : QueueItem{0, 0};
    ring.ticket[1] = atomicAdd(q.next, 1u);
  }
  __syncthreads();
  for (uint32_t cur = 0;; cur = ring_next(cur)) {
    const uint32_t t = ring.ticket[cur];
    if (t >= q.n_items) break;
    const QueueItem it = ring.item[cur];
    const uint32_t kind = it.bucket_kind & 0xFFu, bucket = it.bucket_kind >> 8;
    const QueueBucket& B = s_buckets[bucket];
    uint32_t* publish = nullptr;
    if (kind != kItemWhole) {
      const uint32_t tpl = B.log_n - kTileLog;  // tiles per limb: 2^tpl
      uint32_t* cnt = q.done + B.counter_off + 2 * B.c.ordered(it.bid >> tpl);
      if (kind != kItemColFwd) {
        if (threadIdx.x == 0) wait_count(cnt + (kind == kItemRows ? 0 : 1), 1u << tpl, q.status, q.timeout_ns);
        __syncthreads();
      }
      if (kind != kItemColInv) publish = cnt + (kind == kItemColFwd ? 0 : 1);
    }
    dispatch(kind, s_buckets, bucket, B.log_n, it.bid, &q, &ring, cur);
    __syncthreads();  // every thread's stores issued; the tiles are free again
    if (publish && threadIdx.x == 0) {
      __threadfence();
      atomicAdd(publish, 1u);
    }
  }
}

}  // namespace

size_t queue_smem_bytes() { return 2 * kTileSmemBytes; }

cudaError_t queue_set_attributes() {
  return cudaFuncSetAttribute(k_batch_queue, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)queue_smem_bytes());
}

cudaError_t launch_batch_queue(const QueueLaunch& q, cudaStream_t s) {
  LaunchScope ps("batch_queue", s);
  k_batch_queue<<<q.grid, kQueueThreads, queue_smem_bytes(), s>>>(q);
  g_kernel_launches += 1;
  return cudaGetLastError();
}

}  // namespace yell_gb300
