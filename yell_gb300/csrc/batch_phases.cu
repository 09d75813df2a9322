// The work queue of a batch as three stream-ordered launches, one per phase:
// forward column passes and whole-limb tiles, then row steps, then inverse
// column passes (the queue kernel's items, in the same order).  Launch order
// is the dependency order, so nothing waits on the device, and each phase
// kernel has the register budget of its own item bodies: the inverse column
// pass runs four CTAs per SM at 64 registers as in the one-degree kernels,
// where the single persistent kernel runs every body at 128.  One CTA per
// item; a kernel holds only one item kind per degree.
#include "batch_queue.h"

#include "ntt_kernels.cuh"

namespace yell_gb300 {
namespace {

constexpr int kPhaseThreads = 256;

// One function per degree, not inlined, so that each body gets its own
// register allocation: inlined into one switch, the eight inverse column
// bodies spilled 240 bytes per thread at 64 registers; separately 36-76.
template <int PHASE, int LOGN>
__device__ __noinline__ void run_phase_item(const QueueBucket& B, uint32_t bid) {
  if constexpr (LOGN < (int)kQueueFirstTwoPass) {
    if constexpr (PHASE == 0) {
      using C = TileCfg<(LOGN >= 4 ? kTileLog : kTileLog - 1), LOGN, 0, (LOGN >= 4 ? 4 : 3)>;
      static_assert(C::THREADS == kPhaseThreads, "whole-limb tile of the phase kernel");
      polymul_whole_body<C>(B.c, B.a, B.b, B.mods, bid);
    }
  } else {
    constexpr int K1 = queue_k1(LOGN), LOGB = LOGN - K1;
    using CC = ColCfg<LOGN, K1>;
    using RC = RowCfg<LOGN, K1>;
    static_assert(CC::THREADS == kPhaseThreads && RC::THREADS == kPhaseThreads, "two-pass tiles of the phase kernel");
    if constexpr (PHASE == 0) col_pass2_body<CC, LOGB>(B.a, B.b, B.c, B.s, B.mods, bid);
    else if constexpr (PHASE == 1) polymul_rows_body<RC, K1>(B.c, as_const(B.s), B.mods, bid);
    else col_pass_body<CC, LOGB, true>(as_const(B.c), B.c, B.mods, bid);
  }
}

template <int PHASE>
__device__ __forceinline__ void dispatch_phase(const QueueBucket& B, uint32_t bid) {
  switch (B.log_n) {
    case 3: run_phase_item<PHASE, 3>(B, bid); break;
    case 4: run_phase_item<PHASE, 4>(B, bid); break;
    case 5: run_phase_item<PHASE, 5>(B, bid); break;
    case 6: run_phase_item<PHASE, 6>(B, bid); break;
    case 7: run_phase_item<PHASE, 7>(B, bid); break;
    case 8: run_phase_item<PHASE, 8>(B, bid); break;
    case 9: run_phase_item<PHASE, 9>(B, bid); break;
    case 10: run_phase_item<PHASE, 10>(B, bid); break;
    case 11: run_phase_item<PHASE, 11>(B, bid); break;
    case 12: run_phase_item<PHASE, 12>(B, bid); break;
    case 13: run_phase_item<PHASE, 13>(B, bid); break;
    case 14: run_phase_item<PHASE, 14>(B, bid); break;
    case 15: run_phase_item<PHASE, 15>(B, bid); break;
    case 16: run_phase_item<PHASE, 16>(B, bid); break;
    case 17: run_phase_item<PHASE, 17>(B, bid); break;
    case 18: run_phase_item<PHASE, 18>(B, bid); break;
    case 19: run_phase_item<PHASE, 19>(B, bid); break;
    case 20: run_phase_item<PHASE, 20>(B, bid); break;
    default: break;
  }
}

// The buckets travel as a kernel parameter, read from the constant bank where
// the bodies use them, like the one-degree kernels' own parameters (a copy of
// the bucket in registers made the 64-register inverse pass spill 384 bytes
// per thread).
struct PhaseParams {
  QueueBucket b[kQueueMaxBuckets];
};
static_assert(sizeof(PhaseParams) <= 4000, "kernel parameter size");

// Item first + blockIdx.x of the queue.  Phases 1 and 2 are launched as
// programmatic dependents of the phase before: their CTAs may start while its
// last CTAs run, and wait for it before reading its words.
template <int PHASE>
__global__ void __launch_bounds__(kPhaseThreads, PHASE == 2 ? 4 : 2)
    k_batch_phase(const __grid_constant__ PhaseParams P, const QueueItem* __restrict__ items, uint32_t first) {
  grid_dep_launch();
  const QueueItem it = items[first + blockIdx.x];
  if constexpr (PHASE > 0) grid_dep_wait();
  dispatch_phase<PHASE>(P.b[it.bucket_kind >> 8], it.bid);
}

}  // namespace

cudaError_t phases_set_attributes() {
  cudaError_t e = cudaFuncSetAttribute(k_batch_phase<0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)(2 * kTileSmemBytes));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_batch_phase<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(2 * kTileSmemBytes));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_batch_phase<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTileSmemBytes);
  return e;
}

cudaError_t launch_batch_phases(const QueueBucket* host_buckets, uint32_t n_buckets, const QueueItem* items,
                                const uint32_t counts[3], cudaStream_t s) {
  static const char* const names[3] = {"batch_phase_fwd", "batch_phase_rows", "batch_phase_inv"};
  if (n_buckets > kQueueMaxBuckets) return cudaErrorInvalidValue;
  PhaseParams P{};
  for (uint32_t i = 0; i < n_buckets; ++i) P.b[i] = host_buckets[i];
  uint32_t first = 0;
  for (int ph = 0; ph < 3; ++ph) {
    if (counts[ph] != 0) {
      LaunchScope ps(names[ph], s);
      if (ph == 0) k_batch_phase<0><<<counts[0], kPhaseThreads, 2 * kTileSmemBytes, s>>>(P, items, first);
      else if (ph == 1) launch_dependent(k_batch_phase<1>, counts[1], kPhaseThreads, 2 * kTileSmemBytes, s, P, items, first);
      else launch_dependent(k_batch_phase<2>, counts[2], kPhaseThreads, kTileSmemBytes, s, P, items, first);
      g_kernel_launches += 1;
      const cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return e;
    }
    first += counts[ph];
  }
  return cudaSuccess;
}

}  // namespace yell_gb300
