// Host-side launch interface of the NTT / pointwise kernels (internal).
#pragma once
#include <atomic>
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>
#include "common.cuh"

namespace yell_gb300 {

enum class NttDir : int { kForward = 0, kForwardLazy = 1, kBackward = 2 };
enum class EwOp : int { kMulmod = 0, kAddmod = 1, kSubmod = 2, kMuladd = 3, kNegate = 4 };

// Launch geometry chosen per degree (the autotuner may override it).
struct NttShape {
  uint32_t single_cta_max_log_n = 13;  // whole-limb-in-one-CTA up to this degree
  uint32_t k1 = 0;                     // column-pass stages for the two-pass path (0 = default)
};

constexpr uint32_t kMinLogN = 3;
constexpr uint32_t kMaxLogN = 20;

// Each degree's DevMod array holds two copies per modulus: [cm] for the
// transforms and element-wise ops, [kPolymulConsts + cm] for the fused
// polymul, whose product is a Montgomery product (pn holds -p^-1 mod 2^64)
// and whose inverse scales by N^-1 * 2^64 (inv_n, inv_n_iphi and their Shoup
// forms) to cancel the product's 2^-64.  Equal to kMaxModuli.
constexpr uint32_t kPolymulConsts = 1000;

// Kernel launches made by this library (for the caller's accounting).
extern std::atomic<uint64_t> g_kernel_launches;

// Whether this thread's two-pass launches run as programmatic dependents of
// the stream's previous kernel (their CTAs become resident during its last
// wave and wait there).  PlainLaunches clears it for a scope whose kernels
// share the device with other streams' work (a batch's buckets on forked
// streams, the server's batches in flight), where a waiting CTA would hold an
// SM slot that another stream's kernel could use.
extern thread_local bool g_dependent_launches;
struct PlainLaunches {
  bool saved;
  PlainLaunches() : saved(g_dependent_launches) { g_dependent_launches = false; }
  ~PlainLaunches() { g_dependent_launches = saved; }
  PlainLaunches(const PlainLaunches&) = delete;
  PlainLaunches& operator=(const PlainLaunches&) = delete;
};

// Launch as a programmatic dependent of the stream's previous kernel (unless
// g_dependent_launches is cleared): the kernel's CTAs may start while that
// kernel's last CTAs finish, and wait (grid_dep_wait, common.cuh) before
// they touch global memory other than the library's tables.  Used for the
// two-pass NTT and polymul, the samplers and the staged 32-bit polymul.
template <typename... KArgs, typename... Args>
void launch_dependent(void (*kernel)(KArgs...), dim3 grid, uint32_t threads, size_t smem, cudaStream_t st,
                      Args... args) {
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cfg.attrs = attr;
  cfg.numAttrs = g_dependent_launches ? 1 : 0;
  (void)cudaLaunchKernelEx(&cfg, kernel, args...);  // errors surface through cudaGetLastError
}

// Device and pinned-host allocations made by this library.  Every allocation
// goes through these wrappers, so the count covers all of them.
extern std::atomic<uint64_t> g_allocations;
template <class T>
cudaError_t lib_malloc(T** p, size_t bytes) {
  void* v = nullptr;
  const cudaError_t e = cudaMalloc(&v, bytes);
  if (e == cudaSuccess) {
    *p = static_cast<T*>(v);
    g_allocations += 1;
  }
  return e;
}
template <class T>
cudaError_t lib_malloc_host(T** p, size_t bytes, unsigned flags = cudaHostAllocDefault) {
  void* v = nullptr;
  const cudaError_t e = cudaHostAlloc(&v, bytes, flags);
  if (e == cudaSuccess) {
    *p = static_cast<T*>(v);
    g_allocations += 1;
  }
  return e;
}
// Stream-ordered allocation from a memory pool (counted like the others).
template <class T>
cudaError_t lib_malloc_async(T** p, size_t bytes, cudaMemPool_t pool, cudaStream_t st) {
  void* v = nullptr;
  const cudaError_t e = cudaMallocFromPoolAsync(&v, bytes, pool, st);
  if (e == cudaSuccess) {
    *p = static_cast<T*>(v);
    g_allocations += 1;
  }
  return e;
}

// In-place NTT over every limb of `ls`.  mods: the DevMod array of this
// degree, indexed by modulus index.
cudaError_t launch_ntt(const LimbSet& ls, uint32_t log_n, const DevMod* mods, NttDir dir,
                       const NttShape& shape, cudaStream_t st);

// c = INTT(NTT(a) * NTT(b)) per limb.  scratch: one operand's worth of words
// (count << log_n) when log_n takes the two-pass path, else unused; or, when
// scratch_ptrs is given, a device list of one N-word scratch limb per limb.
cudaError_t launch_polymul(const LimbSet& c, const ConstLimbSet& a, const ConstLimbSet& b,
                           uint32_t log_n, const DevMod* mods, uint64_t* scratch,
                           const NttShape& shape, cudaStream_t st,
                           uint64_t* const* scratch_ptrs = nullptr);

// Element-wise op over `count` limbs of N words:
//   mulmod/addmod/submod: dst = op(a, b);  muladd: dst = barrett(a*b + dst);
//   negate: dst = p - a.
cudaError_t launch_elementwise(EwOp op, const LimbSet& dst, const ConstLimbSet& a,
                               const ConstLimbSet& b, uint32_t log_n, const DevMod* mods,
                               cudaStream_t st);

size_t polymul_scratch_words(uint32_t count, uint32_t log_n, const NttShape& shape);
// True when the degree also has a polymul that needs no scratch
// (launch_polymul falls back to it when given none).
bool polymul_scratch_optional(uint32_t log_n);

// Sets the dynamic shared-memory limits of every kernel on the current
// device (called once per device, outside any stream capture).
cudaError_t init_kernel_attributes();

// Copies between the caller's host limbs (L separate arrays of N words) and
// L contiguous device limbs, by kernels that load and store the host memory
// directly (host_access.cu).  Only for a device that reaches pageable host
// memory through the host's page tables (DeviceContext::host_access); every
// limb must be 16-byte aligned (host_limbs_accessible).
bool host_limbs_accessible(const uint64_t* const* limbs, uint32_t L);
cudaError_t gather_host_limbs(uint64_t* dev, const uint64_t* const* limbs, uint32_t L, uint32_t log_n,
                              cudaStream_t st);
cudaError_t scatter_host_limbs(uint64_t* const* limbs, const uint64_t* dev, uint32_t L, uint32_t log_n,
                               cudaStream_t st);
// The same for `limbs` limbs laid out contiguously at `host`, for pageable
// memory (pageable_host: 16-byte aligned, not pinned or registered; pinned
// memory copies as fast through the copy engines, and asynchronously).
bool pageable_host(const void* p);
cudaError_t gather_host_contiguous(uint64_t* dev, const uint64_t* host, uint32_t limbs, uint32_t log_n,
                                   cudaStream_t st);
cudaError_t scatter_host_contiguous(uint64_t* host, const uint64_t* dev, uint32_t limbs, uint32_t log_n,
                                    cudaStream_t st);

// Kernels launched by one call of launch_ntt / launch_polymul / elementwise.
uint32_t ntt_launch_count(uint32_t log_n, const NttShape& shape);
uint32_t polymul_launch_count(uint32_t log_n, const NttShape& shape);

}  // namespace yell_gb300
