// Copies between the caller's host limbs and device memory done by kernels
// that read and write the host memory directly.
//
// On GB300 the GPU reaches the Grace host's memory over NVLink-C2C and, where
// the device reports cudaDevAttrPageableMemoryAccess with
// cudaDevAttrPageableMemoryAccessUsesHostPageTables, translates addresses
// through the host's own page tables: ordinary pageable allocations (the
// reference's per-limb posix_memalign buffers) are loaded and stored in place,
// with no pinning and no driver staging.  Measured on GB300: a forward NTT of
// 32 limbs of 2^16 run on such limbs where they lie took 0.37 ms against
// 0.82 ms for the same call through pageable cudaMemcpy (34-36 GB/s).
//
// One launch moves up to kHostLimbsPerLaunch limbs; the limb addresses travel
// as a kernel parameter, so only the limb words themselves are read from the
// host.  Each thread moves 16-byte pairs, kUnroll of them in flight, with
// consecutive threads on consecutive pairs.
#include <algorithm>
#include <vector>

#include "kernels.h"
#include "profiler.h"

namespace yell_gb300 {
namespace {

constexpr int kHostLimbsPerLaunch = 256;
constexpr int kCopyThreads = 256;
constexpr int kUnroll = 4;

struct HostLimbPtrs {
  const uint64_t* p[kHostLimbsPerLaunch];
};
static_assert(sizeof(HostLimbPtrs) <= 2048, "kernel parameter size");

// dst_dev[limb][i] = host[limb][i] (GATHER) or host[limb][i] = src_dev[limb][i].
template <bool GATHER>
__global__ void __launch_bounds__(kCopyThreads)
    k_host_limbs(const __grid_constant__ HostLimbPtrs host, uint64_t* __restrict__ dev, uint32_t log_n) {
  const uint32_t pairs = 1u << (log_n - 1);
  const size_t limb_off = (size_t)blockIdx.y << log_n;
  const ulonglong2* src = GATHER ? reinterpret_cast<const ulonglong2*>(host.p[blockIdx.y])
                                 : reinterpret_cast<const ulonglong2*>(dev + limb_off);
  ulonglong2* dst = GATHER ? reinterpret_cast<ulonglong2*>(dev + limb_off)
                           : reinterpret_cast<ulonglong2*>(const_cast<uint64_t*>(host.p[blockIdx.y]));
  const uint32_t stride = gridDim.x * kCopyThreads;
  for (uint32_t i0 = blockIdx.x * kCopyThreads + threadIdx.x; i0 < pairs; i0 += stride * kUnroll) {
    ulonglong2 v[kUnroll];
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) {
      const uint32_t i = i0 + u * stride;
      if (i < pairs) v[u] = src[i];
    }
#pragma unroll
    for (int u = 0; u < kUnroll; ++u) {
      const uint32_t i = i0 + u * stride;
      if (i < pairs) dst[i] = v[u];
    }
  }
}

template <bool GATHER>
cudaError_t host_limbs(const uint64_t* const* limbs, uint64_t* dev, uint32_t L, uint32_t log_n,
                       cudaStream_t st) {
  const uint32_t pairs = 1u << (log_n - 1);
  const uint32_t per_block = kCopyThreads * kUnroll;
  const uint32_t gx = std::max(1u, std::min(64u, pairs / per_block));
  for (uint32_t l0 = 0; l0 < L; l0 += kHostLimbsPerLaunch) {
    const uint32_t nl = std::min<uint32_t>(kHostLimbsPerLaunch, L - l0);
    HostLimbPtrs P{};
    for (uint32_t i = 0; i < nl; ++i) P.p[i] = limbs[l0 + i];
    k_host_limbs<GATHER><<<dim3(gx, nl), kCopyThreads, 0, st>>>(P, dev + ((size_t)l0 << log_n), log_n);
    g_kernel_launches += 1;
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace

bool host_limbs_accessible(const uint64_t* const* limbs, uint32_t L) {
  for (uint32_t i = 0; i < L; ++i)
    if (!limbs[i] || reinterpret_cast<uintptr_t>(limbs[i]) % 16 != 0) return false;
  return true;
}

cudaError_t gather_host_limbs(uint64_t* dev, const uint64_t* const* limbs, uint32_t L, uint32_t log_n,
                              cudaStream_t st) {
  LaunchScope ps("host_gather", st);
  return host_limbs<true>(limbs, dev, L, log_n, st);
}

cudaError_t scatter_host_limbs(uint64_t* const* limbs, const uint64_t* dev, uint32_t L, uint32_t log_n,
                               cudaStream_t st) {
  LaunchScope ps("host_scatter", st);
  return host_limbs<false>(const_cast<const uint64_t* const*>(limbs), const_cast<uint64_t*>(dev), L, log_n, st);
}

bool pageable_host(const void* p) {
  if (!p || reinterpret_cast<uintptr_t>(p) % 16 != 0) return false;
  cudaPointerAttributes attr;
  if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
    cudaGetLastError();  // clear the error the failed query recorded
    return false;
  }
  return attr.type == cudaMemoryTypeUnregistered;
}

cudaError_t gather_host_contiguous(uint64_t* dev, const uint64_t* host, uint32_t limbs, uint32_t log_n,
                                   cudaStream_t st) {
  std::vector<const uint64_t*> ptrs(limbs);
  for (uint32_t i = 0; i < limbs; ++i) ptrs[i] = host + ((size_t)i << log_n);
  return gather_host_limbs(dev, ptrs.data(), limbs, log_n, st);
}

cudaError_t scatter_host_contiguous(uint64_t* host, const uint64_t* dev, uint32_t limbs, uint32_t log_n,
                                    cudaStream_t st) {
  std::vector<uint64_t*> ptrs(limbs);
  for (uint32_t i = 0; i < limbs; ++i) ptrs[i] = host + ((size_t)i << log_n);
  return scatter_host_limbs(ptrs.data(), dev, limbs, log_n, st);
}

}  // namespace yell_gb300
