// yell_dev_polymul_noalloc: the fused polymul with its scratch in a fixed
// device array, for callers that cannot allocate device memory.
//
// Who cannot allocate: callers whose device memory is owned by someone else
// under a fixed budget (a serving process that admits work against an HBM
// budget, a framework with its own pooled allocator that forbids allocations
// outside the pool), and latency-critical callers, since cudaMalloc/cudaFree
// can synchronise the whole device and stall every other stream.  For them
// the scratch of the two-pass polymul (one operand's worth of words at
// N >= 2^13) lives in the file-scope array below instead of in an allocation.
// At 2^13, where a whole-limb polymul also exists, a batch too large for the
// array runs whole-limb instead.
#include <mutex>
#include <string>

#include "kernels.h"
#include "runtime.h"
#include "yell_gb300.h"

using namespace yell_gb300;

namespace {

// 2^21 words = 16 MiB: scratch for up to 32 limbs at N = 2^16 (e.g. one
// pair of 32-limb polys), 16 at 2^17, 2 at 2^20, 64 at 2^15, 128 at 2^14, 256 at 2^13.  Every GPU
// that loads this module holds the array until the process exits.
constexpr size_t kNoAllocScratchWords = size_t(1) << 21;
static __device__ __align__(256) uint64_t g_noalloc_scratch[kNoAllocScratchWords];

// Device address of g_noalloc_scratch per device.  In host code the symbol
// itself is only a host-side stand-in, so the address is looked up once per
// device with that device current and then passed to the kernels.
std::mutex g_addr_mu;
uint64_t* g_addr[64] = {};

int aligned16(const void* p) { return reinterpret_cast<uintptr_t>(p) % 16 == 0; }

}  // namespace

// The lookup loads the module that holds the array, which is when the array
// takes its device memory.  DeviceContext::ensure_tables_list calls this the
// first time it builds tables on a device, so the memory is taken while
// tables are being allocated anyway, never inside yell_dev_polymul_noalloc.
int yell_gb300::noalloc_prepare(int dev) {
  std::lock_guard<std::mutex> g(g_addr_mu);
  if (dev < 0 || dev >= 64) return fail(kInvalidArgument, "device index out of range");
  if (!g_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return fail_cuda(e, "cudaGetSymbolAddress(noalloc scratch)");
    g_addr[dev] = static_cast<uint64_t*>(p);
  }
  return kOk;
}

uint64_t* yell_gb300::noalloc_scratch(int dev) {
  std::lock_guard<std::mutex> g(g_addr_mu);
  return (dev >= 0 && dev < 64) ? g_addr[dev] : nullptr;
}

extern "C" int yell_dev_polymul_noalloc(uint64_t* d_c, const uint64_t* d_a, const uint64_t* d_b,
                                        uint32_t pairs, uint32_t L, uint32_t log_n, uint32_t cm0,
                                        void* stream) {
  if (!d_c || !d_a || !d_b || pairs == 0) return fail(kInvalidArgument, "null pointer or zero pairs");
  if (d_c == d_a || d_c == d_b) return fail(kInvalidArgument, "d_c aliases an operand");
  if (!aligned16(d_c) || !aligned16(d_a) || !aligned16(d_b))
    return fail(kInvalidArgument, "device pointers must be 16-byte aligned");
  int st = check_degree(log_n);
  if (st != kOk) return st;
  st = check_moduli(cm0, L);
  if (st != kOk) return st;
  uint32_t count = 0;
  st = check_limbs(pairs, L, log_n, &count);
  if (st != kOk) return st;
  DeviceContext* ctx = DeviceContext::current(&st);
  if (!ctx) return st;
  size_t need = polymul_scratch_words(count, log_n, ctx->shape);
  if (need > kNoAllocScratchWords && polymul_scratch_optional(log_n)) need = 0;  // scratch-free variant
  if (need > kNoAllocScratchWords)
    return fail(kInvalidArgument,
                "yell_dev_polymul_noalloc: " + std::to_string(count) + " limbs of degree 2^" +
                    std::to_string(log_n) + " need " + std::to_string(need) +
                    " scratch words; the fixed scratch holds " + std::to_string(kNoAllocScratchWords) +
                    " (at most " + std::to_string(kNoAllocScratchWords >> log_n) + " limbs at this degree)");
  // Building tables allocates, so they must already be resident.
  const DevMod* mods = ctx->tables_ready(log_n, cm0, L);
  if (!mods)
    return fail(kInvalidArgument, "twiddle tables for degree 2^" + std::to_string(log_n) + ", moduli " +
                                      std::to_string(cm0) + ".." + std::to_string(cm0 + L - 1) +
                                      " are not resident: call yell_init_ntt_tables_range first");
  // The array was brought up when the tables were built (noalloc_prepare).
  uint64_t* scratch = nullptr;
  if (need) {
    scratch = noalloc_scratch(ctx->device());
    if (!scratch) return fail(kCudaError, "fixed scratch array of this device was not brought up");
  }
  LimbSet c;
  c.base = d_c;
  c.ptrs = nullptr;
  c.cms = nullptr;
  c.count = count;
  c.L = L;
  c.cm0 = cm0;
  c.pad_ = 0;
  ConstLimbSet a{d_a, nullptr, nullptr, count, L, cm0, 0};
  ConstLimbSet b{d_b, nullptr, nullptr, count, L, cm0, 0};
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : ctx->stream();
  const cudaError_t e = launch_polymul(c, a, b, log_n, mods, scratch, ctx->shape, s);
  if (e != cudaSuccess) return fail_cuda(e, "launch polymul (noalloc)");
  return kOk;
}
