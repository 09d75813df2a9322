// Host dispatch of the NTT / polymul variants, the element-wise kernels,
// and the autotuner.
#include <array>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "kernels.h"
#include "ntt_variants.h"
#include "profiler.h"
#include "runtime.h"
#include "yell_gb300.h"

namespace yell_gb300 {

namespace {

__device__ __forceinline__ ulonglong2 ld_pair(const uint64_t* p) {
  return __ldg(reinterpret_cast<const ulonglong2*>(p));
}

__device__ __forceinline__ void st_pair(uint64_t* p, uint64_t a, uint64_t b) {
  *reinterpret_cast<ulonglong2*>(p) = make_ulonglong2(a, b);
}

// ===========================================================================
// Element-wise ops, two words per thread with 128-bit accesses.
// ===========================================================================
template <int OP>
__global__ void __launch_bounds__(256) k_elementwise(LimbSet dst, ConstLimbSet a, ConstLimbSet b,
                                                     uint32_t log_n, const DevMod* __restrict__ mods) {
  const size_t pairs = ((size_t)dst.count << log_n) >> 1;
  const uint32_t nmask = (1u << log_n) - 1u;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < pairs;
       i += (size_t)gridDim.x * blockDim.x) {
    const size_t v = i * 2;
    const uint32_t limb = (uint32_t)(v >> log_n);
    const uint32_t off = (uint32_t)v & nmask;
    const uint32_t cm = dst.cm(limb);
    const uint64_t p = __ldg(&mods[cm].p);
    const ulonglong2 x = ld_pair(a.limb(limb, log_n) + off);
    uint64_t* d = dst.limb(limb, log_n) + off;
    uint64_t r0, r1;
    if (OP == (int)EwOp::kNegate) {
      r0 = p - x.x;
      r1 = p - x.y;
    } else {
      const ulonglong2 y = ld_pair(b.limb(limb, log_n) + off);
      if (OP == (int)EwOp::kAddmod) {
        r0 = addmod(x.x, y.x, p);
        r1 = addmod(x.y, y.y, p);
      } else if (OP == (int)EwOp::kSubmod) {
        r0 = submod(x.x, y.x, p);
        r1 = submod(x.y, y.y, p);
      } else {
        const uint64_t pn = __ldg(&mods[cm].pn);
        if (OP == (int)EwOp::kMulmod) {
          r0 = mulmod_barrett(x.x, y.x, p, pn);
          r1 = mulmod_barrett(x.y, y.y, p, pn);
        } else {
          const ulonglong2 acc = *reinterpret_cast<const ulonglong2*>(d);
          r0 = muladd_barrett(acc.x, x.x, y.x, p, pn);
          r1 = muladd_barrett(acc.y, x.y, y.y, p, pn);
        }
      }
    }
    st_pair(d, r0, r1);
  }
}

int g_num_sms = 0;

int num_sms() {
  if (g_num_sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_num_sms <= 0) g_num_sms = 1;
  }
  return g_num_sms;
}

std::vector<Variant> g_table[kMaxLogN + 1];
std::once_flag g_table_once;
std::array<std::array<std::atomic<uint8_t>, kMaxLogN + 1>, 64> g_selected{};

void build_table() {
  add_whole_variants_small(g_table);
  add_whole_variants_large(g_table);
  add_two_pass_variants_a(g_table);
  add_two_pass_variants_b(g_table);
  add_two_pass_variants_c(g_table);
  add_two_pass_variants_d(g_table);
  add_two_pass_variants_e(g_table);
}

int current_device() {
  int d = 0;
  cudaGetDevice(&d);
  return (d >= 0 && d < 64) ? d : 0;
}

const Variant& pick(uint32_t log_n) {
  const std::vector<Variant>& vs = variants_of(log_n);
  const uint32_t v = selected_variant(current_device(), log_n);
  return vs[v < vs.size() ? v : 0];
}

}  // namespace

const std::vector<Variant>& variants_of(uint32_t log_n) {
  std::call_once(g_table_once, build_table);
  return g_table[log_n];
}

uint32_t selected_variant(int device, uint32_t log_n) {
  return g_selected[device][log_n].load(std::memory_order_relaxed);
}

void select_variant(int device, uint32_t log_n, uint32_t v) {
  g_selected[device][log_n].store((uint8_t)v, std::memory_order_relaxed);
}

cudaError_t init_kernel_attributes() {
  for (uint32_t n = kMinLogN; n <= kMaxLogN; ++n)
    for (const Variant& v : variants_of(n)) {
      const cudaError_t e = v.set_attrs();
      if (e != cudaSuccess) return e;
    }
  return cudaSuccess;
}

uint32_t ntt_launch_count(uint32_t log_n, const NttShape&) { return pick(log_n).ntt_launches; }
uint32_t polymul_launch_count(uint32_t log_n, const NttShape&) { return pick(log_n).polymul_launches; }

// The words a polymul of this degree may need, whichever variant is selected
// (the selection can change between the caller's allocation and its call).
size_t polymul_scratch_words(uint32_t count, uint32_t log_n, const NttShape&) {
  if (log_n < kMinLogN || log_n > kMaxLogN) return 0;
  for (const Variant& v : variants_of(log_n))
    if (v.polymul_scratch) return (size_t)count << log_n;
  return 0;
}

// True when some variant of this degree runs its polymul without scratch.
bool polymul_scratch_optional(uint32_t log_n) {
  if (log_n < kMinLogN || log_n > kMaxLogN) return true;
  for (const Variant& v : variants_of(log_n))
    if (!v.polymul_scratch) return true;
  return false;
}

cudaError_t launch_ntt(const LimbSet& ls, uint32_t log_n, const DevMod* mods, NttDir dir,
                       const NttShape&, cudaStream_t st) {
  if (ls.count == 0) return cudaSuccess;
  if (log_n < kMinLogN || log_n > kMaxLogN) return cudaErrorInvalidValue;
  return pick(log_n).ntt(ls, mods, dir, st);
}

cudaError_t launch_polymul(const LimbSet& c, const ConstLimbSet& a, const ConstLimbSet& b,
                           uint32_t log_n, const DevMod* mods, uint64_t* scratch,
                           const NttShape&, cudaStream_t st, uint64_t* const* scratch_ptrs) {
  if (c.count == 0) return cudaSuccess;
  if (log_n < kMinLogN || log_n > kMaxLogN) return cudaErrorInvalidValue;
  const Variant* v = &pick(log_n);
  if (v->polymul_scratch && scratch == nullptr && scratch_ptrs == nullptr) {
    // Without scratch, the first (selection order) variant that needs none.
    v = nullptr;
    for (const Variant& w : variants_of(log_n))
      if (!w.polymul_scratch) {
        v = &w;
        break;
      }
    if (!v) return cudaErrorInvalidValue;
  }
  return v->polymul(c, a, b, mods, scratch, scratch_ptrs, st);
}

cudaError_t launch_elementwise(EwOp op, const LimbSet& dst, const ConstLimbSet& a,
                               const ConstLimbSet& b, uint32_t log_n, const DevMod* mods,
                               cudaStream_t st) {
  if (dst.count == 0) return cudaSuccess;
  const size_t pairs = ((size_t)dst.count << log_n) >> 1;
  const size_t want = (pairs + 255) / 256;
  const size_t cap = (size_t)num_sms() * 8;
  const uint32_t grid = (uint32_t)(want < cap ? want : cap);
  LaunchScope ps("elementwise", st);
  switch (op) {
    case EwOp::kMulmod: k_elementwise<0><<<grid, 256, 0, st>>>(dst, a, b, log_n, mods); break;
    case EwOp::kAddmod: k_elementwise<1><<<grid, 256, 0, st>>>(dst, a, b, log_n, mods); break;
    case EwOp::kSubmod: k_elementwise<2><<<grid, 256, 0, st>>>(dst, a, b, log_n, mods); break;
    case EwOp::kMuladd: k_elementwise<3><<<grid, 256, 0, st>>>(dst, a, b, log_n, mods); break;
    case EwOp::kNegate: k_elementwise<4><<<grid, 256, 0, st>>>(dst, a, b, log_n, mods); break;
  }
  g_kernel_launches += 1;
  return cudaGetLastError();
}

}  // namespace yell_gb300
