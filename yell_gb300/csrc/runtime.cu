// Host runtime of the YELL GB300 library: prime table, error reporting,
// twiddle-table construction and the per-device context.
#include "runtime.h"

#include <algorithm>
#include <array>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <thread>

namespace yell_gb300 {

namespace {

// {P, Pn, primitive 2^21-th root} per modulus index; generated by
// gen_prime_table.py from the rule stated in include/yell/params_64.hpp:16-38.
const PrimeEntry kPrimes[kMaxModuli] = {
#include "prime_table.inc"
};

thread_local std::string t_last_error;

using u128 = unsigned __int128;

inline uint64_t mulmod_exact(uint64_t a, uint64_t b, uint64_t p) {
  return (uint64_t)(((u128)a * b) % p);
}

uint64_t powmod(uint64_t b, uint64_t e, uint64_t p) {
  uint64_t r = 1;
  while (e) {
    if (e & 1) r = mulmod_exact(r, b, p);
    b = mulmod_exact(b, b, p);
    e >>= 1;
  }
  return r;
}

// floor(x * 2^64 / p), lib/ops.cpp:23-27.
inline uint64_t shoupify(uint64_t x, uint64_t p) { return (uint64_t)(((u128)x << 64) / p); }

// -p^-1 mod 2^64 for odd p (Newton's iteration doubles the correct low bits).
inline uint64_t neg_inv_mod_2_64(uint64_t p) {
  uint64_t x = p;  // p * p = 1 mod 8
  for (int i = 0; i < 5; ++i) x *= 2 - p * x;
  return 0 - x;
}

inline uint32_t bit_reverse(uint32_t x, uint32_t bits) {
  uint32_t r = 0;
  for (uint32_t i = 0; i < bits; ++i) r |= ((x >> i) & 1u) << (bits - 1 - i);
  return r;
}

}  // namespace

std::atomic<uint64_t> g_kernel_launches{0};
thread_local bool g_dependent_launches = true;
std::atomic<uint64_t> g_allocations{0};

const PrimeEntry& prime_entry(uint32_t cm) { return kPrimes[cm]; }

int fail(int code, const std::string& msg) {
  t_last_error = msg;
  return code;
}

int fail_cuda(cudaError_t e, const char* what) {
  const int code = (e == cudaErrorMemoryAllocation) ? kOutOfMemory
                   : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) ? kNoDevice
                                                                                  : kCudaError;
  return fail(code, std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")");
}

const char* last_error() { return t_last_error.c_str(); }
void clear_error() { t_last_error.clear(); }

int check_degree(uint32_t log_n) {
  if (log_n < kMinLogN || log_n > kMaxLogN)
    return fail(kUnsupportedDegree, "log_n " + std::to_string(log_n) + " outside [" +
                                        std::to_string(kMinLogN) + ", " + std::to_string(kMaxLogN) + "]");
  return kOk;
}

int check_moduli(uint32_t cm0, uint32_t L) {
  if (L == 0) return fail(kInvalidArgument, "limb count L is 0");
  if (cm0 >= kMaxModuli || L > kMaxModuli - cm0)
    return fail(kInvalidModulus, "moduli " + std::to_string(cm0) + ".." + std::to_string(cm0 + L - 1) +
                                     " exceed the table of " + std::to_string(kMaxModuli));
  return kOk;
}

int check_limbs(uint64_t count, uint32_t L, uint32_t log_n, uint32_t* limbs) {
  if (count == 0) return fail(kInvalidArgument, "zero polys or pairs");
  const uint64_t total = count * (uint64_t)L;  // count < 2^32, L <= kMaxModuli: no wrap
  // One launch covers every limb: the grid (limbs, or 4096-word tiles of
  // larger limbs) must stay below 2^31 blocks.
  const uint32_t shift = log_n > 12 ? log_n - 12 : 0;
  const uint64_t max_limbs = ((uint64_t(1) << 31) - 1) >> shift;
  if (total > max_limbs)
    return fail(kInvalidArgument, std::to_string(count) + " x " + std::to_string(L) + " = " +
                                      std::to_string(total) + " limbs of degree 2^" + std::to_string(log_n) +
                                      " exceed the " + std::to_string(max_limbs) + " one call can take");
  if (limbs) *limbs = (uint32_t)total;
  return kOk;
}

// The values are the reference's (include/yell/details/ntt.hpp:97-146); they
// are canonical residues, so exact u128 arithmetic reproduces them.
void build_host_tables(uint32_t log_n, uint32_t cm, uint64_t* out4n, uint64_t* sc4) {
  const PrimeEntry& pe = kPrimes[cm];
  const uint64_t p = pe.p;
  const uint32_t n = 1u << log_n;
  // include/yell/details/ntt.hpp:39-43: psi = root^(2^(20 - log_n)), a primitive 2N-th root.
  uint64_t psi = pe.root;
  for (uint32_t i = 0; i < kLogMaxDegree - log_n; ++i) psi = mulmod_exact(psi, psi, p);
  // include/yell/details/ntt.hpp:57-58: invphi = psi^N * psi^(N-1) = psi^(2N-1).
  const uint64_t ipsi = powmod(psi, 2ull * n - 1, p);
  uint64_t* phi = out4n;
  uint64_t* phi_s = out4n + n;
  uint64_t* iphi = out4n + 2 * (size_t)n;
  uint64_t* iphi_s = out4n + 3 * (size_t)n;
  uint64_t a = 1, b = 1;
  for (uint32_t i = 0; i < n; ++i) {
    // include/yell/details/ntt.hpp:45-71: powers, Shoup forms, then bit-reversed order.
    const uint32_t r = bit_reverse(i, log_n);
    phi[r] = a;
    phi_s[r] = shoupify(a, p);
    iphi[r] = b;
    iphi_s[r] = shoupify(b, p);
    a = mulmod_exact(a, psi, p);
    b = mulmod_exact(b, ipsi, p);
  }
  // include/yell/details/ntt.hpp:73-76
  const uint64_t inv_n = powmod(n % p, p - 2, p);
  const uint64_t inv_n_iphi = mulmod_exact(inv_n, iphi[1], p);
  sc4[0] = inv_n;
  sc4[1] = shoupify(inv_n, p);
  sc4[2] = inv_n_iphi;
  sc4[3] = shoupify(inv_n_iphi, p);
}

// ---------------------------------------------------------------------------

DeviceContext::Buffer::~Buffer() {
  // Device memory is released at process exit by the driver; freeing here
  // could run after the CUDA runtime has been torn down.
}

int DeviceContext::Buffer::reserve(size_t w) {
  if (w <= words) return kOk;
  if (ptr) {
    cudaError_t e = cudaFree(ptr);
    ptr = nullptr;
    words = 0;
    if (e != cudaSuccess) return fail_cuda(e, "cudaFree(buffer)");
  }
  cudaError_t e = lib_malloc(&ptr, w * sizeof(uint64_t));
  if (e != cudaSuccess) {
    ptr = nullptr;
    return fail_cuda(e, "cudaMalloc(buffer)");
  }
  words = w;
  return kOk;
}

int DeviceContext::HostMapped::ensure() {
  if (host) return kOk;
  void* h = nullptr;
  cudaError_t e = lib_malloc_host(&h, 3 * kSmallCallWords * sizeof(uint64_t), cudaHostAllocMapped);
  if (e != cudaSuccess) return fail_cuda(e, "cudaHostAlloc(small-call buffer)");
  void* d = nullptr;
  e = cudaHostGetDevicePointer(&d, h, 0);
  if (e != cudaSuccess) {
    cudaFreeHost(h);
    return fail_cuda(e, "cudaHostGetDevicePointer(small-call buffer)");
  }
  host = static_cast<uint64_t*>(h);
  dev = static_cast<uint64_t*>(d);
  return kOk;
}

DeviceContext::DeviceContext(int device) : device_(device) {}

int DeviceContext::scratch_alloc_async(size_t words, cudaStream_t st, uint64_t** out) {
  const cudaError_t e = lib_malloc_async(out, words * sizeof(uint64_t), pool_, st);
  if (e != cudaSuccess) {
    *out = nullptr;
    return fail_cuda(e, "cudaMallocFromPoolAsync(polymul scratch)");
  }
  return kOk;
}

int DeviceContext::scratch_free_async(uint64_t* p, cudaStream_t st) {
  const cudaError_t e = cudaFreeAsync(p, st);
  return e == cudaSuccess ? kOk : fail_cuda(e, "cudaFreeAsync(polymul scratch)");
}

int DeviceContext::init() {
  cudaError_t e = cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking);
  if (e != cudaSuccess) return fail_cuda(e, "cudaStreamCreate");
  for (int i = 0; i < 3; ++i) {
    e = cudaStreamCreateWithFlags(&pipe_stream[i], cudaStreamNonBlocking);
    if (e != cudaSuccess) return fail_cuda(e, "cudaStreamCreate(pipe)");
  }
  for (int i = 0; i < kPipeSlots; ++i) {
    cudaEvent_t* evs[] = {&pipe_h2d[i], &pipe_comp[i], &pipe_d2h[i]};
    for (cudaEvent_t* ev : evs) {
      e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
      if (e != cudaSuccess) return fail_cuda(e, "cudaEventCreate(pipe)");
    }
  }
  cudaMemPoolProps props = {};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = device_;
  e = cudaMemPoolCreate(&pool_, &props);
  if (e != cudaSuccess) return fail_cuda(e, "cudaMemPoolCreate");
  uint64_t keep = ~uint64_t(0);
  e = cudaMemPoolSetAttribute(pool_, cudaMemPoolAttrReleaseThreshold, &keep);
  if (e != cudaSuccess) return fail_cuda(e, "cudaMemPoolSetAttribute");
  e = init_kernel_attributes();
  if (e != cudaSuccess) return fail_cuda(e, "cudaFuncSetAttribute");
  load_tuning(device_);
  int pageable = 0, host_tables = 0;
  if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device_) == cudaSuccess &&
      cudaDeviceGetAttribute(&host_tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device_) ==
          cudaSuccess)
    pageable_access_ = pageable == 1 && host_tables == 1;
  return kOk;
}

std::atomic<bool> g_host_access{true};

bool DeviceContext::host_access() const { return pageable_access_ && g_host_access.load(std::memory_order_relaxed); }

DeviceContext* DeviceContext::current(int* status) {
  static std::mutex mu;
  static std::array<std::unique_ptr<DeviceContext>, 64> ctxs;
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 64) {
    *status = fail_cuda(e == cudaSuccess ? cudaErrorInvalidDevice : e, "cudaGetDevice");
    return nullptr;
  }
  std::lock_guard<std::mutex> g(mu);
  if (!ctxs[dev]) {
    std::unique_ptr<DeviceContext> c(new DeviceContext(dev));
    int st = c->init();
    if (st != kOk) {
      *status = st;
      return nullptr;
    }
    ctxs[dev] = std::move(c);
  }
  *status = kOk;
  return ctxs[dev].get();
}

const DevMod* DeviceContext::mods_if_ready(uint32_t log_n) const {
  std::lock_guard<std::mutex> g(tables_mu_);
  return d_mods_[log_n];
}

const DevMod* DeviceContext::tables_ready(uint32_t log_n, uint32_t cm0, uint32_t L) const {
  std::lock_guard<std::mutex> g(tables_mu_);
  const std::vector<uint8_t>& built = built_[log_n];
  if (built.empty() || !d_mods_[log_n]) return nullptr;
  for (uint32_t i = 0; i < L; ++i)
    if (built[cm0 + i] != 1) return nullptr;
  return d_mods_[log_n];
}

int DeviceContext::ensure_tables(uint32_t log_n, uint32_t cm0, uint32_t L, const DevMod** mods) {
  std::vector<uint32_t> cms(L);
  for (uint32_t i = 0; i < L; ++i) cms[i] = cm0 + i;
  return ensure_tables_list(log_n, cms.data(), L, mods);
}

int DeviceContext::ensure_tables_list(uint32_t log_n, const uint32_t* cms, uint32_t n,
                                      const DevMod** mods) {
  std::lock_guard<std::mutex> g(tables_mu_);
  std::vector<uint8_t>& built = built_[log_n];
  if (built.empty()) built.assign(kMaxModuli, 0);
  std::vector<uint32_t> missing;
  for (uint32_t i = 0; i < n; ++i) {
    if (cms[i] >= kMaxModuli) return fail(kInvalidModulus, "modulus index out of range");
    if (!built[cms[i]]) {
      built[cms[i]] = 2;  // mark as pending so duplicates in the list build once
      missing.push_back(cms[i]);
    }
  }
  if (missing.empty()) {
    *mods = d_mods_[log_n];
    return kOk;
  }
  for (uint32_t cm : missing) built[cm] = 0;
  // Tables are built only here, and yell_dev_polymul_noalloc requires them:
  // bring up its fixed scratch array now, while allocating is allowed.
  const int nst = noalloc_prepare(device_);
  if (nst != kOk) return nst;
  cudaError_t e;
  static_assert(kPolymulConsts == kMaxModuli, "the polymul constants follow the transforms'");
  if (!d_mods_[log_n]) {
    e = lib_malloc(&d_mods_[log_n], 2 * kMaxModuli * sizeof(DevMod));
    if (e != cudaSuccess) {
      d_mods_[log_n] = nullptr;
      return fail_cuda(e, "cudaMalloc(DevMod table)");
    }
    e = cudaMemset(d_mods_[log_n], 0, 2 * kMaxModuli * sizeof(DevMod));
    if (e != cudaSuccess) return fail_cuda(e, "cudaMemset(DevMod table)");
  }
  const uint32_t nwords = 1u << log_n;
  // Build the missing tables on host threads (independent per modulus).
  const size_t per = 4 * (size_t)nwords;
  std::vector<uint64_t> host(per * missing.size());
  std::vector<uint64_t> sc(4 * missing.size());
  const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  const unsigned nth = std::min<unsigned>(hw, (unsigned)missing.size());
  auto work = [&](unsigned t) {
    for (size_t i = t; i < missing.size(); i += nth)
      build_host_tables(log_n, missing[i], host.data() + i * per, sc.data() + 4 * i);
  };
  if (nth <= 1 || nwords < 1024) {
    for (size_t i = 0; i < missing.size(); ++i)
      build_host_tables(log_n, missing[i], host.data() + i * per, sc.data() + 4 * i);
  } else {
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nth; ++t) th.emplace_back(work, t);
    for (auto& t : th) t.join();
  }
  // Interleave {w, w'} pairs for 128-bit loads: fwd then inv, N pairs each.
  std::vector<uint64_t> packed(4 * (size_t)nwords);
  for (size_t i = 0; i < missing.size(); ++i) {
    const uint32_t cm = missing[i];
    const uint64_t* t = host.data() + i * per;
    for (uint32_t k = 0; k < nwords; ++k) {
      packed[2 * (size_t)k] = t[k];
      packed[2 * (size_t)k + 1] = t[nwords + k];
      packed[2 * (size_t)nwords + 2 * (size_t)k] = t[2 * (size_t)nwords + k];
      packed[2 * (size_t)nwords + 2 * (size_t)k + 1] = t[3 * (size_t)nwords + k];
    }
    void* dtab = nullptr;
    e = lib_malloc(&dtab, packed.size() * sizeof(uint64_t));
    if (e != cudaSuccess) return fail_cuda(e, "cudaMalloc(twiddle table)");
    table_allocs_.push_back(dtab);
    e = cudaMemcpy(dtab, packed.data(), packed.size() * sizeof(uint64_t), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail_cuda(e, "cudaMemcpy(twiddle table)");
    DevMod m;
    m.fwd = reinterpret_cast<const ulonglong2*>(dtab);
    m.inv = reinterpret_cast<const ulonglong2*>(dtab) + nwords;
    m.p = kPrimes[cm].p;
    m.pn = kPrimes[cm].pn;
    m.inv_n = sc[4 * i + 0];
    m.inv_n_s = sc[4 * i + 1];
    m.inv_n_iphi = sc[4 * i + 2];
    m.inv_n_iphi_s = sc[4 * i + 3];
    e = cudaMemcpy(d_mods_[log_n] + cm, &m, sizeof(DevMod), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail_cuda(e, "cudaMemcpy(DevMod)");
    // the fused polymul's copy: Montgomery constant, inverse scaling times 2^64
    DevMod pm = m;
    const uint64_t r64 = (uint64_t)(((u128)1 << 64) % m.p);
    pm.pn = neg_inv_mod_2_64(m.p);
    pm.inv_n = mulmod_exact(m.inv_n, r64, m.p);
    pm.inv_n_s = shoupify(pm.inv_n, m.p);
    pm.inv_n_iphi = mulmod_exact(m.inv_n_iphi, r64, m.p);
    pm.inv_n_iphi_s = shoupify(pm.inv_n_iphi, m.p);
    e = cudaMemcpy(d_mods_[log_n] + kPolymulConsts + cm, &pm, sizeof(DevMod), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail_cuda(e, "cudaMemcpy(DevMod)");
    built[cm] = 1;
  }
  *mods = d_mods_[log_n];
  return kOk;
}

}  // namespace yell_gb300
