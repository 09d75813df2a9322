// extern "C" boundary of the library (declared in include/yell_gb300.h).
#include "yell_gb300.h"

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "kernels.h"
#include "profiler.h"
#include "runtime.h"

using namespace yell_gb300;

namespace {

inline cudaStream_t pick_stream(DeviceContext* ctx, void* stream) {
  return stream ? static_cast<cudaStream_t>(stream) : ctx->stream();
}

#define YELL_TRY(expr)          \
  do {                          \
    const int st_ = (expr);     \
    if (st_ != kOk) return st_; \
  } while (0)

#define YELL_CUDA(expr, what)                           \
  do {                                                  \
    const cudaError_t e_ = (expr);                      \
    if (e_ != cudaSuccess) return fail_cuda(e_, what);  \
  } while (0)

int get_ctx(DeviceContext** out) {
  int st = kOk;
  *out = DeviceContext::current(&st);
  return st;
}

LimbSet contiguous(uint64_t* base, uint32_t count, uint32_t L, uint32_t cm0) {
  LimbSet s;
  s.base = base;
  s.ptrs = nullptr;
  s.cms = nullptr;
  s.count = count;
  s.L = L;
  s.cm0 = cm0;
  s.pad_ = 0;
  return s;
}

ConstLimbSet const_contiguous(const uint64_t* base, uint32_t count, uint32_t L, uint32_t cm0) {
  ConstLimbSet s;
  s.base = base;
  s.ptrs = nullptr;
  s.cms = nullptr;
  s.count = count;
  s.L = L;
  s.cm0 = cm0;
  s.pad_ = 0;
  return s;
}

NttDir to_dir(int d) { return static_cast<NttDir>(d); }

// The kernels move words in 16-byte pairs, so every device base address must
// be 16-byte aligned (limb offsets are multiples of N >= 8 words).
int check_aligned(const void* p, const char* what) {
  if (reinterpret_cast<uintptr_t>(p) % 16 != 0)
    return fail(kInvalidArgument, std::string(what) + " is not 16-byte aligned");
  return kOk;
}

// A contiguous host operand that kernels should access in place: the device
// reaches pageable memory through the host's page tables and the operand is
// pageable (pinned memory copies as fast by DMA) and 16-byte aligned.
bool direct_host(DeviceContext* ctx, const void* p) { return ctx->host_access() && pageable_host(p); }

// Host-memory drop-in: copy L limbs (separate host arrays) into the context's
// staging area, run `body`, copy `nout` result limb sets back, synchronise.
// Holds the staging lock for the whole call.
int host_ntt(uint64_t* const* limbs, uint32_t L, uint32_t log_n, uint32_t cm0, NttDir dir) {
  if (!limbs) return fail(kInvalidArgument, "null limb array");
  YELL_TRY(check_degree(log_n));
  YELL_TRY(check_moduli(cm0, L));
  for (uint32_t i = 0; i < L; ++i)
    if (!limbs[i]) return fail(kInvalidArgument, "null limb pointer");
  DeviceContext* ctx;
  YELL_TRY(get_ctx(&ctx));
  const DevMod* mods;
  YELL_TRY(ctx->ensure_tables(log_n, cm0, L, &mods));
  const size_t n = (size_t)1 << log_n;
  cudaStream_t st = ctx->stream();
  if (n * L <= DeviceContext::kSmallCallWords && ntt_launch_count(log_n, ctx->shape) == 1) {
    // small call: one whole-limb launch in place on the mapped host buffer
    std::lock_guard<std::mutex> g(ctx->small.lock);
    YELL_TRY(ctx->small.ensure());
    for (uint32_t i = 0; i < L; ++i) std::memcpy(ctx->small.host + i * n, limbs[i], n * 8);
    YELL_CUDA(launch_ntt(contiguous(ctx->small.dev, L, L, cm0), log_n, mods, dir, ctx->shape, st), "launch ntt");
    YELL_CUDA(cudaStreamSynchronize(st), "synchronize");
    for (uint32_t i = 0; i < L; ++i) std::memcpy(limbs[i], ctx->small.host + i * n, n * 8);
    return kOk;
  }
  std::lock_guard<std::mutex> g(ctx->staging.lock);
  YELL_TRY(ctx->staging.reserve(n * L));
  uint64_t* d = ctx->staging.ptr;
  // the limbs move by kernels that read and write the host memory where it
  // lies when the device can, else by copies through the driver
  const bool direct = ctx->host_access() && host_limbs_accessible(limbs, L);
  if (direct) {
    YELL_CUDA(gather_host_limbs(d, limbs, L, log_n, st), "gather host limbs");
  } else {
    for (uint32_t i = 0; i < L; ++i)
      YELL_CUDA(cudaMemcpyAsync(d + i * n, limbs[i], n * 8, cudaMemcpyHostToDevice, st), "H2D limb");
  }
  YELL_CUDA(launch_ntt(contiguous(d, L, L, cm0), log_n, mods, dir, ctx->shape, st), "launch ntt");
  if (direct) {
    YELL_CUDA(scatter_host_limbs(limbs, d, L, log_n, st), "scatter host limbs");
  } else {
    for (uint32_t i = 0; i < L; ++i)
      YELL_CUDA(cudaMemcpyAsync(limbs[i], d + i * n, n * 8, cudaMemcpyDeviceToHost, st), "D2H limb");
  }
  YELL_CUDA(cudaStreamSynchronize(st), "synchronize");
  return kOk;
}

int host_elementwise(EwOp op, uint64_t* const* dst, const uint64_t* const* a,
                     const uint64_t* const* b, uint32_t L, uint32_t log_n) {
  if (!dst || !a || (op != EwOp::kNegate && !b)) return fail(kInvalidArgument, "null limb array");
  YELL_TRY(check_degree(log_n));
  YELL_TRY(check_moduli(0, L));
  for (uint32_t i = 0; i < L; ++i)
    if (!dst[i] || !a[i] || (op != EwOp::kNegate && !b[i]))
      return fail(kInvalidArgument, "null limb pointer");
  DeviceContext* ctx;
  YELL_TRY(get_ctx(&ctx));
  const DevMod* mods;
  YELL_TRY(ctx->ensure_tables(log_n, 0, L, &mods));
  const size_t n = (size_t)1 << log_n;
  const size_t w = n * L;
  cudaStream_t st = ctx->stream();
  if (w <= DeviceContext::kSmallCallWords) {
    // small call: the kernel reads and writes the mapped host buffer
    std::lock_guard<std::mutex> g(ctx->small.lock);
    YELL_TRY(ctx->small.ensure());
    uint64_t* ha = ctx->small.host;
    uint64_t* hb = ha + w;
    uint64_t* hd = hb + w;
    for (uint32_t i = 0; i < L; ++i) {
      std::memcpy(ha + i * n, a[i], n * 8);
      if (op != EwOp::kNegate) std::memcpy(hb + i * n, b[i], n * 8);
      if (op == EwOp::kMuladd) std::memcpy(hd + i * n, dst[i], n * 8);
    }
    uint64_t* va = ctx->small.dev;
    YELL_CUDA(launch_elementwise(op, contiguous(va + 2 * w, L, L, 0), const_contiguous(va, L, L, 0),
                                 const_contiguous(va + w, L, L, 0), log_n, mods, st),
              "launch elementwise");
    YELL_CUDA(cudaStreamSynchronize(st), "synchronize");
    for (uint32_t i = 0; i < L; ++i) std::memcpy(dst[i], hd + i * n, n * 8);
    return kOk;
  }
  std::lock_guard<std::mutex> g(ctx->staging.lock);
  YELL_TRY(ctx->staging.reserve(3 * w));
  uint64_t* da = ctx->staging.ptr;
  uint64_t* db = da + w;
  uint64_t* dd = db + w;
  const bool direct = ctx->host_access() && host_limbs_accessible(dst, L) && host_limbs_accessible(a, L) &&
                      (op == EwOp::kNegate || host_limbs_accessible(b, L));
  if (direct) {
    YELL_CUDA(gather_host_limbs(da, a, L, log_n, st), "gather a");
    if (op != EwOp::kNegate) YELL_CUDA(gather_host_limbs(db, b, L, log_n, st), "gather b");
    if (op == EwOp::kMuladd) YELL_CUDA(gather_host_limbs(dd, dst, L, log_n, st), "gather acc");
  } else {
    for (uint32_t i = 0; i < L; ++i) {
      YELL_CUDA(cudaMemcpyAsync(da + i * n, a[i], n * 8, cudaMemcpyHostToDevice, st), "H2D a");
      if (op != EwOp::kNegate)
        YELL_CUDA(cudaMemcpyAsync(db + i * n, b[i], n * 8, cudaMemcpyHostToDevice, st), "H2D b");
      if (op == EwOp::kMuladd)
        YELL_CUDA(cudaMemcpyAsync(dd + i * n, dst[i], n * 8, cudaMemcpyHostToDevice, st), "H2D acc");
    }
  }
  YELL_CUDA(launch_elementwise(op, contiguous(dd, L, L, 0), const_contiguous(da, L, L, 0),
                               const_contiguous(db, L, L, 0), log_n, mods, st),
            "launch elementwise");
  if (direct) {
    YELL_CUDA(scatter_host_limbs(dst, dd, L, log_n, st), "scatter result");
  } else {
    for (uint32_t i = 0; i < L; ++i)
      YELL_CUDA(cudaMemcpyAsync(dst[i], dd + i * n, n * 8, cudaMemcpyDeviceToHost, st), "D2H");
  }
  YELL_CUDA(cudaStreamSynchronize(st), "synchronize");
  return kOk;
}

}  // namespace

extern "C" {

int yell_abi_version(void) { return YELL_GB300_ABI_VERSION; }

const char* yell_status_string(int status) {
  switch (status) {
    case YELL_OK: return "ok";
    case YELL_ERR_INVALID_ARGUMENT: return "invalid argument";
    case YELL_ERR_UNSUPPORTED_DEGREE: return "unsupported degree";
    case YELL_ERR_INVALID_MODULUS: return "invalid modulus index";
    case YELL_ERR_CUDA: return "CUDA error";
    case YELL_ERR_OUT_OF_MEMORY: return "out of memory";
    case YELL_ERR_BUDGET: return "HBM budget exceeded";
    case YELL_ERR_TIMEOUT: return "timed out";
    case YELL_ERR_CANCELLED: return "cancelled";
    case YELL_ERR_NOT_FOUND: return "not found";
    case YELL_ERR_NO_DEVICE: return "no CUDA device";
    default: return "unknown status";
  }
}

const char* yell_last_error(void) { return last_error(); }
uint64_t yell_kernel_launches(void) { return g_kernel_launches.load(); }

uint64_t yell_allocations(void) { return g_allocations.load(); }

uint32_t yell_max_moduli(void) { return kMaxModuli; }
uint32_t yell_min_log_degree(void) { return kMinLogN; }
uint32_t yell_max_log_degree(void) { return kMaxLogN; }
uint64_t yell_prime(uint32_t cm) { return cm < kMaxModuli ? prime_entry(cm).p : 0; }
uint64_t yell_prime_pn(uint32_t cm) { return cm < kMaxModuli ? prime_entry(cm).pn : 0; }
uint64_t yell_primitive_root(uint32_t cm) { return cm < kMaxModuli ? prime_entry(cm).root : 0; }

int yell_init_table(uint32_t log_n, uint32_t cm) { return yell_init_ntt_tables_range(log_n, cm, 1); }

int yell_init_ntt_tables(uint32_t log_n, uint32_t K) { return yell_init_ntt_tables_range(log_n, 0, K); }

int yell_init_ntt_tables_range(uint32_t log_n, uint32_t cm0, uint32_t L) {
  YELL_TRY(check_degree(log_n));
  YELL_TRY(check_moduli(cm0, L));
  DeviceContext* ctx;
  YELL_TRY(get_ctx(&ctx));
  const DevMod* mods;
  return ctx->ensure_tables(log_n, cm0, L, &mods);
}

int yell_ntt_tables(uint32_t log_n, uint32_t cm, uint64_t* out4n, uint64_t* scalars4) {
  if (!out4n || !scalars4) return fail(kInvalidArgument, "null output");
  YELL_TRY(check_degree(log_n));
  YELL_TRY(check_moduli(cm, 1));
  build_host_tables(log_n, cm, out4n, scalars4);
  return kOk;
}

int yell_ntt_forward(uint64_t* op, uint32_t log_n, uint32_t cm) {
  return host_ntt(&op, 1, log_n, cm, NttDir::kForward);
}
int yell_ntt_forward_lazy(uint64_t* op, uint32_t log_n, uint32_t cm) {
  return host_ntt(&op, 1, log_n, cm, NttDir::kForwardLazy);
}
int yell_ntt_backward(uint64_t* op, uint32_t log_n, uint32_t cm) {
  return host_ntt(&op, 1, log_n, cm, NttDir::kBackward);
}

int yell_poly_forward(uint64_t* const* limbs, uint32_t L, uint32_t log_n) {
  return host_ntt(limbs, L, log_n, 0, NttDir::kForward);
}
int yell_poly_forward_lazy(uint64_t* const* limbs, uint32_t L, uint32_t log_n) {
  return host_ntt(limbs, L, log_n, 0, NttDir::kForwardLazy);
}
int yell_poly_backward(uint64_t* const* limbs, uint32_t L, uint32_t log_n) {
  return host_ntt(limbs, L, log_n, 0, NttDir::kBackward);
}

int yell_poly_mulmod(uint64_t* const* dst, const uint64_t* const* a, const uint64_t* const* b,
                     uint32_t L, uint32_t log_n) {
  return host_elementwise(EwOp::kMulmod, dst, a, b, L, log_n);
}
int yell_poly_addmod(uint64_t* const* dst, const uint64_t* const* a, const uint64_t* const* b,
                     uint32_t L, uint32_t log_n) {
  return host_elementwise(EwOp::kAddmod, dst, a, b, L, log_n);
}
int yell_poly_submod(uint64_t* const* dst, const uint64_t* const* a, const uint64_t* const* b,
                     uint32_t L, uint32_t log_n) {
  return host_elementwise(EwOp::kSubmod, dst, a, b, L, log_n);
}
int yell_poly_add_product_of(uint64_t* const* acc, const uint64_t* const* a,
                             const uint64_t* const* b, uint32_t L, uint32_t log_n) {
  return host_elementwise(EwOp::kMuladd, acc, a, b, L, log_n);
}
int yell_poly_negate(uint64_t* const* limbs, uint32_t L, uint32_t log_n) {
  return host_elementwise(EwOp::kNegate, limbs, limbs, nullptr, L, log_n);
}

int yell_set_host_access(int enable) {
  g_host_access.store(enable != 0);
  return kOk;
}

int yell_host_access(int* in_use) {
  if (!in_use) return fail(kInvalidArgument, "null output");
  DeviceContext* ctx;
  YELL_TRY(get_ctx(&ctx));
  *in_use = ctx->host_access() ? 1 : 0;
  return kOk;
}

void* yell_host_alloc(size_t bytes) {
  void* p = nullptr;
  if (lib_malloc_host(&p, bytes) != cudaSuccess) return nullptr;
  return p;
}

void yell_host_free(void* p) {
  if (p) cudaFreeHost(p);
}

// Pipelined host polymul: chunks of whole pairs move through three streams
// (H2D, compute, D2H) using kPipeSlots device buffer sets in turn, so the
// copy engines move chunk k+1 in and chunk k-1 out while chunk k computes.
// Reusing a slot waits (on the GPU) for the compute that read its operands
// and for the copy-out that read its product.
int yell_polymul_host(uint64_t* c, const uint64_t* a, const uint64_t* b, uint32_t pairs,
                      uint32_t L, uint32_t log_n, uint32_t cm0) {
  TraceRange trace("yell polymul_host");
  if (!c || !a || !b) return fail(kInvalidArgument, "null pointer");
  if (pairs == 0) return fail(kInvalidArgument, "pairs is 0");
  YELL_TRY(check_degree(log_n));
  YELL_TRY(check_moduli(cm0, L));
  YELL_TRY(check_limbs(pairs, L, log_n, nullptr));
  DeviceContext* ctx;
  YELL_TRY(get_ctx(&ctx));
  const DevMod* mods;
  YELL_TRY(ctx->ensure_tables(log_n, cm0, L, &mods));
  const size_t pair_words = ((size_t)L) << log_n;
  if ((size_t)pairs * pair_words <= DeviceContext::kSmallCallWords &&
      polymul_launch_count(log_n, ctx->shape) == 1) {
    // small call: one whole-limb launch on the mapped host buffer
    const size_t w = (size_t)pairs * pair_words;
    std::lock_guard<std::mutex> g(ctx->small.lock);
    YELL_TRY(ctx->small.ensure());
    std::memcpy(ctx->small.host, a, w * 8);
    std::memcpy(ctx->small.host + w, b, w * 8);
    uint64_t* va = ctx->small.dev;
    cudaStream_t st = ctx->stream();
    YELL_CUDA(launch_polymul(contiguous(va + 2 * w, pairs * L, L, cm0), const_contiguous(va, pairs * L, L, cm0),
                             const_contiguous(va + w, pairs * L, L, cm0), log_n, mods, nullptr, ctx->shape, st),
              "launch polymul");
    YELL_CUDA(cudaStreamSynchronize(st), "synchronize");
    std::memcpy(c, ctx->small.host + 2 * w, w * 8);
    return kOk;
  }
  // ~64 MiB of operands per chunk, at least one pair.
  const size_t target = (64ull << 20) / 8;
  uint32_t cp = (uint32_t)std::max<size_t>(1, target / (2 * pair_words));
  if (cp > pairs) cp = pairs;
  const size_t cw = cp * pair_words;
  const size_t sw = polymul_scratch_words(cp * L, log_n, ctx->shape);
  std::lock_guard<std::mutex> g(ctx->pipe_lock);
  for (int s = 0; s < DeviceContext::kPipeSlots; ++s) {
    std::lock_guard<std::mutex> gb(ctx->pipe_buf[s].lock);
    YELL_TRY(ctx->pipe_buf[s].reserve(3 * cw + sw));
  }
  cudaStream_t h2d = ctx->pipe_stream[0], comp = ctx->pipe_stream[1], d2h = ctx->pipe_stream[2];
  // Pageable operands move by kernels that access them in place where the
  // device can (copies from pageable memory run through driver staging at a
  // sixth of the link's rate); pinned ones by the copy engines.
  const bool dir_a = direct_host(ctx, a), dir_b = direct_host(ctx, b), dir_c = direct_host(ctx, c);
  auto copy_in = [&](uint64_t* dst, const uint64_t* src, size_t words, bool direct) {
    return direct ? gather_host_contiguous(dst, src, (uint32_t)(words >> log_n), log_n, h2d)
                  : cudaMemcpyAsync(dst, src, words * 8, cudaMemcpyHostToDevice, h2d);
  };
  auto copy_out = [&](uint64_t* dst, const uint64_t* src, size_t words) {
    return dir_c ? scatter_host_contiguous(dst, src, (uint32_t)(words >> log_n), log_n, d2h)
                 : cudaMemcpyAsync(dst, src, words * 8, cudaMemcpyDeviceToHost, d2h);
  };
  uint32_t k = 0;
  for (uint32_t p0 = 0, np = 0; p0 < pairs; p0 += np, ++k) {
    const int s = (int)(k % DeviceContext::kPipeSlots);
    const bool reuse = k >= (uint32_t)DeviceContext::kPipeSlots;
    // the last cp pairs go one at a time: the compute and D2H left after the
    // final H2D (the pipeline's tail) then cover one pair, not cp
    np = pairs - p0 > cp ? cp : 1;
    const size_t w = np * pair_words;
    uint64_t* da = ctx->pipe_buf[s].ptr;
    uint64_t* db = da + cw;
    uint64_t* dc = db + cw;
    uint64_t* ds = dc + cw;
    if (reuse) YELL_CUDA(cudaStreamWaitEvent(h2d, ctx->pipe_comp[s], 0), "pipe order");
    YELL_CUDA(copy_in(da, a + p0 * pair_words, w, dir_a), "H2D a");
    YELL_CUDA(copy_in(db, b + p0 * pair_words, w, dir_b), "H2D b");
    YELL_CUDA(cudaEventRecord(ctx->pipe_h2d[s], h2d), "pipe event");
    YELL_CUDA(cudaStreamWaitEvent(comp, ctx->pipe_h2d[s], 0), "pipe order");
    if (reuse) YELL_CUDA(cudaStreamWaitEvent(comp, ctx->pipe_d2h[s], 0), "pipe order");
    YELL_CUDA(launch_polymul(contiguous(dc, np * L, L, cm0), const_contiguous(da, np * L, L, cm0),
                             const_contiguous(db, np * L, L, cm0), log_n, mods, sw ? ds : nullptr,
                             ctx->shape, comp),
              "launch polymul");
    YELL_CUDA(cudaEventRecord(ctx->pipe_comp[s], comp), "pipe event");
    YELL_CUDA(cudaStreamWaitEvent(d2h, ctx->pipe_comp[s], 0), "pipe order");
    YELL_CUDA(copy_out(c + p0 * pair_words, dc, w), "D2H c");
    YELL_CUDA(cudaEventRecord(ctx->pipe_d2h[s], d2h), "pipe event");
  }
  for (int i = 0; i < 3; ++i) YELL_CUDA(cudaStreamSynchronize(ctx->pipe_stream[i]), "synchronize");
  return kOk;
}

int yell_dev_ntt(uint64_t* d_polys, uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0,
                 int direction, void* stream) {
  if (!d_polys || count == 0) return fail(kInvalidArgument, "null pointer or zero count");
  if (direction < 0 || direction > 2) return fail(kInvalidArgument, "bad direction");
  YELL_TRY(check_aligned(d_polys, "d_polys"));
  YELL_TRY(check_degree(log_n));
  YELL_TRY(check_moduli(cm0, L));
  uint32_t limbs;
  YELL_TRY(check_limbs(count, L, log_n, &limbs));
  DeviceContext* ctx;
  YELL_TRY(get_ctx(&ctx));
  const DevMod* mods;
  YELL_TRY(ctx->ensure_tables(log_n, cm0, L, &mods));
  YELL_CUDA(launch_ntt(contiguous(d_polys, limbs, L, cm0), log_n, mods, to_dir(direction),
                       ctx->shape, pick_stream(ctx, stream)),
            "launch ntt");
  return kOk;
}

int yell_dev_ntt_limbs(uint64_t* const* d_limbs, const uint32_t* d_cms, uint32_t count,
                       uint32_t log_n, int direction, void* stream) {
  if (!d_limbs || !d_cms || count == 0) return fail(kInvalidArgument, "null pointer or zero count");
  if (direction < 0 || direction > 2) return fail(kInvalidArgument, "bad direction");
  YELL_TRY(check_degree(log_n));
  DeviceContext* ctx;
  YELL_TRY(get_ctx(&ctx));
  cudaStream_t st = pick_stream(ctx, stream);
  // The modulus list and the limb addresses are checked on the host: tables
  // must exist for every modulus and every limb must be 16-byte aligned.
  std::vector<uint32_t> cms(count);
  std::vector<uintptr_t> addrs(count);
  YELL_CUDA(cudaMemcpyAsync(cms.data(), d_cms, count * sizeof(uint32_t), cudaMemcpyDeviceToHost, st),
            "D2H modulus list");
  YELL_CUDA(cudaMemcpyAsync(addrs.data(), d_limbs, count * sizeof(uintptr_t), cudaMemcpyDeviceToHost,
                            st),
            "D2H limb list");
  YELL_CUDA(cudaStreamSynchronize(st), "synchronize");
  for (uint32_t i = 0; i < count; ++i) {
    if (addrs[i] == 0) return fail(kInvalidArgument, "null limb pointer");
    YELL_TRY(check_aligned(reinterpret_cast<const void*>(addrs[i]), "limb pointer"));
  }
  const DevMod* mods;
  YELL_TRY(ctx->ensure_tables_list(log_n, cms.data(), count, &mods));
  LimbSet s;
  s.base = nullptr;
  s.ptrs = d_limbs;
  s.cms = d_cms;
  s.count = count;
  s.L = 1;
  s.cm0 = 0;
  s.pad_ = 0;
  YELL_CUDA(launch_ntt(s, log_n, mods, to_dir(direction), ctx->shape, st), "launch ntt");
  return kOk;
}

int yell_dev_elementwise(int op, uint64_t* d_dst, const uint64_t* d_a, const uint64_t* d_b,
                         uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0, void* stream) {
  if (op < 0 || op > 4) return fail(kInvalidArgument, "bad op");
  if (!d_dst || !d_a || (op != YELL_OP_NEGATE && !d_b) || count == 0)
    return fail(kInvalidArgument, "null pointer or zero count");
  YELL_TRY(check_aligned(d_dst, "d_dst"));
  YELL_TRY(check_aligned(d_a, "d_a"));
  if (d_b) YELL_TRY(check_aligned(d_b, "d_b"));
  YELL_TRY(check_degree(log_n));
  YELL_TRY(check_moduli(cm0, L));
  uint32_t limbs;
  YELL_TRY(check_limbs(count, L, log_n, &limbs));
  DeviceContext* ctx;
  YELL_TRY(get_ctx(&ctx));
  const DevMod* mods;
  YELL_TRY(ctx->ensure_tables(log_n, cm0, L, &mods));
  YELL_CUDA(launch_elementwise(static_cast<EwOp>(op), contiguous(d_dst, limbs, L, cm0),
                               const_contiguous(d_a, limbs, L, cm0),
                               const_contiguous(d_b ? d_b : d_a, limbs, L, cm0), log_n, mods,
                               pick_stream(ctx, stream)),
            "launch elementwise");
  return kOk;
}

size_t yell_polymul_scratch_words(uint32_t pairs, uint32_t L, uint32_t log_n) {
  uint32_t limbs;
  if (log_n < kMinLogN || log_n > kMaxLogN || L == 0 || L > kMaxModuli) return 0;
  if (check_limbs(pairs, L, log_n, &limbs) != kOk) return 0;
  NttShape shape;
  return polymul_scratch_words(limbs, log_n, shape);
}

int yell_dev_polymul(uint64_t* d_c, const uint64_t* d_a, const uint64_t* d_b, uint32_t pairs,
                     uint32_t L, uint32_t log_n, uint32_t cm0, uint64_t* d_scratch,
                     size_t scratch_words, void* stream) {
  if (!d_c || !d_a || !d_b || pairs == 0) return fail(kInvalidArgument, "null pointer or zero pairs");
  if (d_c == d_a || d_c == d_b) return fail(kInvalidArgument, "d_c aliases an operand");
  YELL_TRY(check_aligned(d_c, "d_c"));
  YELL_TRY(check_aligned(d_a, "d_a"));
  YELL_TRY(check_aligned(d_b, "d_b"));
  if (d_scratch) YELL_TRY(check_aligned(d_scratch, "d_scratch"));
  YELL_TRY(check_degree(log_n));
  YELL_TRY(check_moduli(cm0, L));
  uint32_t count;
  YELL_TRY(check_limbs(pairs, L, log_n, &count));
  DeviceContext* ctx;
  YELL_TRY(get_ctx(&ctx));
  const DevMod* mods;
  YELL_TRY(ctx->ensure_tables(log_n, cm0, L, &mods));
  const size_t need = polymul_scratch_words(count, log_n, ctx->shape);
  cudaStream_t st = pick_stream(ctx, stream);
  if (need == 0 || d_scratch) {
    if (need && scratch_words < need)
      return fail(kInvalidArgument, "scratch of " + std::to_string(scratch_words) + " words < " +
                                        std::to_string(need) + " needed");
    YELL_CUDA(launch_polymul(contiguous(d_c, count, L, cm0), const_contiguous(d_a, count, L, cm0),
                             const_contiguous(d_b, count, L, cm0), log_n, mods, d_scratch,
                             ctx->shape, st),
              "launch polymul");
    return kOk;
  }
  // Library scratch, stream-ordered: allocated and freed on `st` around the
  // launches, so the call does not wait for the GPU.
  uint64_t* scratch = nullptr;
  YELL_TRY(ctx->scratch_alloc_async(need, st, &scratch));
  const cudaError_t le = launch_polymul(contiguous(d_c, count, L, cm0), const_contiguous(d_a, count, L, cm0),
                                        const_contiguous(d_b, count, L, cm0), log_n, mods, scratch, ctx->shape, st);
  const int fs = ctx->scratch_free_async(scratch, st);
  if (le != cudaSuccess) return fail_cuda(le, "launch polymul");
  return fs;
}

int yell_profile_start(void) { return profile_start() == 0 ? kOk : fail(kCudaError, "profile start"); }

int yell_profile_stop(void) {
  return profile_stop() == 0 ? kOk : fail(kCudaError, "profile stop: event wait failed");
}

int yell_profile_count(void) { return profile_count(); }

int yell_profile_get(int i, char* name, size_t name_len, uint64_t* launches, double* total_ms) {
  if (!name || name_len == 0 || !launches || !total_ms) return fail(kInvalidArgument, "null output");
  std::string n;
  if (profile_get(i, &n, launches, total_ms) != 0) return fail(kNotFound, "no such profile entry");
  std::strncpy(name, n.c_str(), name_len - 1);
  name[name_len - 1] = '\0';
  return kOk;
}

int yell_synchronize(void) {
  DeviceContext* ctx;
  YELL_TRY(get_ctx(&ctx));
  YELL_CUDA(cudaStreamSynchronize(ctx->stream()), "synchronize");
  return kOk;
}

}  // extern "C"
