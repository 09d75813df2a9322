// Device-resident poly handles and asynchronous polymul batches.
//
// A handle is one poly<N> kept in HBM: L limbs of N words in one allocation,
// limb l under prime cm0 + l.  It stands where the reference's poly<N> object
// stands (include/yell/poly.hpp:43-121: per-limb buffers, forward/backward,
// the operators of include/yell/poly.hpp:163-168, add_product_of, negate),
// but the coefficients stay on the device between calls; host memory is only
// touched by upload and download, which are synchronous.  Every other handle
// call is ordered on the device's library stream, so calls on the same
// handles run in the order they were made.
#include <chrono>
#include <thread>

#include "runtime.h"
#include "yell_gb300.h"

using namespace yell_gb300;

struct yell_dev_poly {
  uint64_t* data = nullptr;
  uint32_t L = 0, log_n = 0, cm0 = 0;
  int device = -1;
};

struct yell_batch {
  cudaEvent_t done = nullptr;
  int device = -1;
};

namespace {

int context_for(int device, DeviceContext** out) {
  int st = kOk;
  DeviceContext* ctx = DeviceContext::current(&st);
  if (!ctx) return st;
  if (device >= 0 && ctx->device() != device)
    return fail(kInvalidArgument, "handle belongs to device " + std::to_string(device) +
                                      ", current device is " + std::to_string(ctx->device()));
  *out = ctx;
  return kOk;
}

size_t limb_words(const yell_dev_poly* p) { return (size_t)1 << p->log_n; }

int same_shape(const yell_dev_poly* a, const yell_dev_poly* b) {
  if (a->log_n != b->log_n || a->L != b->L || a->cm0 != b->cm0 || a->device != b->device)
    return fail(kInvalidArgument, "handles differ in degree, limb count, moduli or device");
  return kOk;
}

}  // namespace

extern "C" {

int yell_dev_poly_alloc(uint32_t L, uint32_t log_n, uint32_t cm0, yell_dev_poly** out) {
  if (!out || L == 0) return fail(kInvalidArgument, "null output or zero limbs");
  int st = check_degree(log_n);
  if (st != kOk) return st;
  st = check_moduli(cm0, L);
  if (st != kOk) return st;
  DeviceContext* ctx = nullptr;
  st = context_for(-1, &ctx);
  if (st != kOk) return st;
  const DevMod* mods;
  st = ctx->ensure_tables(log_n, cm0, L, &mods);
  if (st != kOk) return st;
  auto* p = new yell_dev_poly;
  p->L = L;
  p->log_n = log_n;
  p->cm0 = cm0;
  p->device = ctx->device();
  const cudaError_t e = lib_malloc(&p->data, ((size_t)L << log_n) * sizeof(uint64_t));
  if (e != cudaSuccess) {
    delete p;
    return e == cudaErrorMemoryAllocation ? fail(kOutOfMemory, "cudaMalloc(poly)") : fail_cuda(e, "cudaMalloc(poly)");
  }
  *out = p;
  return kOk;
}

int yell_dev_poly_free(yell_dev_poly* p) {
  if (!p) return kOk;
  DeviceContext* ctx = nullptr;
  int st = context_for(p->device, &ctx);
  if (st != kOk) return st;
  // pending work on the library stream may still use the buffer
  cudaError_t e = cudaStreamSynchronize(ctx->stream());
  if (e == cudaSuccess) e = cudaFree(p->data);
  delete p;
  return e == cudaSuccess ? kOk : fail_cuda(e, "free poly");
}

int yell_dev_poly_info(const yell_dev_poly* p, uint64_t** d_data, uint32_t* L, uint32_t* log_n, uint32_t* cm0) {
  if (!p) return fail(kInvalidArgument, "null handle");
  if (d_data) *d_data = p->data;
  if (L) *L = p->L;
  if (log_n) *log_n = p->log_n;
  if (cm0) *cm0 = p->cm0;
  return kOk;
}

int yell_dev_poly_upload(yell_dev_poly* p, const uint64_t* const* limbs) {
  if (!p || !limbs) return fail(kInvalidArgument, "null handle or limb array");
  DeviceContext* ctx = nullptr;
  int st = context_for(p->device, &ctx);
  if (st != kOk) return st;
  const size_t n = limb_words(p);
  cudaStream_t s = ctx->stream();
  for (uint32_t l = 0; l < p->L; ++l)
    if (!limbs[l]) return fail(kInvalidArgument, "null limb pointer");
  if (ctx->host_access() && host_limbs_accessible(limbs, p->L)) {
    // one kernel reads every limb where it lies (no pageable copies)
    const cudaError_t e = gather_host_limbs(p->data, limbs, p->L, p->log_n, s);
    if (e != cudaSuccess) return fail_cuda(e, "upload");
  } else {
    for (uint32_t l = 0; l < p->L; ++l) {
      const cudaError_t e = cudaMemcpyAsync(p->data + l * n, limbs[l], n * 8, cudaMemcpyHostToDevice, s);
      if (e != cudaSuccess) return fail_cuda(e, "upload limb");
    }
  }
  const cudaError_t e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? kOk : fail_cuda(e, "upload");
}

int yell_dev_poly_download(const yell_dev_poly* p, uint64_t* const* limbs) {
  if (!p || !limbs) return fail(kInvalidArgument, "null handle or limb array");
  DeviceContext* ctx = nullptr;
  int st = context_for(p->device, &ctx);
  if (st != kOk) return st;
  const size_t n = limb_words(p);
  cudaStream_t s = ctx->stream();
  for (uint32_t l = 0; l < p->L; ++l)
    if (!limbs[l]) return fail(kInvalidArgument, "null limb pointer");
  if (ctx->host_access() && host_limbs_accessible(limbs, p->L)) {
    const cudaError_t e = scatter_host_limbs(limbs, p->data, p->L, p->log_n, s);
    if (e != cudaSuccess) return fail_cuda(e, "download");
  } else {
    for (uint32_t l = 0; l < p->L; ++l) {
      const cudaError_t e = cudaMemcpyAsync(limbs[l], p->data + l * n, n * 8, cudaMemcpyDeviceToHost, s);
      if (e != cudaSuccess) return fail_cuda(e, "download limb");
    }
  }
  const cudaError_t e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? kOk : fail_cuda(e, "download");
}

int yell_dev_poly_ntt(yell_dev_poly* p, int direction) {
  if (!p) return fail(kInvalidArgument, "null handle");
  DeviceContext* ctx = nullptr;
  int st = context_for(p->device, &ctx);
  if (st != kOk) return st;
  return yell_dev_ntt(p->data, 1, p->L, p->log_n, p->cm0, direction, nullptr);
}

int yell_dev_poly_op(int op, yell_dev_poly* dst, const yell_dev_poly* a, const yell_dev_poly* b) {
  if (!dst || !a || (op != YELL_OP_NEGATE && !b)) return fail(kInvalidArgument, "null handle");
  int st = same_shape(dst, a);
  if (st == kOk && op != YELL_OP_NEGATE) st = same_shape(dst, b);
  if (st != kOk) return st;
  DeviceContext* ctx = nullptr;
  st = context_for(dst->device, &ctx);
  if (st != kOk) return st;
  return yell_dev_elementwise(op, dst->data, a->data, op == YELL_OP_NEGATE ? nullptr : b->data, 1, dst->L,
                              dst->log_n, dst->cm0, nullptr);
}

int yell_dev_poly_mul(yell_dev_poly* c, const yell_dev_poly* a, const yell_dev_poly* b) {
  if (!c || !a || !b) return fail(kInvalidArgument, "null handle");
  if (c == a || c == b) return fail(kInvalidArgument, "the product may not overwrite an operand");
  int st = same_shape(c, a);
  if (st == kOk) st = same_shape(c, b);
  if (st != kOk) return st;
  DeviceContext* ctx = nullptr;
  st = context_for(c->device, &ctx);
  if (st != kOk) return st;
  return yell_dev_polymul(c->data, a->data, b->data, 1, c->L, c->log_n, c->cm0, nullptr, 0, nullptr);
}

int yell_batch_submit(yell_dev_poly* const* c, const yell_dev_poly* const* a, const yell_dev_poly* const* b,
                      uint32_t n, yell_batch** ticket) {
  if (!c || !a || !b || !ticket || n == 0) return fail(kInvalidArgument, "null arrays, null ticket or empty batch");
  std::vector<yell_polymul_desc> descs(n);
  int device = -1;
  for (uint32_t i = 0; i < n; ++i) {
    if (!c[i] || !a[i] || !b[i]) return fail(kInvalidArgument, "null handle in batch");
    if (c[i] == a[i] || c[i] == b[i]) return fail(kInvalidArgument, "a product may not overwrite an operand");
    int st = same_shape(c[i], a[i]);
    if (st == kOk) st = same_shape(c[i], b[i]);
    if (st != kOk) return st;
    if (device >= 0 && c[i]->device != device) return fail(kInvalidArgument, "batch spans devices");
    device = c[i]->device;
    descs[i] = yell_polymul_desc{c[i]->data, a[i]->data, b[i]->data, c[i]->log_n, c[i]->L, c[i]->cm0, 0};
  }
  DeviceContext* ctx = nullptr;
  int st = context_for(device, &ctx);
  if (st != kOk) return st;
  st = yell_dev_polymul_batch(descs.data(), n, nullptr);
  if (st != kOk) return st;
  auto* t = new yell_batch;
  t->device = device;
  cudaError_t e = cudaEventCreateWithFlags(&t->done, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventRecord(t->done, ctx->stream());
  if (e != cudaSuccess) {
    if (t->done) cudaEventDestroy(t->done);
    delete t;
    return fail_cuda(e, "batch ticket");
  }
  *ticket = t;
  return kOk;
}

int yell_batch_wait(yell_batch* t, double timeout_s) {
  if (!t) return fail(kInvalidArgument, "null ticket");
  const auto deadline = std::chrono::steady_clock::now() + std::chrono::duration<double>(timeout_s);
  for (;;) {
    const cudaError_t e = cudaEventQuery(t->done);
    if (e == cudaSuccess) break;
    if (e != cudaErrorNotReady) return fail_cuda(e, "batch");
    if (std::chrono::steady_clock::now() >= deadline) return fail(kTimeout, "batch still running");
    std::this_thread::sleep_for(std::chrono::microseconds(20));
  }
  cudaEventDestroy(t->done);
  delete t;
  return kOk;
}

int yell_batch_release(yell_batch* t) {
  if (!t) return kOk;
  cudaEventDestroy(t->done);  // the batch itself still completes
  delete t;
  return kOk;
}

}  // extern "C"
