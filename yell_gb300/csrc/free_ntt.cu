// The reference's runtime-N free functions negacylic_forward_lazy /
// negacylic_backward_lazy (include/yell/details/ntt.hpp:10-23, bodies
// lib/ntt.cpp:89-210): an in-place lazy transform of any power-of-two degree
// with caller-supplied twiddles {w, w'} and modulus p.  They are drop-ins, not
// the hot path: the words go to the device, one CTA applies the reference's
// stage sequence butterfly for butterfly (a barrier between stages, the
// words in L2), and come back.
//   forward : stages (m, h) = (2^s, N / 2^(s+1)), s = 0 .. log N - 1, CT
//             butterflies on (2hr + i, 2hr + i + h) with w[m + r]; [0, 4p) in/out
//   backward: (N/2, 1) and (N/4, 2), then while m > 1; GS butterflies; the
//             layer m = 1 is left to the caller for N >= 8 (at N = 4 the
//             second stage already is that layer, as in the reference)
#include <algorithm>

#include "common.cuh"
#include "kernels.h"
#include "profiler.h"
#include "runtime.h"
#include "yell_gb300.h"

using namespace yell_gb300;

namespace {

constexpr int kFreeThreads = 1024;
constexpr int kMaxFreeStages = 24;

struct FreeStages {
  uint32_t count;
  uint8_t log_h[kMaxFreeStages];  // m = N / (2h)
};

__global__ void __launch_bounds__(kFreeThreads) k_free_ntt(uint64_t* __restrict__ x, const uint64_t* __restrict__ w,
                                                           const uint64_t* __restrict__ ws, uint64_t p, uint32_t log_n,
                                                           FreeStages st, int inverse) {
  const uint64_t np = 0 - p, p2 = p << 1;
  const uint32_t half = 1u << (log_n - 1);
  for (uint32_t s = 0; s < st.count; ++s) {
    const uint32_t lh = st.log_h[s];
    const uint32_t m = half >> lh;
    for (uint32_t k = threadIdx.x; k < half; k += blockDim.x) {
      const uint32_t r = k >> lh, i = k & ((1u << lh) - 1u);
      const uint32_t j = (r << (lh + 1)) + i;
      uint64_t a = x[j], b = x[j + (1u << lh)];
      const uint64_t wr = __ldg(&w[m + r]), wsr = __ldg(&ws[m + r]);
      if (inverse) gs_bfly(a, b, wr, wsr, np, p2);
      else ct_bfly(a, b, wr, wsr, np, p2);
      x[j] = a;
      x[j + (1u << lh)] = b;
    }
    __syncthreads();
  }
}

int free_ntt(uint64_t* x, uint64_t degree, const uint64_t* w, const uint64_t* wshoup, uint64_t p, bool inverse) {
  if (!x || !w || !wshoup) return fail(kInvalidArgument, "null pointer");
  if (degree < 4 || degree > (1ull << 20) || (degree & (degree - 1)))
    return fail(kUnsupportedDegree, "degree must be a power of two in [4, 2^20]");
  if (p < 3 || p >= (1ull << 62)) return fail(kInvalidArgument, "p must be below 2^62 (4p < 2^64)");
  uint32_t log_n = 0;
  while ((1ull << log_n) < degree) ++log_n;
  FreeStages st{};
  if (!inverse) {
    for (uint32_t s = 0; s < log_n; ++s) st.log_h[st.count++] = (uint8_t)(log_n - 1 - s);
  } else {
    st.log_h[st.count++] = 0;  // m = N/2, h = 1
    st.log_h[st.count++] = 1;  // m = N/4, h = 2
    // then while m = N / 2^(lh+1) > 1
    for (uint32_t lh = 2; lh + 1 < log_n; ++lh) st.log_h[st.count++] = (uint8_t)lh;
  }
  int status = kOk;
  DeviceContext* ctx = DeviceContext::current(&status);
  if (!ctx) return status;
  const size_t n = (size_t)degree;
  std::lock_guard<std::mutex> g(ctx->staging.lock);
  status = ctx->staging.reserve(3 * n);
  if (status != kOk) return status;
  uint64_t* dx = ctx->staging.ptr;
  uint64_t* dw = dx + n;
  uint64_t* dws = dw + n;
  cudaStream_t s = ctx->stream();
  cudaError_t e = cudaMemcpyAsync(dx, x, n * 8, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dw, w, n * 8, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dws, wshoup, n * 8, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return fail_cuda(e, "H2D");
  {
    LaunchScope ps(inverse ? "negacyclic_backward_lazy" : "negacyclic_forward_lazy", s);
    const int threads = (int)std::min<uint64_t>(kFreeThreads, degree / 2);
    k_free_ntt<<<1, threads, 0, s>>>(dx, dw, dws, p, log_n, st, inverse ? 1 : 0);
    g_kernel_launches += 1;
  }
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(x, dx, n * 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? kOk : fail_cuda(e, inverse ? "negacyclic_backward_lazy" : "negacyclic_forward_lazy");
}

}  // namespace

extern "C" {

int yell_negacyclic_forward_lazy(uint64_t* x, uint64_t degree, const uint64_t* w, const uint64_t* wshoup,
                                 uint64_t p) {
  return free_ntt(x, degree, w, wshoup, p, false);
}

int yell_negacyclic_backward_lazy(uint64_t* x, uint64_t degree, const uint64_t* w, const uint64_t* wshoup,
                                  uint64_t p) {
  return free_ntt(x, degree, w, wshoup, p, true);
}

}  // extern "C"
