// Integer roofline of this GPU for the path's butterflies.
//
// The NTT kernels are bound by the 64-bit modular multiply (built from
// 32-bit IMAD), not by HBM.  This kernel measures the ceiling directly: every
// thread keeps 16 words and 15 twiddles in registers and applies rounds of
// 4 radix-2 stages of the production CT (or GS) butterfly with no memory
// traffic, so the rate it reaches is the most butterflies per second the
// arithmetic allows on this device and clock.
#include <cuda_runtime.h>

#include "common.cuh"
#include "runtime.h"
#include "yell_gb300.h"

using namespace yell_gb300;

namespace {

template <bool GS>
__global__ void __launch_bounds__(256) k_butterfly_ceiling(uint64_t* out, const ulonglong2* tw, uint64_t p,
                                                           int iters) {
  uint64_t x[16];
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  for (int i = 0; i < 16; ++i) x[i] = (tid * 0x9E3779B97F4A7C15ull + i * 0xBF58476D1CE4E5B9ull) % (2 * p);
  const uint64_t p2 = 2 * p, np = 0 - p;
  ulonglong2 w[15];
  for (int i = 0; i < 15; ++i) w[i] = tw[(tid + i) & 63];
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int d = 1 << (3 - k);
#pragma unroll
      for (int jj = 0; jj < (1 << k); ++jj)
#pragma unroll
        for (int q = 0; q < d; ++q) {
          const int j = jj * 2 * d + q;
          const ulonglong2 ww = w[(1 << k) - 1 + jj];
          if (GS)
            gs_bfly(x[j], x[j + d], ww.x, ww.y, np, p2);
          else
            ct_bfly(x[j], x[j + d], ww.x, ww.y, np, p2);
        }
    }
  }
  for (int i = 0; i < 16; ++i) out[(size_t)tid * 16 + i] = x[i];
}

// The same loop on 32-bit words with the 32-bit mode's butterflies (the
// twiddles are arbitrary residues of a 30-bit modulus with their Shoup
// companions; the rate does not depend on their values).
template <bool GS>
__global__ void __launch_bounds__(256) k_butterfly_ceiling32(uint32_t* out, const uint2* tw, uint32_t p, int iters) {
  uint32_t x[16];
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  for (int i = 0; i < 16; ++i) x[i] = (tid * 0x9E3779B9u + i * 0x85EBCA6Bu) % (2 * p);
  const uint32_t p2 = 2 * p, np = 0u - p;
  uint2 w[15];
  for (int i = 0; i < 15; ++i) w[i] = tw[(tid + i) & 63];
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int d = 1 << (3 - k);
#pragma unroll
      for (int jj = 0; jj < (1 << k); ++jj)
#pragma unroll
        for (int q = 0; q < d; ++q) {
          const int j = jj * 2 * d + q;
          const uint2 ww = w[(1 << k) - 1 + jj];
          if (GS)
            gs_bfly(x[j], x[j + d], ww.x, ww.y, np, p2);
          else
            ct_bfly(x[j], x[j + d], ww.x, ww.y, np, p2);
        }
    }
  }
  for (int i = 0; i < 16; ++i) out[(size_t)tid * 16 + i] = x[i];
}

}  // namespace

extern "C" int yell32_calibrate_butterflies(double* ct_per_s, double* gs_per_s) {
  if (!ct_per_s || !gs_per_s) return fail(kInvalidArgument, "null output");
  int st = kOk;
  DeviceContext* ctx = DeviceContext::current(&st);
  if (!ctx) return st;
  int sms = 0;
  cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device());
  if (e != cudaSuccess) return fail_cuda(e, "cudaDeviceGetAttribute");
  const uint32_t p = yell32_prime(0);
  uint2 htw[64];
  uint64_t s = 0x243F6A8885A308D3ull;
  for (uint2& t : htw) {
    s = s * 6364136223846793005ull + 1442695040888963407ull;
    t.x = (uint32_t)((s >> 20) % p);
    t.y = (uint32_t)(((uint64_t)t.x << 32) / p);
  }
  const int blocks = sms * 8, threads = 256, iters = 400;
  uint2* tw = nullptr;
  uint32_t* out = nullptr;
  e = lib_malloc(&tw, sizeof(htw));
  if (e == cudaSuccess) e = lib_malloc(&out, (size_t)blocks * threads * 16 * sizeof(uint32_t));
  cudaStream_t strm = ctx->stream();
  if (e == cudaSuccess) e = cudaMemcpyAsync(tw, htw, sizeof(htw), cudaMemcpyHostToDevice, strm);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  const double bfly = (double)blocks * threads * iters * 32;
  double rates[2] = {0, 0};
  for (int gs = 0; gs < 2 && e == cudaSuccess; ++gs) {
    float best = 1e30f;
    for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {
      cudaEventRecord(e0, strm);
      if (gs)
        k_butterfly_ceiling32<true><<<blocks, threads, 0, strm>>>(out, tw, p, iters);
      else
        k_butterfly_ceiling32<false><<<blocks, threads, 0, strm>>>(out, tw, p, iters);
      g_kernel_launches += 1;
      cudaEventRecord(e1, strm);
      e = cudaEventSynchronize(e1);
      float ms = 0;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
      if (rep > 0 && ms < best) best = ms;  // first run is the warm-up
    }
    rates[gs] = bfly / (best * 1e-3);
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (tw) cudaFree(tw);
  if (out) cudaFree(out);
  if (e != cudaSuccess) return fail_cuda(e, "calibration run (32-bit)");
  *ct_per_s = rates[0];
  *gs_per_s = rates[1];
  return kOk;
}

extern "C" int yell_calibrate_butterflies(double* ct_per_s, double* gs_per_s) {
  if (!ct_per_s || !gs_per_s) return fail(kInvalidArgument, "null output");
  int st = kOk;
  DeviceContext* ctx = DeviceContext::current(&st);
  if (!ctx) return st;
  int sms = 0;
  cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device());
  if (e != cudaSuccess) return fail_cuda(e, "cudaDeviceGetAttribute");
  const DevMod* mods;
  st = ctx->ensure_tables(12, 0, 1, &mods);  // any resident table supplies twiddles
  if (st != kOk) return st;
  DevMod m;
  e = cudaMemcpy(&m, mods, sizeof(DevMod), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return fail_cuda(e, "cudaMemcpy(DevMod)");
  const int blocks = sms * 8, threads = 256, iters = 200;
  uint64_t* out = nullptr;
  e = lib_malloc(&out, (size_t)blocks * threads * 16 * sizeof(uint64_t));
  if (e != cudaSuccess) return fail_cuda(e, "cudaMalloc(calibration)");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaStream_t s = ctx->stream();
  const double bfly = (double)blocks * threads * iters * 32;
  double rates[2] = {0, 0};
  for (int gs = 0; gs < 2 && e == cudaSuccess; ++gs) {
    float best = 1e30f;
    for (int rep = 0; rep < 4 && e == cudaSuccess; ++rep) {
      cudaEventRecord(e0, s);
      if (gs)
        k_butterfly_ceiling<true><<<blocks, threads, 0, s>>>(out, m.fwd + 64, m.p, iters);
      else
        k_butterfly_ceiling<false><<<blocks, threads, 0, s>>>(out, m.fwd + 64, m.p, iters);
      g_kernel_launches += 1;
      cudaEventRecord(e1, s);
      e = cudaEventSynchronize(e1);
      float ms = 0;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
      if (rep > 0 && ms < best) best = ms;  // first run is the warm-up
    }
    rates[gs] = bfly / (best * 1e-3);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess) return fail_cuda(e, "calibration run");
  *ct_per_s = rates[0];
  *gs_per_s = rates[1];
  return kOk;
}
