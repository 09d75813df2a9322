// RNS -> big-integer lifting (CRT) on the device: gmp::poly2mpz of the
// reference (include/yell/gmp.hpp:42-70, tables lib/gmp.cpp:6-51).
//
// For residues r_j mod q_j (j < L), the lifted value is the unique
// x in [0, Q), Q = prod q_j, with x = r_j mod q_j.  The reference sums
// r_j * lift_j (lift_j = ((Q/q_j)^-1 mod q_j) * Q/q_j) and reduces the sum mod
// Q with a Shoup quotient; for residues below their moduli that returns x.
// Here, per coefficient:
//   y_j = r_j * ((Q/q_j)^-1 mod q_j) mod q_j          (Shoup product, exact)
//   v   = floor(sum_j y_j / q_j), estimated with 64-bit fractions
//         f_j = floor(y_j * floor(2^125 / q_j) / 2^61); the estimate is v or v - 1
//   x   = sum_j y_j * (Q/q_j) - v * Q, minus Q once more when still >= Q
// sum_j y_j * (Q/q_j) = Q * sum_j y_j / q_j, so with the exact v this is x.
// The multi-word sums run column by column (product scanning): a thread owns
// one coefficient, keeps its y_j in shared memory and streams out the words
// of x, least significant first; x is written as W little-endian words per
// coefficient, W = words of Q, coefficient-major.
#include <cstring>
#include <map>
#include <memory>
#include <tuple>
#include <mutex>
#include <set>
#include <utility>
#include <vector>

#include "common.cuh"
#include "kernels.h"
#include "profiler.h"
#include "runtime.h"
#include "yell_gb300.h"

using namespace yell_gb300;

namespace {

typedef unsigned __int128 u128;

constexpr uint32_t kCrtThreads = 64;
constexpr uint32_t kCrtMaxModuli = 400;  // 64 threads * 400 words * 8 B = 200 KB of y per block

// Per (device, cm0, L) constants, device resident:
//   mods[j] = {q_j, inv_j, inv_j', c_j} with inv_j = (Q/q_j)^-1 mod q_j, inv_j' its
//   Shoup companion floor(inv_j * 2^64 / q_j), c_j = floor(2^125 / q_j);
//   words[j * W + w] = word w of Q/q_j; qwords[w] = word w of Q.
struct CrtConst {
  uint64_t q, inv, inv_s, c;
};

struct CrtTables {
  uint32_t W = 0;
  CrtConst* mods = nullptr;
  uint64_t* cofactors = nullptr;
  uint64_t* q = nullptr;
};

// Host big integers: little-endian 64-bit words.
using Big = std::vector<uint64_t>;

void big_mul_small(Big& a, uint64_t m) {
  uint64_t carry = 0;
  for (uint64_t& w : a) {
    const u128 t = (u128)w * m + carry;
    w = (uint64_t)t;
    carry = (uint64_t)(t >> 64);
  }
  if (carry) a.push_back(carry);
}

// a / m (exact or not), remainder returned.
uint64_t big_divmod_small(const Big& a, uint64_t m, Big* quot) {
  quot->assign(a.size(), 0);
  u128 rem = 0;
  for (size_t i = a.size(); i-- > 0;) {
    const u128 cur = (rem << 64) | a[i];
    (*quot)[i] = (uint64_t)(cur / m);
    rem = cur % m;
  }
  while (!quot->empty() && quot->back() == 0) quot->pop_back();
  return (uint64_t)rem;
}

uint64_t pow_mod(uint64_t b, uint64_t e, uint64_t m) {
  uint64_t r = 1;
  b %= m;
  while (e) {
    if (e & 1) r = (uint64_t)((u128)r * b % m);
    b = (uint64_t)((u128)b * b % m);
    e >>= 1;
  }
  return r;
}

int build_crt_tables(uint32_t cm0, uint32_t L, CrtTables* t) {
  Big Q{1};
  for (uint32_t j = 0; j < L; ++j) big_mul_small(Q, prime_entry(cm0 + j).p);
  const uint32_t W = (uint32_t)Q.size();
  std::vector<CrtConst> mods(L);
  std::vector<uint64_t> cof((size_t)L * W, 0);
  for (uint32_t j = 0; j < L; ++j) {
    const uint64_t q = prime_entry(cm0 + j).p;
    Big m;
    const uint64_t rem = big_divmod_small(Q, q, &m);
    if (rem != 0) return fail(kInvalidArgument, "CRT: modulus does not divide the product");
    uint64_t mq;
    {
      Big unused;
      mq = big_divmod_small(m, q, &unused);
    }
    const uint64_t inv = pow_mod(mq, q - 2, q);  // q prime
    mods[j].q = q;
    mods[j].inv = inv;
    mods[j].inv_s = (uint64_t)(((u128)inv << 64) / q);
    mods[j].c = (uint64_t)(((u128)1 << 125) / q);
    for (size_t w = 0; w < m.size(); ++w) cof[(size_t)j * W + w] = m[w];
  }
  cudaError_t e = cudaMalloc(&t->mods, L * sizeof(CrtConst));
  if (e == cudaSuccess) e = cudaMalloc(&t->cofactors, cof.size() * 8);
  if (e == cudaSuccess) e = cudaMalloc(&t->q, (size_t)W * 8);
  if (e == cudaSuccess) e = cudaMemcpy(t->mods, mods.data(), L * sizeof(CrtConst), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(t->cofactors, cof.data(), cof.size() * 8, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(t->q, Q.data(), (size_t)W * 8, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(t->mods);
    cudaFree(t->cofactors);
    cudaFree(t->q);
    return fail_cuda(e, "CRT tables");
  }
  t->W = W;
  return kOk;
}

int crt_tables(int device, uint32_t cm0, uint32_t L, const CrtTables** out) {
  static std::mutex mu;
  static std::map<std::tuple<int, uint32_t, uint32_t>, CrtTables> cache;
  std::lock_guard<std::mutex> g(mu);
  const auto key = std::make_tuple(device, cm0, L);
  auto it = cache.find(key);
  if (it == cache.end()) {
    CrtTables t;
    const int st = build_crt_tables(cm0, L, &t);
    if (st != kOk) return st;
    it = cache.emplace(key, t).first;
  }
  *out = &it->second;
  return kOk;
}

uint32_t crt_words(uint32_t cm0, uint32_t L) {
  // bits of Q = sum of bit lengths, up to one less per product; exact count
  // from the product itself (cheap on the host).
  Big Q{1};
  for (uint32_t j = 0; j < L; ++j) big_mul_small(Q, prime_entry(cm0 + j).p);
  return (uint32_t)Q.size();
}

__device__ __forceinline__ void acc_mac(uint64_t& a0, uint64_t& a1, uint64_t& a2, uint64_t x, uint64_t y) {
  const uint64_t lo = x * y;
  const uint64_t hi = __umul64hi(x, y);
  asm("add.cc.u64 %0, %0, %3;\n\t"
      "addc.cc.u64 %1, %1, %4;\n\t"
      "addc.u64 %2, %2, 0;"
      : "+l"(a0), "+l"(a1), "+l"(a2)
      : "l"(lo), "l"(hi));
}

// d = a - b - borrow_in, returns the borrow out.
__device__ __forceinline__ uint32_t sub_borrow(uint64_t a, uint64_t b, uint32_t bin, uint64_t* d) {
  const uint64_t t = a - b;
  const uint32_t b1 = a < b;
  *d = t - bin;
  return b1 | (t < (uint64_t)bin);
}

__global__ void __launch_bounds__(kCrtThreads) k_crt_lift(uint64_t* __restrict__ out, const uint64_t* __restrict__ in,
                                                          uint32_t count, uint32_t L, uint32_t log_n,
                                                          const CrtConst* __restrict__ mods,
                                                          const uint64_t* __restrict__ cof,
                                                          const uint64_t* __restrict__ qw, uint32_t W) {
  extern __shared__ uint64_t ys[];  // [L][kCrtThreads]
  const uint64_t coeffs = (uint64_t)count << log_n;
  const uint64_t g = (uint64_t)blockIdx.x * kCrtThreads + threadIdx.x;
  const bool live = g < coeffs;
  const uint64_t poly = g >> log_n;
  const uint64_t i = g & ((1ull << log_n) - 1);
  const uint64_t n = 1ull << log_n;

  // y_j and the 64-bit-fraction sum of y_j / q_j
  uint64_t f_lo = 0, f_hi = 0;
  for (uint32_t j = 0; j < L; ++j) {
    uint64_t y = 0;
    if (live) {
      const CrtConst m = mods[j];
      const uint64_t r = in[(poly * L + j) * n + i];
      y = mulmod_shoup(r, m.inv, m.inv_s, m.q);
      const uint64_t pl = y * m.c, ph = __umul64hi(y, m.c);
      const uint64_t f = (pl >> 61) | (ph << 3);  // floor(y c / 2^61) < 2^64
      asm("add.cc.u64 %0, %0, %2;\n\taddc.u64 %1, %1, 0;" : "+l"(f_lo), "+l"(f_hi) : "l"(f));
    }
    ys[j * kCrtThreads + threadIdx.x] = y;
  }
  __syncthreads();
  if (!live) return;
  const uint64_t v = f_hi;

  uint64_t* dst = out + g * W;
  uint64_t x0 = 0, x1 = 0, x2 = 0;  // column accumulator of sum y_j (Q/q_j)
  uint64_t q0 = 0, q1 = 0;          // column accumulator of v Q
  uint32_t br = 0, bq = 0;          // borrows of x - vQ and of (x - vQ) - Q
  for (uint32_t w = 0; w <= W; ++w) {
    if (w < W) {
      for (uint32_t j = 0; j < L; ++j) acc_mac(x0, x1, x2, ys[j * kCrtThreads + threadIdx.x], __ldg(&cof[(size_t)j * W + w]));
      const uint64_t qword = __ldg(&qw[w]);
      const uint64_t lo = v * qword, hi = __umul64hi(v, qword);
      asm("add.cc.u64 %0, %0, %2;\n\taddc.u64 %1, %1, %3;" : "+l"(q0), "+l"(q1) : "l"(lo), "l"(hi));
    }
    uint64_t r;
    br = sub_borrow(x0, q0, br, &r);
    uint64_t alt;
    bq = sub_borrow(r, w < W ? __ldg(&qw[w]) : 0ull, bq, &alt);
    if (w < W) dst[w] = r;
    x0 = x1;
    x1 = x2;
    x2 = 0;
    q0 = q1;
    q1 = 0;
  }
  if (bq == 0) {  // x - vQ >= Q: the estimate of v was one short
    uint32_t b = 0;
    for (uint32_t w = 0; w < W; ++w) {
      uint64_t d;
      b = sub_borrow(dst[w], __ldg(&qw[w]), b, &d);
      dst[w] = d;
    }
  }
}

int crt_lift(uint64_t* d_out, const uint64_t* d_in, uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0,
             cudaStream_t st, int device) {
  const CrtTables* t = nullptr;
  int s = crt_tables(device, cm0, L, &t);
  if (s != kOk) return s;
  const size_t smem = (size_t)L * kCrtThreads * sizeof(uint64_t);
  cudaError_t e = cudaSuccess;
  {
    // the shared-memory limit is a per-device attribute of the kernel
    static std::mutex mu;
    static std::set<int> done;
    std::lock_guard<std::mutex> g(mu);
    if (!done.count(device)) {
      e = cudaFuncSetAttribute(k_crt_lift, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)(kCrtMaxModuli * kCrtThreads * sizeof(uint64_t)));
      if (e != cudaSuccess) return fail_cuda(e, "crt attributes");
      done.insert(device);
    }
  }
  const uint64_t coeffs = (uint64_t)count << log_n;
  const uint32_t blocks = (uint32_t)((coeffs + kCrtThreads - 1) / kCrtThreads);
  {
    LaunchScope ps("crt_lift", st);
    k_crt_lift<<<blocks, kCrtThreads, smem, st>>>(d_out, d_in, count, L, log_n, t->mods, t->cofactors, t->q, t->W);
    g_kernel_launches += 1;
  }
  e = cudaGetLastError();
  return e == cudaSuccess ? kOk : fail_cuda(e, "crt_lift");
}

int check_crt_args(uint32_t L, uint32_t log_n, uint32_t cm0) {
  int st = check_degree(log_n);
  if (st != kOk) return st;
  st = check_moduli(cm0, L);
  if (st != kOk) return st;
  if (L > kCrtMaxModuli) return fail(kInvalidArgument, "CRT lifting takes at most 400 moduli");
  return kOk;
}

}  // namespace

extern "C" {

int yell_crt_words(uint32_t L, uint32_t cm0, uint32_t* words) {
  if (!words) return fail(kInvalidArgument, "null output");
  const int st = check_moduli(cm0, L);
  if (st != kOk) return st;
  *words = crt_words(cm0, L);
  return kOk;
}

int yell_dev_crt_lift(uint64_t* d_out, const uint64_t* d_in, uint32_t count, uint32_t L, uint32_t log_n,
                      uint32_t cm0, void* stream) {
  if (!d_out || !d_in || count == 0) return fail(kInvalidArgument, "null pointer or zero count");
  int st = check_crt_args(L, log_n, cm0);
  if (st != kOk) return st;
  DeviceContext* ctx = DeviceContext::current(&st);
  if (!ctx) return st;
  return crt_lift(d_out, d_in, count, L, log_n, cm0, stream ? static_cast<cudaStream_t>(stream) : ctx->stream(),
                  ctx->device());
}

int yell_poly_to_bigint(uint64_t* out, const uint64_t* const* limbs, uint32_t L, uint32_t log_n) {
  if (!out || !limbs) return fail(kInvalidArgument, "null pointer");
  int st = check_crt_args(L, log_n, 0);
  if (st != kOk) return st;
  for (uint32_t j = 0; j < L; ++j)
    if (!limbs[j]) return fail(kInvalidArgument, "null limb pointer");
  DeviceContext* ctx = DeviceContext::current(&st);
  if (!ctx) return st;
  const size_t n = (size_t)1 << log_n;
  const uint32_t W = crt_words(0, L);
  std::lock_guard<std::mutex> g(ctx->staging.lock);
  st = ctx->staging.reserve(n * L + n * W);
  if (st != kOk) return st;
  cudaStream_t s = ctx->stream();
  uint64_t* d_in = ctx->staging.ptr;
  uint64_t* d_out = d_in + n * L;
  cudaError_t e = cudaSuccess;
  for (uint32_t j = 0; j < L && e == cudaSuccess; ++j)
    e = cudaMemcpyAsync(d_in + j * n, limbs[j], n * 8, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return fail_cuda(e, "H2D limbs");
  st = crt_lift(d_out, d_in, 1, L, log_n, 0, s, ctx->device());
  if (st != kOk) return st;
  e = cudaMemcpyAsync(out, d_out, n * W * 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? kOk : fail_cuda(e, "D2H / synchronize");
}

}  // extern "C"
