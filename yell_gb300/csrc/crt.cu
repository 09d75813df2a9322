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
// The multi-word sums run over 32-bit digits: a thread owns one coefficient
// and keeps its y_j in shared memory; the cofactor digits are staged per tile
// of output digits and shared by the block; x is written as W little-endian
// words per coefficient, W = words of Q, coefficient-major.
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

constexpr uint32_t kCrtMaxModuli = 400;  // 32 threads * 400 words * 8 B = 100 KB of y per block

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
  cudaError_t e = lib_malloc(&t->mods, L * sizeof(CrtConst));
  if (e == cudaSuccess) e = lib_malloc(&t->cofactors, cof.size() * 8);
  if (e == cudaSuccess) e = lib_malloc(&t->q, (size_t)W * 8);
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

// 32-bit digit d of a little-endian word array of `words` words (0 outside).
__device__ __forceinline__ uint32_t digit(const uint64_t* w, int d, uint32_t words) {
  return (d >= 0 && (uint32_t)d < 2 * words) ? __ldg(reinterpret_cast<const uint32_t*>(w) + d) : 0u;
}

// (r0, r1, r2) += a * b, a 64-bit product into a 96-bit accumulator.
__device__ __forceinline__ void mac32(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t a, uint32_t b) {
  asm("mad.lo.cc.u32 %0, %3, %4, %0;\n\t"
      "madc.hi.cc.u32 %1, %3, %4, %1;\n\t"
      "addc.u32 %2, %2, 0;"
      : "+r"(r0), "+r"(r1), "+r"(r2)
      : "r"(a), "r"(b));
}

// d = a - b - bin (32-bit), returns the borrow out.
__device__ __forceinline__ uint32_t sub_borrow32(uint32_t a, uint32_t b, uint32_t bin, uint32_t* d) {
  const uint32_t t = a - b;
  *d = t - bin;
  return (uint32_t)(a < b) | (uint32_t)(t < bin);
}

__device__ __forceinline__ uint32_t sub_borrow(uint64_t a, uint64_t b, uint32_t bin, uint64_t* d) {
  const uint64_t t = a - b;
  *d = t - bin;
  return (uint32_t)(a < b) | (uint32_t)(t < (uint64_t)bin);
}

// Output digits are produced in tiles of kDigitTile 32-bit digits.  For one
// tile the block stages digits [e0 - 1, e0 + kDigitTile) of every cofactor in
// shared memory; each thread then runs over j once, adding
// y_j[0] * C_j[d] + y_j[1] * C_j[d - 1] into one 96-bit accumulator per digit
// d of the tile (independent chains), and finally resolves the carries digit
// by digit, subtracting v * Q on the way.
constexpr int kDigitTile = 8;  // 8: 72 registers, 0.77 ms at L = 32; 16: 114 registers, 0.87 ms

template <int T>
__global__ void __launch_bounds__(T) k_crt_lift(uint64_t* __restrict__ out, const uint64_t* __restrict__ in,
                                                uint32_t count, uint32_t L, uint32_t log_n,
                                                const CrtConst* __restrict__ mods, const uint64_t* __restrict__ cof,
                                                const uint64_t* __restrict__ qw, uint32_t W) {
  extern __shared__ __align__(16) uint64_t smem_crt[];
  uint64_t* ys = smem_crt;                                          // [L][T]
  uint32_t* cs = reinterpret_cast<uint32_t*>(smem_crt + (size_t)L * T);  // [L][kDigitTile + 1]
  constexpr int CT = kDigitTile + 1;
  const uint64_t coeffs = (uint64_t)count << log_n;
  const uint64_t g = (uint64_t)blockIdx.x * T + threadIdx.x;
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
      y = mulmod_shoup(in[(poly * L + j) * n + i], m.inv, m.inv_s, m.q);
      const uint64_t pl = y * m.c, ph = __umul64hi(y, m.c);
      const uint64_t f = (pl >> 61) | (ph << 3);  // floor(y c / 2^61) < 2^64
      asm("add.cc.u64 %0, %0, %2;\n\taddc.u64 %1, %1, 0;" : "+l"(f_lo), "+l"(f_hi) : "l"(f));
    }
    ys[j * T + threadIdx.x] = y;
  }
  const uint64_t v = f_hi;
  const uint32_t v0 = (uint32_t)v, v1 = (uint32_t)(v >> 32);

  uint64_t* dst = out + g * W;
  const int digits = 2 * (int)W + 2;  // two digits past Q for the borrow chains
  uint64_t cx = 0, cq = 0;            // carries of sum y_j (Q/q_j) and of v Q, in digits
  uint32_t br = 0, bq = 0, lo_digit = 0;
  for (int e0 = 0; e0 < digits; e0 += kDigitTile) {
    __syncthreads();  // previous tile's cofactor digits are no longer read
    for (uint32_t k = threadIdx.x; k < L * CT; k += T) {
      const uint32_t j = k / CT;
      const int d = e0 - 1 + (int)(k - j * CT);
      cs[k] = digit(cof + (size_t)j * W, d, W);
    }
    __syncthreads();
    if (live) {
      uint32_t r0[kDigitTile], r1[kDigitTile], r2[kDigitTile];
#pragma unroll
      for (int t = 0; t < kDigitTile; ++t) r0[t] = r1[t] = r2[t] = 0;
      for (uint32_t j = 0; j < L; ++j) {
        const uint64_t y = ys[j * T + threadIdx.x];
        const uint32_t y0 = (uint32_t)y, y1 = (uint32_t)(y >> 32);
        const uint32_t* c = cs + j * CT;  // c[t + 1] = C_j[e0 + t]
        uint32_t prev = c[0];
#pragma unroll
        for (int t = 0; t < kDigitTile; ++t) {
          const uint32_t cur = c[t + 1];
          mac32(r0[t], r1[t], r2[t], y0, cur);
          mac32(r0[t], r1[t], r2[t], y1, prev);
          prev = cur;
        }
      }
#pragma unroll
      for (int t = 0; t < kDigitTile; ++t) {
        const int d = e0 + t;
        if (d < digits) {
          // x digit: accumulator + carry
          uint64_t xl = ((uint64_t)r1[t] << 32 | r0[t]);
          const uint64_t s = xl + cx;
          const uint64_t xh = (uint64_t)r2[t] + (s < xl ? 1u : 0u);
          const uint32_t xd = (uint32_t)s;
          cx = (s >> 32) | (xh << 32);
          // (v Q) digit
          const uint32_t qd0 = digit(qw, d, W), qd1 = digit(qw, d - 1, W);
          const uint64_t pq = (uint64_t)v0 * qd0, pq2 = (uint64_t)v1 * qd1;
          const uint64_t sq = pq + pq2;
          const uint64_t sq2 = sq + cq;
          const uint64_t qh = (uint64_t)(sq < pq) + (uint64_t)(sq2 < sq);
          const uint32_t qd = (uint32_t)sq2;
          cq = (sq2 >> 32) | (qh << 32);
          uint32_t rd, ad;
          br = sub_borrow32(xd, qd, br, &rd);
          bq = sub_borrow32(rd, qd0, bq, &ad);
          if (d < 2 * (int)W) {
            if (d & 1) dst[d >> 1] = (uint64_t)rd << 32 | lo_digit;
            else lo_digit = rd;
          }
        }
      }
    }
  }
  if (live && bq == 0) {  // x - vQ >= Q: the estimate of v was one short
    uint32_t b = 0;
    for (uint32_t w = 0; w < W; ++w) {
      uint64_t d;
      b = sub_borrow(dst[w], __ldg(&qw[w]), b, &d);
      dst[w] = d;
    }
  }
}

size_t crt_smem(uint32_t L, int threads) {
  return (size_t)L * threads * sizeof(uint64_t) + (size_t)L * (kDigitTile + 1) * sizeof(uint32_t);
}

int crt_lift(uint64_t* d_out, const uint64_t* d_in, uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0,
             cudaStream_t st, int device) {
  const CrtTables* t = nullptr;
  int s = crt_tables(device, cm0, L, &t);
  if (s != kOk) return s;
  // 64 threads per block while their y_j fit in 160 KB of shared memory, else 32
  // (128-thread blocks measured 2% slower at L = 32)
  const int threads = crt_smem(L, 64) <= (160u << 10) ? 64 : 32;
  const size_t smem = crt_smem(L, threads);
  cudaError_t e = cudaSuccess;
  {
    // the shared-memory limit is a per-device attribute of each kernel
    static std::mutex mu;
    static std::set<int> done;
    std::lock_guard<std::mutex> g(mu);
    if (!done.count(device)) {
      e = cudaFuncSetAttribute(k_crt_lift<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(160u << 10));
      if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_crt_lift<32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)crt_smem(kCrtMaxModuli, 32));
      if (e != cudaSuccess) return fail_cuda(e, "crt attributes");
      done.insert(device);
    }
  }
  const uint64_t coeffs = (uint64_t)count << log_n;
  const uint32_t blocks = (uint32_t)((coeffs + threads - 1) / threads);
  {
    LaunchScope ps("crt_lift", st);
    if (threads == 64)
      k_crt_lift<64><<<blocks, 64, smem, st>>>(d_out, d_in, count, L, log_n, t->mods, t->cofactors, t->q, t->W);
    else
      k_crt_lift<32><<<blocks, 32, smem, st>>>(d_out, d_in, count, L, log_n, t->mods, t->cofactors, t->q, t->W);
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
  st = check_limbs(count, L, log_n, nullptr);
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
