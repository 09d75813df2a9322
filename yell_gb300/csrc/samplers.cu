// Seeded device samplers for RNS polynomials (poly<N>::set(...) of the
// reference, include/yell/details/poly.hpp:195-330).
//
// The reference draws from an unseeded stream (Salsa20 keyed from
// /dev/urandom).  Here every random word is splitmix64 of a counter, so a
// sample is a pure function of (seed, position) and can be regenerated on the
// host; the transformation of random words into coefficients follows the
// reference's algorithm for each distribution:
//   uniform  (include/yell/details/poly.hpp:200-228): per limb, w & (2^(floor(log2 p)+1) - 1), minus p
//            once if still >= p; independent words for every limb.
//   ZO(rho)  (include/yell/details/poly.hpp:267-280): one random byte r per coefficient, shared by all
//            limbs: r <= rho ? (r & 2 ? p - 1 : 1) : 0.
//   HWT(h)   (include/yell/details/poly.hpp:287-330): exactly h coefficients set to +-1 (same positions
//            and signs in every limb), the positions a pseudorandom h-subset (a
//            keyed permutation of the indices, below); sign bit 1 of a random
//            word: set -> +1, clear -> p - 1.
//   gaussian (include/yell/details/poly.hpp:236-260): a centred integer e per coefficient, shared by all
//            limbs, times an amplifier, mapped e < 0 ? p + e : e.  e comes from a
//            cumulative table of 64-bit thresholds (search of one random word), not
//            the reference's FastGaussianNoise lookup tables: the same truncated
//            distribution exp(-e^2 / 2 sigma^2) on |e| <= tail, a different algorithm.
// Random word k of a stream with seed s is splitmix64(s + (k + 1) * 0x9E3779B97F4A7C15).
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <string>
#include <vector>

#include "kernels.h"
#include "profiler.h"
#include "runtime.h"
#include "yell_gb300.h"

using namespace yell_gb300;

namespace {

__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__host__ __device__ __forceinline__ uint64_t rand_word(uint64_t seed, uint64_t k) {
  return mix64(seed + (k + 1) * 0x9E3779B97F4A7C15ull);
}

// Derived stream seeds for the parts of one sampler.
constexpr uint64_t kSeedPositions = 0x5ca1ab1e0ddba11ull;
constexpr uint64_t kSeedSigns = 0x0b5e55edc0ffee5ull;

// A warp writes 128 consecutive words per step as two 512-byte stores: lane j
// holds words 2j, 2j + 1 and 64 + 2j, 65 + 2j of the chunk.  The total is a
// multiple of 8 words (N >= 8), so a pair never straddles two limbs.
__global__ void k_sample_uniform(uint64_t* out, uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0,
                                 const DevMod* __restrict__ mods, uint64_t seed) {
  const size_t words = ((size_t)count * L) << log_n;
  const uint32_t lane = threadIdx.x & 31u;
  const size_t warp = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5;
  const size_t warps = ((size_t)gridDim.x * blockDim.x) >> 5;
  for (size_t c = warp << 7; c < words; c += warps << 7) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const size_t k = c + ((size_t)h << 6) + (lane << 1);
      if (k >= words) break;
      const uint32_t l = (uint32_t)(k >> log_n) % L;
      const uint64_t p = __ldg(&mods[cm0 + l].p);
      const uint64_t mask = (2ull << (63 - __clzll(p))) - 1ull;  // 2^(floor(log2 p) + 1) - 1
      const uint64_t z = seed + (k + 1) * 0x9E3779B97F4A7C15ull;  // counter of word k; + gamma per word
      uint64_t v0 = mix64(z) & mask, v1 = mix64(z + 0x9E3779B97F4A7C15ull) & mask;
      if (v0 >= p) v0 -= p;
      if (v1 >= p) v1 -= p;
      *reinterpret_cast<ulonglong2*>(out + k) = make_ulonglong2(v0, v1);
    }
  }
}

// mode 0: ZO with threshold rho; mode 1: gaussian through the cumulative
// table.  Two adjacent coefficients per thread (N >= 8 is even), so every
// limb row is written with 16-byte stores.
__device__ __forceinline__ int64_t shared_int(uint64_t r, int mode, uint32_t rho, const uint64_t* __restrict__ cdt,
                                              uint32_t cdt_len, int32_t tail, uint64_t amplifier) {
  if (mode == 0) {
    const uint32_t byte = (uint32_t)(r & 0xFF);
    return byte <= rho ? ((byte & 2) ? -1 : 1) : 0;
  }
  // first index with r < cdt[idx] (upper bound), clamped to the table
  uint32_t lo = 0, hi = cdt_len;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (r < __ldg(&cdt[mid])) hi = mid;
    else lo = mid + 1;
  }
  if (lo >= cdt_len) lo = cdt_len - 1;
  return ((int64_t)lo - tail) * (int64_t)amplifier;
}

__global__ void k_sample_shared_int(uint64_t* out, uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0,
                                    const DevMod* __restrict__ mods, uint64_t seed, int mode, uint32_t rho,
                                    const uint64_t* __restrict__ cdt, uint32_t cdt_len, int32_t tail,
                                    uint64_t amplifier) {
  const size_t pairs = ((size_t)count << log_n) >> 1;
  const uint32_t nmask = (1u << log_n) - 1u;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < pairs; t += (size_t)gridDim.x * blockDim.x) {
    const size_t k = t << 1;
    const int64_t e0 = shared_int(rand_word(seed, k), mode, rho, cdt, cdt_len, tail, amplifier);
    const int64_t e1 = shared_int(rand_word(seed, k + 1), mode, rho, cdt, cdt_len, tail, amplifier);
    const size_t poly = k >> log_n;
    const uint32_t i = (uint32_t)k & nmask;
    for (uint32_t l = 0; l < L; ++l) {
      const uint64_t p = __ldg(&mods[cm0 + l].p);
      *reinterpret_cast<ulonglong2*>(out + (((poly * L) + l) << log_n) + i) =
          make_ulonglong2(e0 < 0 ? p + (uint64_t)e0 : (uint64_t)e0, e1 < 0 ? p + (uint64_t)e1 : (uint64_t)e1);
    }
  }
}

// HWT: coefficient i of poly j is nonzero exactly when pi_j(i) < h, pi_j a
// keyed pseudorandom permutation of [0, N) (a 6-round Feistel network over
// the log2 N index bits, alternating halves of floor/ceil(log2 N / 2) bits,
// round function splitmix64 of the round key plus the half).  A permutation
// maps exactly h indices below h, so every poly has Hamming weight h; the
// positions are a pseudorandom h-subset, as the reference's reservoir
// sampling over a PRNG stream gives (details/poly.hpp:282-325).
constexpr int kFeistelRounds = 6;

__host__ __device__ __forceinline__ uint32_t feistel(uint32_t x, uint32_t bits, uint64_t key) {
  uint32_t b = bits >> 1, a = bits - b;  // low field b bits, high field a bits
  for (int r = 0; r < kFeistelRounds; ++r) {
    const uint32_t lo = x & ((1u << b) - 1u), hi = x >> b;
    const uint32_t f = (uint32_t)mix64(rand_word(key, (uint64_t)r) + lo);
    x = (lo << a) | ((hi ^ f) & ((1u << a) - 1u));
    const uint32_t t = a;  // the mixed field is now the low one
    a = b;
    b = t;
  }
  return x;
}

__global__ void k_sample_hwt(uint64_t* out, uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0,
                             const DevMod* __restrict__ mods, uint64_t seed, uint32_t h) {
  // two adjacent coefficients per thread: 16-byte stores per limb row
  const size_t pairs = ((size_t)count << log_n) >> 1;
  const uint32_t nmask = (1u << log_n) - 1u;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < pairs; t += (size_t)gridDim.x * blockDim.x) {
    const size_t k = t << 1;
    const size_t poly = k >> log_n;
    const uint32_t i = (uint32_t)k & nmask;
    const uint64_t key = rand_word(seed ^ kSeedPositions, poly);
    const bool take0 = feistel(i, log_n, key) < h, take1 = feistel(i + 1, log_n, key) < h;
    const bool plus0 = (rand_word(seed ^ kSeedSigns, k) & 2) != 0;
    const bool plus1 = (rand_word(seed ^ kSeedSigns, k + 1) & 2) != 0;
    for (uint32_t l = 0; l < L; ++l) {
      const uint64_t p = __ldg(&mods[cm0 + l].p);
      *reinterpret_cast<ulonglong2*>(out + (((poly * L) + l) << log_n) + i) =
          make_ulonglong2(take0 ? (plus0 ? 1ull : p - 1) : 0ull, take1 ? (plus1 ? 1ull : p - 1) : 0ull);
    }
  }
}

int grid_for(size_t items) {
  const size_t g = (items + 255) / 256;
  return (int)(g < 152 * 16 ? (g ? g : 1) : 152 * 16);
}

// Cumulative table of P(e) ~ exp(-e^2 / 2 sigma^2) on |e| <= tail, scaled to
// 64-bit thresholds (the last one is 2^64 - 1).
std::vector<uint64_t> gaussian_cdt(double sigma, int tail) {
  std::vector<long double> w;
  long double sum = 0;
  for (int e = -tail; e <= tail; ++e) {
    const long double v = std::exp(-(long double)e * e / (2.0L * sigma * sigma));
    w.push_back(v);
    sum += v;
  }
  std::vector<uint64_t> cdt;
  long double acc = 0;
  for (size_t i = 0; i < w.size(); ++i) {
    acc += w[i];
    long double t = std::floor(acc / sum * 18446744073709551616.0L);
    cdt.push_back(t >= 18446744073709551615.0L ? ~0ull : (uint64_t)t);
  }
  cdt.back() = ~0ull;
  return cdt;
}

constexpr uint32_t kMaxGaussianTail = 1024;

// Device copies of the cumulative tables, one per (device, sigma, tail), built
// on first use and kept for the life of the process (a few KB each).
int gaussian_table(int device, double sigma, uint32_t tail, const uint64_t** out, uint32_t* len) {
  static std::mutex mu;
  static std::map<std::tuple<int, uint64_t, uint32_t>, std::pair<uint64_t*, uint32_t>> tables;
  uint64_t sigma_bits;
  std::memcpy(&sigma_bits, &sigma, sizeof sigma_bits);
  const auto key = std::make_tuple(device, sigma_bits, tail);
  std::lock_guard<std::mutex> g(mu);
  auto it = tables.find(key);
  if (it == tables.end()) {
    const std::vector<uint64_t> cdt = gaussian_cdt(sigma, (int)tail);
    uint64_t* d = nullptr;
    cudaError_t e = lib_malloc(&d, cdt.size() * sizeof(uint64_t));
    if (e != cudaSuccess) return fail_cuda(e, "cudaMalloc(gaussian table)");
    e = cudaMemcpy(d, cdt.data(), cdt.size() * sizeof(uint64_t), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      cudaFree(d);
      return fail_cuda(e, "upload gaussian table");
    }
    it = tables.emplace(key, std::make_pair(d, (uint32_t)cdt.size())).first;
  }
  *out = it->second.first;
  *len = it->second.second;
  return kOk;
}

struct SamplerArgs {
  DeviceContext* ctx = nullptr;
  const DevMod* mods = nullptr;
  cudaStream_t st = nullptr;
};

int prepare(uint64_t* d_out, uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0, void* stream,
            SamplerArgs* a) {
  if (!d_out || count == 0) return fail(kInvalidArgument, "null output or zero count");
  if (reinterpret_cast<uintptr_t>(d_out) % 16) return fail(kInvalidArgument, "d_out is not 16-byte aligned");
  int st = check_degree(log_n);
  if (st != kOk) return st;
  st = check_moduli(cm0, L);
  if (st != kOk) return st;
  st = check_limbs(count, L, log_n, nullptr);
  if (st != kOk) return st;
  a->ctx = DeviceContext::current(&st);
  if (!a->ctx) return st;
  st = a->ctx->ensure_tables(log_n, cm0, L, &a->mods);
  if (st != kOk) return st;
  a->st = stream ? static_cast<cudaStream_t>(stream) : a->ctx->stream();
  return kOk;
}

}  // namespace

extern "C" {

int yell_dev_sample_uniform(uint64_t* d_out, uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0,
                            uint64_t seed, void* stream) {
  SamplerArgs a;
  int st = prepare(d_out, count, L, log_n, cm0, stream, &a);
  if (st != kOk) return st;
  LaunchScope ps("sample_uniform", a.st);
  k_sample_uniform<<<grid_for((((size_t)count * L) << log_n) >> 2), 256, 0, a.st>>>(d_out, count, L, log_n, cm0,
                                                                            a.mods, seed);
  g_kernel_launches += 1;
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? kOk : fail_cuda(e, "sample_uniform");
}

int yell_dev_sample_zo(uint64_t* d_out, uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0,
                       uint32_t rho, uint64_t seed, void* stream) {
  if (rho > 255) return fail(kInvalidArgument, "rho must be a byte (0..255)");
  SamplerArgs a;
  int st = prepare(d_out, count, L, log_n, cm0, stream, &a);
  if (st != kOk) return st;
  LaunchScope ps("sample_zo", a.st);
  k_sample_shared_int<<<grid_for(((size_t)count << log_n) >> 1), 256, 0, a.st>>>(
      d_out, count, L, log_n, cm0, a.mods, seed, 0, rho, nullptr, 0, 0, 1);
  g_kernel_launches += 1;
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? kOk : fail_cuda(e, "sample_zo");
}

int yell_dev_sample_hwt(uint64_t* d_out, uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0,
                        uint32_t h, uint64_t seed, void* stream) {
  if (h == 0 || h > (1u << log_n)) return fail(kInvalidArgument, "hamming weight must be in [1, N]");
  SamplerArgs a;
  int st = prepare(d_out, count, L, log_n, cm0, stream, &a);
  if (st != kOk) return st;
  LaunchScope ps("sample_hwt", a.st);
  k_sample_hwt<<<grid_for(((size_t)count << log_n) >> 1), 256, 0, a.st>>>(d_out, count, L, log_n, cm0, a.mods,
                                                                          seed, h);
  g_kernel_launches += 1;
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? kOk : fail_cuda(e, "sample_hwt");
}

int yell_dev_sample_gaussian(uint64_t* d_out, uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0,
                             double sigma, uint32_t tail, uint64_t amplifier, uint64_t seed, void* stream) {
  if (!(sigma > 0) || !(sigma < 1e6) || tail == 0 || tail > kMaxGaussianTail)
    return fail(kInvalidArgument, "need 0 < sigma < 1e6 and 0 < tail <= 1024");
  if (amplifier == 0 || (unsigned __int128)tail * amplifier >= (1ull << 61))
    return fail(kInvalidArgument, "tail * amplifier must be below 2^61 (below every modulus)");
  SamplerArgs a;
  int st = prepare(d_out, count, L, log_n, cm0, stream, &a);
  if (st != kOk) return st;
  const uint64_t* cdt = nullptr;
  uint32_t len = 0;
  st = gaussian_table(a.ctx->device(), sigma, tail, &cdt, &len);
  if (st != kOk) return st;
  LaunchScope ps("sample_gaussian", a.st);
  k_sample_shared_int<<<grid_for(((size_t)count << log_n) >> 1), 256, 0, a.st>>>(
      d_out, count, L, log_n, cm0, a.mods, seed, 1, 0, cdt, len, (int32_t)tail, amplifier);
  g_kernel_launches += 1;
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? kOk : fail_cuda(e, "sample_gaussian");
}

}  // extern "C"
