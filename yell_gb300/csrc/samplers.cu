// Seeded device samplers for RNS polynomials (poly<N>::set(...) of the
// reference, include/yell/details/poly.hpp:195-330).
//
// The reference draws every random byte from yell::fastrandombytes, an
// unseeded stream (Salsa20 keyed from /dev/urandom).  Here the stream is a
// counter stream: random word k of the stream with seed s is
// splitmix64(s + (k + 1) * 0x9E3779B97F4A7C15), and its bytes are those words
// in little-endian order.  A sample is a pure function of (seed, position),
// and the coefficients are what the reference's own set(...) makes of the
// same stream (checked against the reference's code run on this stream):
//   uniform  (details/poly.hpp:200-228): limb after limb, poly after poly,
//            word w -> w & (2^(floor(log2 p)+1) - 1), minus p once if still >= p.
//   ZO(rho)  (details/poly.hpp:267-280): one byte r of the stream per
//            coefficient (poly after poly, shared by all limbs):
//            r <= rho ? (r & 2 ? p - 1 : 1) : 0.
//   HWT(h)   (details/poly.hpp:287-330): poly j draws from its own stream,
//            seeded with word j of the batch seed's stream.  Reservoir
//            sampling of h positions: the first h positions, then for
//            k = h .. N-1 a draw d, rejected while d > floor((2^64-1)/k) * k
//            and taken mod k otherwise, replaces position d when d < h.  The
//            positions, sorted, get signs from the h words that follow the
//            draws (the reference refills its buffer h words at a time, so
//            they start at word ceil(draws / h) * h): bit 1 set -> +1, clear
//            -> p - 1.  The same positions and signs in every limb.
//   gaussian (details/poly.hpp:236-260): a centred integer e per coefficient,
//            shared by all limbs, times the amplifier, mapped e < 0 ? p + e : e.
//            e is found by inversion of one random word against a cumulative
//            table of 64-bit thresholds of exp(-e^2 / 2 sigma^2) on |e| <= tail.
//            The reference's FastGaussianNoise (include/yell/prng/
//            FastGaussianNoise.hpp) inverts a wider random number against
//            the same cumulative distribution through lookup tables; the two
//            agree in distribution (per value within 2^-63), not draw for draw.
#include <algorithm>
#include <cmath>
#include <cstdlib>
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

// A warp writes 128 consecutive words per step as two 512-byte stores: lane j
// holds words 2j, 2j + 1 and 64 + 2j, 65 + 2j of the chunk.  The total is a
// multiple of 8 words (N >= 8), so a pair never straddles two limbs.  Each
// warp walks one contiguous run of chunks, so the limb (and with it p and the
// mask) changes rarely and is worked out only when it does.
__global__ void k_sample_uniform(uint64_t* out, uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0,
                                 const DevMod* __restrict__ mods, uint64_t seed) {
  grid_dep_launch();
  grid_dep_wait();  // out may be in use by the stream's previous kernel
  const size_t words = ((size_t)count * L) << log_n;
  const size_t chunks = (words + 127) >> 7;
  const uint32_t lane = threadIdx.x & 31u;
  const size_t warp = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5;
  const size_t warps = ((size_t)gridDim.x * blockDim.x) >> 5;
  const size_t per = (chunks + warps - 1) / warps;
  const size_t c0 = warp * per, c1 = min(c0 + per, chunks);
  size_t row = ~(size_t)0;
  uint64_t p = 0, mask = 0;
  if (log_n >= 7) {
    // A chunk lies inside one limb and the total is a multiple of 128 words:
    // no bound check, one limb check and one counter product per chunk.
    constexpr uint64_t kGamma = 0x9E3779B97F4A7C15ull;
    for (size_t ch = c0; ch < c1; ++ch) {
      const size_t k = (ch << 7) + (lane << 1);
      if ((k >> log_n) != row) {
        row = k >> log_n;
        p = __ldg(&mods[cm0 + (uint32_t)(row % L)].p);
        mask = (2ull << (63 - __clzll(p))) - 1ull;  // 2^(floor(log2 p) + 1) - 1
      }
      const uint64_t z = seed + (k + 1) * kGamma;  // counter of word k; + gamma per word
      const uint64_t v0 = csub(mix64(z) & mask, p), v1 = csub(mix64(z + kGamma) & mask, p);
      const uint64_t v2 = csub(mix64(z + 64 * kGamma) & mask, p), v3 = csub(mix64(z + 65 * kGamma) & mask, p);
      *reinterpret_cast<ulonglong2*>(out + k) = make_ulonglong2(v0, v1);
      *reinterpret_cast<ulonglong2*>(out + k + 64) = make_ulonglong2(v2, v3);
    }
    return;
  }
  for (size_t ch = c0; ch < c1; ++ch) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const size_t k = (ch << 7) + ((size_t)h << 6) + (lane << 1);
      if (k >= words) break;
      if ((k >> log_n) != row) {
        row = k >> log_n;
        p = __ldg(&mods[cm0 + (uint32_t)(row % L)].p);
        mask = (2ull << (63 - __clzll(p))) - 1ull;  // 2^(floor(log2 p) + 1) - 1
      }
      const uint64_t z = seed + (k + 1) * 0x9E3779B97F4A7C15ull;  // counter of word k; + gamma per word
      uint64_t v0 = mix64(z) & mask, v1 = mix64(z + 0x9E3779B97F4A7C15ull) & mask;
      if (v0 >= p) v0 -= p;
      if (v1 >= p) v1 -= p;
      *reinterpret_cast<ulonglong2*>(out + k) = make_ulonglong2(v0, v1);
    }
  }
}

__device__ __forceinline__ uint64_t residue(int64_t e, uint64_t p) { return e < 0 ? p + (uint64_t)e : (uint64_t)e; }

// Writes the signed coefficients e0, e1 of positions (i, i + 1) of `poly` to
// every limb, one 16-byte store per limb row.
__device__ __forceinline__ void put_pair(uint64_t* out, size_t poly, uint32_t i, uint32_t L, uint32_t log_n,
                                         uint32_t cm0, const DevMod* __restrict__ mods, int64_t e0, int64_t e1) {
  for (uint32_t l = 0; l < L; ++l) {
    const uint64_t p = __ldg(&mods[cm0 + l].p);
    *reinterpret_cast<ulonglong2*>(out + (((poly * L) + l) << log_n) + i) =
        make_ulonglong2(residue(e0, p), residue(e1, p));
  }
}

// ZO: coefficient k (poly-major over the batch) takes byte k of the stream.
// Two adjacent coefficients per thread (k even), both bytes of one word.
__global__ void k_sample_zo(uint64_t* out, uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0,
                            const DevMod* __restrict__ mods, uint64_t seed, uint32_t rho) {
  grid_dep_launch();
  grid_dep_wait();  // out may be in use by the stream's previous kernel
  const size_t pairs = ((size_t)count << log_n) >> 1;
  const uint32_t nmask = (1u << log_n) - 1u;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < pairs; t += (size_t)gridDim.x * blockDim.x) {
    const size_t k = t << 1;
    const uint64_t w = rand_word(seed, k >> 3);
    const uint32_t sh = 8u * (uint32_t)(k & 7);
    const uint32_t r0 = (uint32_t)(w >> sh) & 0xFFu, r1 = (uint32_t)(w >> (sh + 8)) & 0xFFu;
    const int64_t e0 = r0 <= rho ? ((r0 & 2) ? -1 : 1) : 0;
    const int64_t e1 = r1 <= rho ? ((r1 & 2) ? -1 : 1) : 0;
    put_pair(out, k >> log_n, (uint32_t)k & nmask, L, log_n, cm0, mods, e0, e1);
  }
}

// Gaussian: coefficient k takes word k; e is the first index with
// word < cdt[index], minus the tail.
__device__ __forceinline__ int64_t gaussian_int(uint64_t r, const uint64_t* __restrict__ cdt, uint32_t cdt_len,
                                                int32_t tail, uint64_t amplifier) {
  uint32_t lo = 0, hi = cdt_len;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (r < __ldg(&cdt[mid])) hi = mid;
    else lo = mid + 1;
  }
  if (lo >= cdt_len) lo = cdt_len - 1;
  return ((int64_t)lo - tail) * (int64_t)amplifier;
}

__global__ void k_sample_gaussian(uint64_t* out, uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0,
                                  const DevMod* __restrict__ mods, uint64_t seed, const uint64_t* __restrict__ cdt,
                                  uint32_t cdt_len, int32_t tail, uint64_t amplifier) {
  grid_dep_launch();
  grid_dep_wait();  // out may be in use by the stream's previous kernel
  const size_t pairs = ((size_t)count << log_n) >> 1;
  const uint32_t nmask = (1u << log_n) - 1u;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < pairs; t += (size_t)gridDim.x * blockDim.x) {
    const size_t k = t << 1;
    const int64_t e0 = gaussian_int(rand_word(seed, k), cdt, cdt_len, tail, amplifier);
    const int64_t e1 = gaussian_int(rand_word(seed, k + 1), cdt, cdt_len, tail, amplifier);
    put_pair(out, k >> log_n, (uint32_t)k & nmask, L, log_n, cm0, mods, e0, e1);
  }
}

// ---- HWT ----------------------------------------------------------------------
// Scratch per poly: the h reservoir entries, a control pair, and an N-bit set
// of the chosen positions with the number of set bits before each 32-bit word
// (the rank of a position among the sorted positions).
struct HwtCtl {
  uint32_t first_reject;  // smallest k whose draw was rejected (N when none)
  uint32_t draws;         // draws the reservoir consumed, rejections included
};

// Largest draw the reference accepts for bound k: floor((2^64 - 1) / k) * k.
__host__ __device__ __forceinline__ uint64_t accept_limit(uint32_t k) { return (~0ull / k) * k; }

__global__ void k_hwt_init(uint32_t* hitted, HwtCtl* ctl, uint32_t count, uint32_t h, uint32_t n) {
  grid_dep_launch();
  grid_dep_wait();  // the scratch may be the previous kernel's
  const size_t total = (size_t)count * h;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x)
    hitted[t] = (uint32_t)(t % h);
  for (size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x; j < count; j += (size_t)gridDim.x * blockDim.x)
    ctl[j] = HwtCtl{n, n - h};
}

// Draw d of poly j belongs to k = h + d as long as no earlier draw of the
// poly was rejected, which makes every draw independent: the last k that hits
// a reservoir slot owns it (atomicMax over the initial slot index).  A
// rejection (probability below k / 2^64) shifts every later draw; it is
// recorded, and the poly is redone in draw order by k_hwt_rank.  Poly j is
// grid row j; the acceptance limit floor((2^64 - 1) / k) * k is at least
// 2^64 - k, so only a draw above that needs the division.
__global__ void k_hwt_reservoir(uint32_t* hitted, HwtCtl* ctl, uint32_t log_n, uint32_t h, uint64_t seed) {
  grid_dep_launch();
  const uint32_t per = (1u << log_n) - h;
  const uint32_t j = blockIdx.y;
  const uint64_t s = rand_word(seed, j);
  grid_dep_wait();  // the initialised slots
  for (uint32_t d = blockIdx.x * blockDim.x + threadIdx.x; d < per; d += gridDim.x * blockDim.x) {
    const uint32_t k = h + d;
    const uint64_t w = rand_word(s, d);
    if (w > 0ull - (uint64_t)k && w > accept_limit(k)) {
      atomicMin(&ctl[j].first_reject, k);
      continue;
    }
    const uint32_t pos = (uint32_t)(w % k);
    if (pos < h) atomicMax(&hitted[(size_t)j * h + pos], k);
  }
}

constexpr int kRankThreads = 1024;

// One CTA per poly.  Redoes the reservoir in draw order (one thread) when a
// draw was rejected or `sequential` is set, then marks the chosen positions
// in a shared bit set and writes it with the exclusive prefix of set bits per
// 32-bit word.  Dynamic shared memory: max(N / 32, 1) words + 32 words.
__global__ void __launch_bounds__(kRankThreads) k_hwt_rank(uint32_t* hitted, HwtCtl* ctl, uint32_t* bits,
                                                           uint32_t* prefix, uint32_t log_n, uint32_t h, uint64_t seed,
                                                           int sequential) {
  extern __shared__ uint32_t sbits[];
  grid_dep_launch();
  const uint32_t j = blockIdx.x, tid = threadIdx.x;
  const uint32_t n = 1u << log_n, nw = n >= 32 ? n >> 5 : 1u;
  uint32_t* hit = hitted + (size_t)j * h;
  uint32_t* warp_sum = sbits + nw;
  grid_dep_wait();  // the reservoir
  if (tid == 0 && (sequential || ctl[j].first_reject < n)) {
    const uint64_t s = rand_word(seed, j);
    for (uint32_t t = 0; t < h; ++t) hit[t] = t;
    uint64_t d = 0;
    for (uint32_t k = h; k < n; ++k) {
      uint64_t w;
      do w = rand_word(s, d++);
      while (w > accept_limit(k));
      const uint32_t pos = (uint32_t)(w % k);
      if (pos < h) hit[pos] = k;
    }
    ctl[j].draws = (uint32_t)d;
  }
  for (uint32_t w = tid; w < nw; w += kRankThreads) sbits[w] = 0;
  __syncthreads();
  for (uint32_t t = tid; t < h; t += kRankThreads) {
    const uint32_t v = hit[t];
    atomicOr(&sbits[v >> 5], 1u << (v & 31u));
  }
  __syncthreads();
  // exclusive scan of the per-word bit counts: each thread a contiguous chunk
  const uint32_t chunk = (nw + kRankThreads - 1) / kRankThreads;
  const uint32_t w0 = min(tid * chunk, nw), w1 = min(w0 + chunk, nw);
  uint32_t mine = 0;
  for (uint32_t w = w0; w < w1; ++w) mine += __popc(sbits[w]);
  const uint32_t lane = tid & 31u, warp = tid >> 5;
  uint32_t incl = mine;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= (uint32_t)o) incl += v;
  }
  if (lane == 31) warp_sum[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t ws = warp_sum[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t v = __shfl_up_sync(0xffffffffu, ws, o);
      if (lane >= (uint32_t)o) ws += v;
    }
    warp_sum[lane] = ws;  // inclusive over warps
  }
  __syncthreads();
  uint32_t run = incl - mine + (warp ? warp_sum[warp - 1] : 0u);
  for (uint32_t w = w0; w < w1; ++w) {
    const uint32_t b = sbits[w];
    bits[(size_t)j * nw + w] = b;
    prefix[(size_t)j * nw + w] = run;
    run += __popc(b);
  }
}

// Coefficient i of poly j: chosen when its bit is set; its sign is sign word
// (signs start) + rank of the position of the poly's stream.
__global__ void k_hwt_write(uint64_t* out, uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0,
                            const DevMod* __restrict__ mods, uint64_t seed, uint32_t h, const HwtCtl* __restrict__ ctl,
                            const uint32_t* __restrict__ bits, const uint32_t* __restrict__ prefix) {
  const size_t pairs = ((size_t)count << log_n) >> 1;
  const uint32_t nmask = (1u << log_n) - 1u;
  const uint32_t nw = log_n >= 5 ? 1u << (log_n - 5) : 1u;
  grid_dep_wait();  // the bit sets and ranks
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < pairs; t += (size_t)gridDim.x * blockDim.x) {
    const size_t k = t << 1;
    const size_t poly = k >> log_n;
    const uint32_t i = (uint32_t)k & nmask;  // even: i and i + 1 share a bit word
    const size_t wi = poly * nw + (i >> 5);
    const uint32_t b = __ldg(&bits[wi]);
    const uint32_t sh = i & 31u;
    const uint32_t b0 = (b >> sh) & 1u, b1 = (b >> (sh + 1)) & 1u;
    int64_t e0 = 0, e1 = 0;
    if (b0 | b1) {
      const uint64_t s = rand_word(seed, poly);
      const uint32_t draws = __ldg(&ctl[poly].draws);
      const uint64_t signs = (uint64_t)((draws + h - 1) / h) * h;
      const uint32_t rank0 = __ldg(&prefix[wi]) + __popc(b & ((1u << sh) - 1u));
      if (b0) e0 = (rand_word(s, signs + rank0) & 2) ? 1 : -1;
      if (b1) e1 = (rand_word(s, signs + rank0 + b0) & 2) ? 1 : -1;
    }
    put_pair(out, poly, i, L, log_n, cm0, mods, e0, e1);
  }
}

int grid_for(size_t items) {
  const size_t g = (items + 255) / 256;
  return (int)(g < 152 * 16 ? (g ? g : 1) : 152 * 16);
}

// ---- Gaussian table ----------------------------------------------------------
// Thresholds t_e = floor(2^64 * S(e) / S(tail)), S(e) = the sum of
// exp(-j^2 c) over -tail <= j <= e, c = 1 / (2 sigma^2) as an IEEE double; the
// last threshold is 2^64 - 1.  Computed in 128-bit fixed point with integer
// operations only, so every host builds the same table (long double differs
// between x86 and Arm).
using u128 = unsigned __int128;
constexpr int kFix = 120;  // fractional bits of the fixed-point values

// floor(a * b / 2^s), 64 <= s <= 128, for a result below 2^128.
u128 mul_shr(u128 a, u128 b, int s) {
  const uint64_t a0 = (uint64_t)a, a1 = (uint64_t)(a >> 64), b0 = (uint64_t)b, b1 = (uint64_t)(b >> 64);
  const u128 p00 = (u128)a0 * b0, p01 = (u128)a0 * b1, p10 = (u128)a1 * b0, p11 = (u128)a1 * b1;
  const u128 mid = (p00 >> 64) + (uint64_t)p01 + (uint64_t)p10;
  const u128 lo = (mid << 64) | (uint64_t)p00;
  const u128 hi = p11 + (p01 >> 64) + (p10 >> 64) + (mid >> 64);
  return s == 128 ? hi : (hi << (128 - s)) | (lo >> s);
}

// ln 2 = sum over k >= 1 of 2^-k / k.
u128 ln2_fixed() {
  const u128 one = (u128)1 << kFix;
  u128 s = 0;
  for (int k = 1; k <= kFix; ++k) s += (one >> k) / (u128)k;
  return s;
}

// exp(-x) for a fixed-point x >= 0: x = n ln 2 + r, exp(-r) by its Taylor
// series (r < ln 2), shifted right by n.
u128 exp_neg_fixed(u128 x) {
  static const u128 ln2 = ln2_fixed();
  const u128 n = x / ln2;
  if (n >= (u128)kFix) return 0;
  const u128 r = x - n * ln2;
  u128 term = (u128)1 << kFix, pos = term, neg = 0;
  for (int k = 1; k < 64 && term != 0; ++k) {
    term = mul_shr(term, r, kFix) / (u128)k;
    if (k & 1) neg += term;
    else pos += term;
  }
  return (pos - neg) >> (int)n;
}

// floor(2^kFix / (2 sigma^2)) for the double sigma, exactly: sigma =
// m 2^(e - 53) with a 53-bit integer m, so the value is floor(2^P / m^2) with
// P = kFix - 1 - 2 (e - 53), found by binary long division.  Only called for
// 1/(2 sigma^2) < 100 (P stays below 233, the quotient below 2^128).
u128 inv_two_sigma_sq_fixed(double sigma) {
  int e = 0;
  const double f = std::frexp(sigma, &e);
  const u128 m = (u128)(uint64_t)std::ldexp(f, 53);
  const u128 M = m * m;  // < 2^106
  const int P = kFix - 1 - 2 * (e - 53);
  u128 q = 0, r = 0;
  for (int bit = P; bit >= 0; --bit) {
    r = (r << 1) | (bit == P ? 1u : 0u);
    if (r >= M) {
      r -= M;
      q |= (u128)1 << bit;
    }
  }
  return q;
}

std::vector<uint64_t> gaussian_cdt(double sigma, int tail) {
  const double c = 1.0 / (2.0 * sigma * sigma);  // only to skip negligible weights
  const u128 cf = c < 100.0 ? inv_two_sigma_sq_fixed(sigma) : 0;
  std::vector<u128> w(2 * (size_t)tail + 1);
  u128 total = 0;
  for (int j = -tail; j <= tail; ++j) {
    u128 v = 0;
    const double x = (double)j * j * c;
    if (j == 0) {
      v = (u128)1 << kFix;
    } else if (x < 100.0) {
      v = exp_neg_fixed(cf * (u128)((uint64_t)j * (uint64_t)j));
    }
    w[j + tail] = v >> 8;  // 2^112 scale: the sum of at most 2049 weights stays below 2^124
    total += w[j + tail];
  }
  std::vector<uint64_t> cdt(w.size());
  u128 acc = 0;
  for (size_t i = 0; i < w.size(); ++i) {
    acc += w[i];
    // floor(acc * 2^64 / total) by long division (acc <= total < 2^124)
    const bool full = acc >= total;
    u128 r = acc;
    uint64_t q = 0;
    for (int b = 0; b < 64 && !full; ++b) {
      r <<= 1;
      q <<= 1;
      if (r >= total) {
        r -= total;
        q |= 1;
      }
    }
    cdt[i] = full ? ~0ull : q;
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

size_t align_words(size_t w) { return (w + 31) & ~(size_t)31; }  // 256-byte pieces

}  // namespace

extern "C" {

int yell_dev_sample_uniform(uint64_t* d_out, uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0,
                            uint64_t seed, void* stream) {
  SamplerArgs a;
  int st = prepare(d_out, count, L, log_n, cm0, stream, &a);
  if (st != kOk) return st;
  LaunchScope ps("sample_uniform", a.st);
  launch_dependent(k_sample_uniform, grid_for((((size_t)count * L) << log_n) >> 2), 256, 0, a.st, d_out, count, L,
                   log_n, cm0, a.mods, seed);
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
  launch_dependent(k_sample_zo, grid_for(((size_t)count << log_n) >> 1), 256, 0, a.st, d_out, count, L, log_n, cm0,
                   a.mods, seed, rho);
  g_kernel_launches += 1;
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? kOk : fail_cuda(e, "sample_zo");
}

// Four launches: reservoir slots initialised, every draw at once, ranks of
// the chosen positions (one CTA per poly), coefficients written.  Scratch
// (reservoir, bit sets, ranks) comes stream-ordered from the context's pool.
// YELL_GB300_HWT_SEQUENTIAL=1 redoes every poly's reservoir in draw order,
// the path a rejected draw takes (for tests).
int yell_dev_sample_hwt(uint64_t* d_out, uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0,
                        uint32_t h, uint64_t seed, void* stream) {
  if (log_n < kMinLogN || log_n > kMaxLogN) return check_degree(log_n);
  if (h == 0 || h > (1u << log_n)) return fail(kInvalidArgument, "hamming weight must be in [1, N]");
  SamplerArgs a;
  int st = prepare(d_out, count, L, log_n, cm0, stream, &a);
  if (st != kOk) return st;
  const uint32_t n = 1u << log_n, nw = n >= 32 ? n >> 5 : 1u;
  const size_t w_hit = align_words(((size_t)count * h + 1) / 2), w_ctl = align_words(count);
  const size_t w_bits = align_words(((size_t)count * nw + 1) / 2);
  uint64_t* scratch = nullptr;
  st = a.ctx->scratch_alloc_async(w_hit + w_ctl + 2 * w_bits, a.st, &scratch);
  if (st != kOk) return st;
  uint32_t* hitted = reinterpret_cast<uint32_t*>(scratch);
  HwtCtl* ctl = reinterpret_cast<HwtCtl*>(scratch + w_hit);
  uint32_t* bits = reinterpret_cast<uint32_t*>(scratch + w_hit + w_ctl);
  uint32_t* prefix = reinterpret_cast<uint32_t*>(scratch + w_hit + w_ctl + w_bits);
  const char* seq = std::getenv("YELL_GB300_HWT_SEQUENTIAL");
  const int sequential = seq && seq[0] == '1';
  const size_t smem = (size_t)(nw + 32) * sizeof(uint32_t);
  cudaError_t e = cudaSuccess;
  if (smem > 48 * 1024) e = cudaFuncSetAttribute(k_hwt_rank, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) {
    LaunchScope ps("sample_hwt", a.st);
    launch_dependent(k_hwt_init, grid_for((size_t)count * h), 256, 0, a.st, hitted, ctl, count, h, n);
    if (n > h) {
      // grid rows = polys (at most 65535 per launch); columns cover a poly's draws
      const uint32_t cols = (uint32_t)std::min<size_t>(((size_t)(n - h) + 255) / 256, 152u * 16u);
      for (uint32_t j0 = 0; j0 < count; j0 += 65535u) {
        const uint32_t rows = std::min(count - j0, 65535u);
        // rand_word(seed, j0 + j) = rand_word(seed + j0 * gamma, j)
        launch_dependent(k_hwt_reservoir, dim3(cols, rows), 256, 0, a.st, hitted + (size_t)j0 * h, ctl + j0, log_n, h,
                         seed + (uint64_t)j0 * 0x9E3779B97F4A7C15ull);
      }
    }
    launch_dependent(k_hwt_rank, count, kRankThreads, smem, a.st, hitted, ctl, bits, prefix, log_n, h, seed,
                     sequential);
    launch_dependent(k_hwt_write, grid_for(((size_t)count << log_n) >> 1), 256, 0, a.st, d_out, count, L, log_n, cm0,
                     a.mods, seed, h, static_cast<const HwtCtl*>(ctl), static_cast<const uint32_t*>(bits),
                     static_cast<const uint32_t*>(prefix));
    g_kernel_launches += 3 + (n > h ? (count + 65534u) / 65535u : 0u);
    e = cudaGetLastError();
  }
  const int fs = a.ctx->scratch_free_async(scratch, a.st);
  if (e != cudaSuccess) return fail_cuda(e, "sample_hwt");
  return fs;
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
  launch_dependent(k_sample_gaussian, grid_for(((size_t)count << log_n) >> 1), 256, 0, a.st, d_out, count, L, log_n,
                   cm0, a.mods, seed, cdt, len, (int32_t)tail, amplifier);
  g_kernel_launches += 1;
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? kOk : fail_cuda(e, "sample_gaussian");
}

// The cumulative table the Gaussian sampler uses for (sigma, tail): 2 * tail
// + 1 thresholds (host computation, no device needed).
int yell_gaussian_table(double sigma, uint32_t tail, uint64_t* out, uint32_t cap) {
  if (!out) return fail(kInvalidArgument, "null output");
  if (!(sigma > 0) || !(sigma < 1e6) || tail == 0 || tail > kMaxGaussianTail)
    return fail(kInvalidArgument, "need 0 < sigma < 1e6 and 0 < tail <= 1024");
  if (cap < 2 * tail + 1) return fail(kInvalidArgument, "output holds fewer than 2 * tail + 1 thresholds");
  const std::vector<uint64_t> cdt = gaussian_cdt(sigma, (int)tail);
  std::memcpy(out, cdt.data(), cdt.size() * sizeof(uint64_t));
  return kOk;
}

}  // extern "C"
