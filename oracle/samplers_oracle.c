/*
 * CPU oracle for the seeded samplers (TEST INFRASTRUCTURE ONLY: the parity
 * tests load it as the checker; no product code calls it).
 *
 * Restates, coefficient by coefficient, what the reference's samplers
 * (fionser/YELL include/yell/details/poly.hpp:195-330) make of a random byte
 * stream, driven by the counter stream the GPU samplers use instead of the
 * reference's unseeded Salsa20: random word k of stream s =
 * splitmix64(s + (k + 1) * 0x9E3779B97F4A7C15), bytes in little-endian order.
 *   uniform  include/yell/details/poly.hpp:200-228  one word per coefficient, limb after
 *            limb, poly after poly; mask to the bit length of p, subtract p once
 *   ZO       include/yell/details/poly.hpp:267-280  one byte per coefficient, poly after
 *            poly: r <= rho ? (r & 2 ? p - 1 : 1) : 0 in every limb
 *   HWT      include/yell/details/poly.hpp:287-330  poly j on the stream seeded with word
 *            j of the batch stream: reservoir sampling with rejection, the
 *            sorted positions signed by the h words after the draws
 *   gaussian include/yell/details/poly.hpp:236-260  e * amplifier, e < 0 ? p + e : e, every
 *            limb; e by inversion of one word against the device sampler's
 *            cumulative table (the distribution of
 *            include/yell/prng/FastGaussianNoise.hpp, not its lookup-table
 *            draw sequence)
 * These rules are pinned to the reference's own set(...) run on the same
 * stream (tests/golden/yell_ref_samplers.npz, oracle/ref_samplers_harness.cpp).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

uint64_t orc_prime(uint32_t cm);

static uint64_t word(uint64_t seed, uint64_t k) {
  uint64_t z = seed + (k + 1) * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

/* details/poly.hpp:213: mask = 2^(floor(log2 p) + 1) - 1 */
static uint64_t bitlen_mask(uint64_t p) {
  int b = 0;
  while (b < 64 && (p >> b) > 1) ++b; /* b = floor(log2 p) */
  return b >= 63 ? ~0ull : ((2ull << b) - 1);
}

/* details/poly.hpp:200-228 */
void orc_sample_uniform(uint64_t* out, uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0, uint64_t seed) {
  const uint64_t n = 1ull << log_n;
  for (uint64_t row = 0; row < (uint64_t)count * L; ++row) {
    const uint64_t p = orc_prime(cm0 + (uint32_t)(row % L)), mask = bitlen_mask(p);
    for (uint64_t k = row * n; k < (row + 1) * n; ++k) {
      const uint64_t v = word(seed, k) & mask;
      out[k] = v >= p ? v - p : v;
    }
  }
}

static void put_all_limbs(uint64_t* out, uint64_t poly, uint32_t L, uint32_t log_n, uint32_t cm0, uint64_t i,
                          int64_t e) {
  for (uint32_t l = 0; l < L; ++l) {
    const uint64_t p = orc_prime(cm0 + l);
    out[((poly * L + l) << log_n) + i] = e < 0 ? p - (uint64_t)(-e) : (uint64_t)e;
  }
}

/* details/poly.hpp:267-280: byte k of the stream for coefficient k */
void orc_sample_zo(uint64_t* out, uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0, uint32_t rho,
                   uint64_t seed) {
  const uint64_t n = 1ull << log_n;
  for (uint64_t k = 0; k < (uint64_t)count * n; ++k) {
    const uint32_t r = (uint32_t)(word(seed, k >> 3) >> (8 * (k & 7))) & 0xFF;
    const int64_t e = r <= rho ? ((r & 2) ? -1 : 1) : 0;
    put_all_limbs(out, k >> log_n, L, log_n, cm0, k & (n - 1), e);
  }
}

static int cmp_u32(const void* a, const void* b) {
  const uint32_t x = *(const uint32_t*)a, y = *(const uint32_t*)b;
  return x < y ? -1 : x > y;
}

/* details/poly.hpp:287-330.  The reference's buffer of h words is refilled
 * whenever it runs dry (:302-306), so the draws read words 0, 1, 2, ... of the
 * stream and the sign buffer (:319) starts at ceil(draws / h) * h. */
int orc_sample_hwt(uint64_t* out, uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0, uint32_t h,
                   uint64_t seed) {
  const uint64_t n = 1ull << log_n;
  if (h == 0 || h > n) return -1;
  uint32_t* hitted = (uint32_t*)malloc(sizeof(uint32_t) * h);
  if (!hitted) return -2;
  for (uint64_t poly = 0; poly < count; ++poly) {
    const uint64_t s = word(seed, poly);
    for (uint32_t t = 0; t < h; ++t) hitted[t] = t; /* :290-291 */
    uint64_t d = 0;
    for (uint64_t k = h; k < n; ++k) { /* :296-315 */
      const uint64_t limit = (~0ull / k) * k;
      uint64_t pos;
      for (;;) {
        pos = word(s, d++);
        if (pos <= limit) {
          pos %= k;
          break;
        }
      }
      if (pos < h) hitted[pos] = (uint32_t)k;
    }
    qsort(hitted, h, sizeof(uint32_t), cmp_u32); /* :317 */
    const uint64_t signs = (d + h - 1) / h * h;
    for (uint64_t i = 0; i < n; ++i) put_all_limbs(out, poly, L, log_n, cm0, i, 0); /* :318 clear() */
    for (uint32_t t = 0; t < h; ++t) /* :320-327 */
      put_all_limbs(out, poly, L, log_n, cm0, hitted[t], (word(s, signs + t) & 2) ? 1 : -1);
  }
  free(hitted);
  return 0;
}

/* ---- the Gaussian sampler's cumulative table ------------------------------
 * t_e = floor(2^64 * S(e) / S(tail)), S(e) = sum of exp(-j^2 c) over
 * -tail <= j <= e, c = 1 / (2 sigma^2); last threshold 2^64 - 1.  The same
 * 128-bit fixed-point evaluation as the device sampler's host code (integer
 * operations only, identical on every host); its distance to the reference's
 * MPFR-built FastGaussianNoise barriers is checked separately. */
typedef unsigned __int128 u128;
#define FIX 120

static u128 mul_shr(u128 a, u128 b, int s) {
  const uint64_t a0 = (uint64_t)a, a1 = (uint64_t)(a >> 64), b0 = (uint64_t)b, b1 = (uint64_t)(b >> 64);
  const u128 p00 = (u128)a0 * b0, p01 = (u128)a0 * b1, p10 = (u128)a1 * b0, p11 = (u128)a1 * b1;
  const u128 mid = (p00 >> 64) + (uint64_t)p01 + (uint64_t)p10;
  const u128 lo = (mid << 64) | (uint64_t)p00;
  const u128 hi = p11 + (p01 >> 64) + (p10 >> 64) + (mid >> 64);
  return s == 128 ? hi : (hi << (128 - s)) | (lo >> s);
}

static u128 exp_neg_fixed(u128 x) {
  u128 ln2 = 0;
  for (int k = 1; k <= FIX; ++k) ln2 += (((u128)1 << FIX) >> k) / (u128)k;
  const u128 n = x / ln2;
  if (n >= (u128)FIX) return 0;
  const u128 r = x - n * ln2;
  u128 term = (u128)1 << FIX, pos = term, neg = 0;
  for (int k = 1; k < 64 && term != 0; ++k) {
    term = mul_shr(term, r, FIX) / (u128)k;
    if (k & 1) neg += term;
    else pos += term;
  }
  return (pos - neg) >> (int)n;
}

/* floor(2^FIX / (2 sigma^2)) exactly, sigma = m 2^(e - 53). */
static u128 inv_two_sigma_sq_fixed(double sigma) {
  int e = 0;
  const double f = frexp(sigma, &e);
  const u128 m = (u128)(uint64_t)ldexp(f, 53);
  const u128 M = m * m;
  const int P = FIX - 1 - 2 * (e - 53);
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

/* 2 * tail + 1 thresholds into out; returns the count. */
uint32_t orc_gaussian_cdt(double sigma, uint32_t tail, uint64_t* out) {
  const int t = (int)tail;
  const double c = 1.0 / (2.0 * sigma * sigma);
  const u128 cf = c < 100.0 ? inv_two_sigma_sq_fixed(sigma) : 0;
  u128* w = (u128*)malloc(sizeof(u128) * (2 * (size_t)t + 1));
  u128 total = 0;
  for (int j = -t; j <= t; ++j) {
    u128 v = 0;
    const double x = (double)j * j * c;
    if (j == 0) v = (u128)1 << FIX;
    else if (x < 100.0) v = exp_neg_fixed(cf * (u128)((uint64_t)j * (uint64_t)j));
    w[j + t] = v >> 8;
    total += w[j + t];
  }
  u128 acc = 0;
  const uint32_t len = 2 * tail + 1;
  for (uint32_t i = 0; i < len; ++i) {
    acc += w[i];
    if (acc >= total) {
      out[i] = ~0ull;
      continue;
    }
    u128 r = acc;
    uint64_t q = 0;
    for (int b = 0; b < 64; ++b) {
      r <<= 1;
      q <<= 1;
      if (r >= total) {
        r -= total;
        q |= 1;
      }
    }
    out[i] = q;
  }
  out[len - 1] = ~0ull;
  free(w);
  return len;
}

void orc_sample_gaussian(uint64_t* out, uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0,
                         const uint64_t* cdt, uint32_t len, uint32_t tail, uint64_t amplifier, uint64_t seed) {
  const uint64_t n = 1ull << log_n;
  for (uint64_t k = 0; k < (uint64_t)count * n; ++k) {
    const uint64_t r = word(seed, k);
    uint32_t idx = 0;
    while (idx + 1 < len && r >= cdt[idx]) ++idx;
    const int64_t e = ((int64_t)idx - (int64_t)tail) * (int64_t)amplifier;
    put_all_limbs(out, k >> log_n, L, log_n, cm0, k & (n - 1), e);
  }
}
