/*
 * CPU oracle for the seeded samplers (TEST INFRASTRUCTURE ONLY: the parity
 * tests load it as the checker; no product code calls it).
 *
 * Restates, coefficient by coefficient, the reference's rules for turning
 * random words into RNS coefficients (fionser/YELL
 * include/yell/details/poly.hpp:195-330), driven by the counter-based stream
 * the GPU samplers use instead of the reference's unseeded Salsa20:
 * random word k of stream s = splitmix64(s + (k + 1) * 0x9E3779B97F4A7C15).
 *   uniform  include/yell/details/poly.hpp:200-228  mask to the bit length of p, subtract p once
 *   ZO       include/yell/details/poly.hpp:267-280  byte r: r <= rho ? (r & 2 ? p - 1 : 1) : 0
 *   HWT      include/yell/details/poly.hpp:287-330  exactly h coefficients +-1 ((rnd & 2) ? 1 : p - 1),
 *                              positions = the indices a keyed Feistel permutation
 *                              maps below h (a pseudorandom h-subset)
 *   gaussian include/yell/details/poly.hpp:236-260  e * amplifier, e < 0 ? p + e : e, every limb
 * The gaussian integer e is the index of the first cumulative threshold above
 * one random word, thresholds floor(2^64 * CDF) of exp(-e^2 / 2 sigma^2)
 * on |e| <= tail (the stated distribution of lib/prng/FastGaussianNoise.cpp,
 * sampled by inversion instead of its lookup tables).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

uint64_t orc_prime(uint32_t cm);

#define SEED_POSITIONS 0x5ca1ab1e0ddba11ull
#define SEED_SIGNS 0x0b5e55edc0ffee5ull

static uint64_t word(uint64_t seed, uint64_t k) {
  uint64_t z = seed + (k + 1) * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static uint64_t bitlen_mask(uint64_t p) {
  int b = 0;
  while (b < 64 && (p >> b) > 1) ++b; /* b = floor(log2 p) */
  return b >= 63 ? ~0ull : ((2ull << b) - 1);
}

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

void orc_sample_zo(uint64_t* out, uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0, uint32_t rho,
                   uint64_t seed) {
  const uint64_t n = 1ull << log_n;
  for (uint64_t k = 0; k < (uint64_t)count * n; ++k) {
    const uint32_t r = (uint32_t)(word(seed, k) & 0xFF);
    const int64_t e = r <= rho ? ((r & 2) ? -1 : 1) : 0;
    put_all_limbs(out, k >> log_n, L, log_n, cm0, k & (n - 1), e);
  }
}

/* Keyed permutation of [0, 2^bits): 6 Feistel rounds over alternating index
 * fields of floor/ceil(bits / 2) bits, round function splitmix64 of the
 * round key plus the low field.  Coefficient i is nonzero when pi(i) < h. */
static uint64_t mix(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static uint32_t feistel(uint32_t x, uint32_t bits, uint64_t key) {
  uint32_t b = bits >> 1, a = bits - b;
  for (int r = 0; r < 6; ++r) {
    const uint32_t lo = x & ((1u << b) - 1u), hi = x >> b;
    const uint32_t f = (uint32_t)mix(word(key, (uint64_t)r) + lo);
    x = (lo << a) | ((hi ^ f) & ((1u << a) - 1u));
    const uint32_t t = a;
    a = b;
    b = t;
  }
  return x;
}

int orc_sample_hwt(uint64_t* out, uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0, uint32_t h,
                   uint64_t seed) {
  const uint64_t n = 1ull << log_n;
  if (h == 0 || h > n) return -1;
  for (uint64_t poly = 0; poly < count; ++poly) {
    const uint64_t key = word(seed ^ SEED_POSITIONS, poly);
    for (uint64_t i = 0; i < n; ++i) {
      const int take = feistel((uint32_t)i, log_n, key) < h;
      const int plus = (word(seed ^ SEED_SIGNS, (poly << log_n) + i) & 2) != 0;
      put_all_limbs(out, poly, L, log_n, cm0, i, take ? (plus ? 1 : -1) : 0);
    }
  }
  return 0;
}

/* 2 * tail + 1 thresholds into out; returns the count. */
uint32_t orc_gaussian_cdt(double sigma, uint32_t tail, uint64_t* out) {
  const int t = (int)tail;
  long double sum = 0;
  for (int e = -t; e <= t; ++e) sum += expl(-(long double)e * e / (2.0L * sigma * sigma));
  long double acc = 0;
  uint32_t m = 0;
  for (int e = -t; e <= t; ++e) {
    acc += expl(-(long double)e * e / (2.0L * sigma * sigma));
    const long double v = floorl(acc / sum * 18446744073709551616.0L);
    out[m++] = v >= 18446744073709551615.0L ? ~0ull : (uint64_t)v;
  }
  out[m - 1] = ~0ull;
  return m;
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
