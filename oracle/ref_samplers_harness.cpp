// Harness around the reference's own samplers and CRT lifting (fionser/YELL).
//
// TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles this file with the
// reference's unmodified yell/poly.hpp (the samplers, details/poly.hpp:195-330),
// yell/gmp.hpp + lib/gmp.cpp (CRT lifting) and
// yell/prng/FastGaussianNoise.hpp, where they lie in the reference checkout,
// into oracle/_ref/libyellref_samplers.so.  <gmp.h> and <mpfr.h> come from the
// declarations-only stand-ins in oracle/shim/ and the calls go to the
// installed libgmp.so.10 / libmpfr.so.6.  It is built only where the
// reference checkout and those two runtimes exist; tests/golden/
// make_golden_samplers.py stores its outputs as fixtures.
//
// Randomness.  Every random byte the reference draws comes from
// yell::fastrandombytes (include/yell/prng/fastrandombytes.h:9), which in the
// reference is an unseeded Salsa20 stream (lib/prng/fastrandombytes.cpp).
// This harness defines it instead as the counter stream the library's device
// samplers use: random word k of the stream with seed s is
// splitmix64(s + (k + 1) * 0x9E3779B97F4A7C15), and the bytes are those words
// in little-endian order, consumed in sequence across calls.  So the
// reference's own set(uniform), set(ZO_dist), set(hwt_dist) and its Gaussian
// sampler run here on exactly the randomness the device samplers read.
#include <algorithm>
#include <array>
#include <atomic>
#include <cassert>
#include <climits>
#include <cmath>
#include <condition_variable>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <iosfwd>
#include <iostream>
#include <iterator>
#include <list>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <string>
#include <thread>
#include <tuple>
#include <type_traits>
#include <typeinfo>
#include <unordered_map>
#include <vector>

// The Gaussian sampler keeps its barrier table private; the harness reads it
// to compare the reference's distribution with the library's.
#define private public
#include "yell/prng/FastGaussianNoise.hpp"
#undef private
#include "yell/gmp.hpp"
#include "yell/poly.hpp"

namespace {

uint64_t g_seed = 0;
uint64_t g_byte = 0;  // bytes of the stream consumed so far

uint64_t stream_word(uint64_t seed, uint64_t k) {
  uint64_t z = seed + (k + 1) * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

void reseed(uint64_t seed) {
  g_seed = seed;
  g_byte = 0;
}

}  // namespace

namespace yell {
void fastrandombytes(unsigned char* r, unsigned long long rlen) {
  for (unsigned long long i = 0; i < rlen; ++i, ++g_byte)
    r[i] = (unsigned char)(stream_word(g_seed, g_byte >> 3) >> (8 * (g_byte & 7)));
}
}  // namespace yell

namespace {

template <size_t N>
void copy_out(const yell::poly<N>& p, uint64_t* out) {
  for (size_t cm = 0; cm < p.moduli_count(); ++cm) std::memcpy(out + cm * N, p.cptr_at(cm), N * 8);
}

// count polys of L limbs, filled in sequence from one stream.
template <size_t N>
void uniform_polys(uint64_t* out, uint32_t count, uint32_t L) {
  for (uint32_t j = 0; j < count; ++j) {
    yell::poly<N> p(L, yell::uniform{});
    copy_out(p, out + (size_t)j * L * N);
  }
}

template <size_t N>
void zo_polys(uint64_t* out, uint32_t count, uint32_t L, uint8_t rho) {
  for (uint32_t j = 0; j < count; ++j) {
    yell::poly<N> p(L, yell::ZO_dist(rho));
    copy_out(p, out + (size_t)j * L * N);
  }
}

// Poly j of an HWT batch draws from its own stream, seeded with word j of
// the batch seed's stream.
template <size_t N>
void hwt_polys(uint64_t* out, uint32_t count, uint32_t L, uint32_t h, uint64_t seed) {
  for (uint32_t j = 0; j < count; ++j) {
    reseed(stream_word(seed, j));
    yell::poly<N> p(L, yell::hwt_dist(h));
    copy_out(p, out + (size_t)j * L * N);
  }
}

// gmp::poly2mpz of one poly, each integer written as W little-endian words.
template <size_t N>
int lift(uint64_t* out, const uint64_t* limbs, uint32_t L, uint32_t W) {
  yell::poly<N> p(L);
  for (uint32_t cm = 0; cm < L; ++cm) std::memcpy(p.ptr_at(cm), limbs + (size_t)cm * N, N * 8);
  auto z = yell::gmp::poly2mpz(p);
  int rc = 0;
  for (size_t i = 0; i < N; ++i) {
    uint64_t* o = out + i * W;
    std::memset(o, 0, W * 8);
    if (mpz_sizeinbase(z[i], 2) > (size_t)W * 64) rc = -2;
    else mpz_export(o, nullptr, -1, 8, 0, 0, z[i]);
    mpz_clear(z[i]);
  }
  return rc;
}

#define YELL_SAMPLER_SWITCH(LOGN, CALL) \
  switch (LOGN) {                       \
    case 3: CALL(8); break;             \
    case 4: CALL(16); break;            \
    case 5: CALL(32); break;            \
    case 6: CALL(64); break;            \
    case 7: CALL(128); break;           \
    case 8: CALL(256); break;           \
    case 9: CALL(512); break;           \
    case 10: CALL(1024); break;         \
    case 11: CALL(2048); break;         \
    case 12: CALL(4096); break;         \
    case 13: CALL(8192); break;         \
    case 14: CALL(16384); break;        \
    case 15: CALL(32768); break;        \
    case 16: CALL(65536); break;        \
    default: return -1;                 \
  }

using Gauss = yell::FastGaussianNoise<uint16_t, uint64_t, 2>;

}  // namespace

extern "C" {

int refs_sample_uniform(uint64_t* out, uint32_t count, uint32_t L, uint32_t log_n, uint64_t seed) {
  reseed(seed);
#define CALL(n) uniform_polys<n>(out, count, L)
  YELL_SAMPLER_SWITCH(log_n, CALL)
#undef CALL
  return 0;
}

int refs_sample_zo(uint64_t* out, uint32_t count, uint32_t L, uint32_t log_n, uint32_t rho, uint64_t seed) {
  reseed(seed);
#define CALL(n) zo_polys<n>(out, count, L, (uint8_t)rho)
  YELL_SAMPLER_SWITCH(log_n, CALL)
#undef CALL
  return 0;
}

int refs_sample_hwt(uint64_t* out, uint32_t count, uint32_t L, uint32_t log_n, uint32_t h, uint64_t seed) {
  if (h == 0 || h > (1u << log_n)) return -1;
#define CALL(n) hwt_polys<n>(out, count, L, h, seed)
  YELL_SAMPLER_SWITCH(log_n, CALL)
#undef CALL
  return 0;
}

int refs_poly2mpz(uint64_t* out, const uint64_t* limbs, uint32_t L, uint32_t log_n, uint32_t W) {
  int rc = 0;
#define CALL(n) rc = lift<n>(out, limbs, L, W)
  YELL_SAMPLER_SWITCH(log_n, CALL)
#undef CALL
  return rc;
}

// The reference's Gaussian sampler FastGaussianNoise<uint16_t, uint64_t, 2>
// (the instantiation of example.cpp:7-9) for (sigma, security, samples):
// info = {number of barriers, bit precision, words of precision};
// top64[i] = the 64 most significant bits of barrier i (the cumulative
// probability of the i-th value times 2^bit_precision - 1).
int refs_gaussian_barriers(double sigma, uint32_t security, uint32_t samples, uint32_t* info, uint64_t* top64,
                           uint32_t cap) {
  Gauss g(sigma, security, samples);
  info[0] = g._number_of_barriers;
  info[1] = g._bit_precision;
  info[2] = g._word_precision;
  if (g._number_of_barriers > cap || g._word_precision < 4) return -1;
  for (unsigned i = 0; i < g._number_of_barriers; ++i) {
    uint64_t v = 0;
    for (int w = 0; w < 4; ++w) v = (v << 16) | g.barriers[i][w];
    top64[i] = v;
  }
  return 0;
}

// n draws of the same sampler on the counter stream with this seed.
int refs_gaussian_sample(double sigma, uint32_t security, uint32_t samples, uint64_t seed, int64_t* out,
                         uint64_t n) {
  Gauss g(sigma, security, samples);
  reseed(seed);
  g.getNoise(reinterpret_cast<uint64_t*>(out), n);
  return 0;
}

}  // extern "C"
