// Drop-in for yell/utils/math.hpp (include/yell/utils/math.hpp:6-47 and
// lib/math.cpp:5-27): the host helpers the reference uses to build tables.
// Header-only; same results, written as plain loops.
#pragma once
#include <cstddef>
#include <cstdint>
#include <utility>
#include "yell/ops.hpp"
#include "yell/params.hpp"

namespace yell {
namespace math {

// a^(P[cm] - 2) mod P[cm], square-and-multiply with ops::mulmod (math.hpp:8-21).
template <typename T>
T inv_mod_prime(T a, size_t cm) {
  ops::mulmod mul;
  T r{1};
  for (T e = params::P[cm] - 2; e != 0; e >>= 1u) {
    if (e & 1u) r = mul(r, a, cm);
    a = mul(a, a, cm);
  }
  return r;
}

// Rounds half away from zero through a float offset, as math.hpp:23-27.
template <typename T, typename F>
inline T round(F a) {
  return a >= 0 ? (T)(a + 0.5f) : (T)(a - 0.5f);
}

// All 32 bits of v in reverse order (lib/math.cpp:5-19).
inline uint32_t reverse_bits(uint32_t v) {
  uint32_t r = 0;
  for (int i = 0; i < 32; ++i, v >>= 1) r = (r << 1) | (v & 1u);
  return r;
}

// The low bit_count bits of operand reversed, bit_count < 32 (lib/math.cpp:23-27;
// bit_count 0 gives 0).
inline uint32_t reverse_bits(uint32_t operand, int32_t bit_count) {
  return (uint32_t)((uint64_t)reverse_bits(operand) >> (32 - bit_count));
}

// In-place bit-reversal permutation of a power-of-two-length array
// (math.hpp:29-41); lengths <= 2 and null arrays are left alone.
template <typename T>
void revbin_permute(T* array, int length) {
  if (!array || length <= 2) return;
  int bits = 0;
  while ((1 << bits) < length) ++bits;
  for (int i = 1; i < length; ++i) {
    const int j = (int)reverse_bits((uint32_t)i, bits);
    if (i < j) std::swap(array[i], array[j]);
  }
}

}  // namespace math
}  // namespace yell
