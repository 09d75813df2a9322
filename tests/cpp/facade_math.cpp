// yell/utils/math.hpp of the facade against values the reference's helpers
// give (lib/math.cpp, include/yell/utils/math.hpp).  Host only.  Prints "OK".
#include <cstdio>
#include <cstdint>
#include <vector>
#include "yell/utils/math.hpp"

static int fail(const char* what) {
  std::printf("FAIL %s\n", what);
  return 1;
}

int main() {
  using yell::math::reverse_bits;
  if (reverse_bits(1u) != 0x80000000u || reverse_bits(0xF0000000u) != 0xFu) return fail("reverse_bits");
  if (reverse_bits(1u, 3) != 4u || reverse_bits(6u, 3) != 3u || reverse_bits(5u, 0) != 0u) return fail("reverse_bits n");
  std::vector<int> a(16);
  for (int i = 0; i < 16; ++i) a[i] = i;
  yell::math::revbin_permute(a.data(), 16);
  for (int i = 0; i < 16; ++i)
    if (a[i] != (int)reverse_bits((uint32_t)i, 4)) return fail("revbin_permute");
  int two[2] = {7, 9};
  yell::math::revbin_permute(two, 2);
  if (two[0] != 7 || two[1] != 9) return fail("revbin_permute length 2");
  for (size_t cm : {0u, 5u, 999u}) {
    const uint64_t p = yell::params::P[cm];
    for (uint64_t x : {uint64_t(2), uint64_t(12345), p - 1}) {
      const uint64_t inv = yell::math::inv_mod_prime(x, cm);
      if ((uint64_t)(((unsigned __int128)inv * x) % p) != 1) return fail("inv_mod_prime");
    }
  }
  if (yell::math::round<int>(2.5) != 3 || yell::math::round<int>(-2.5) != -3) return fail("round");
  std::printf("OK\n");
  return 0;
}
