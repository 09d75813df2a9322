// The reference's call pattern in its 32-bit moduli mode (-DYELL_USE_32BITS_MODULI):
// a.forward(); b.forward(); c = a * b; c.backward(), and the forward_lazy +
// add_product_of path of example.cpp, compiled unchanged against the
// yell_gb300 facade in 32-bit mode and checked against a schoolbook
// negacyclic product in uint64.  Prints "OK".
#include <cstdint>
#include <cstdio>
#include "yell/poly.hpp"

static_assert(sizeof(yell::params::value_type) == 4, "build with -DYELL_USE_32BITS_MODULI");

constexpr size_t Deg = 2048;
constexpr size_t NdM = 3;

static uint64_t splitmix64(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static void fill(yell::poly<Deg>& a, uint64_t seed) {
  for (size_t cm = 0; cm < a.moduli_count(); ++cm)
    for (size_t i = 0; i < Deg; ++i) a(cm, i) = (uint32_t)(splitmix64(seed) % yell::params::P[cm]);
}

static uint32_t schoolbook_coeff(const yell::poly<Deg>& a, const yell::poly<Deg>& b, size_t cm, size_t k) {
  const uint64_t p = yell::params::P[cm];
  uint64_t pos = 0, neg = 0;
  for (size_t i = 0; i <= k; ++i) pos = (pos + (uint64_t)a(cm, i) * b(cm, k - i)) % p;
  for (size_t i = k + 1; i < Deg; ++i) neg = (neg + (uint64_t)a(cm, i) * b(cm, Deg + k - i)) % p;
  return (uint32_t)((pos + p - neg) % p);
}

int main() {
  yell::ntt<Deg>::init_ntt_tables(NdM);
  yell::poly<Deg> a(NdM), b(NdM);
  fill(a, 21);
  fill(b, 22);
  const yell::poly<Deg> a0 = a, b0 = b;
  a.forward();
  b.forward();
  yell::poly<Deg> c = a * b;
  c.backward();
  for (size_t cm = 0; cm < NdM; ++cm)
    for (size_t k = 0; k < Deg; k += 89)
      if (c(cm, k) != schoolbook_coeff(a0, b0, cm, k)) {
        std::printf("MISMATCH cm=%zu k=%zu\n", cm, k);
        return 1;
      }
  yell::poly<Deg> e = b0, u = a0;
  u.forward();
  e.forward_lazy();
  e.add_product_of(u, a);
  e.backward();
  yell::poly<Deg> s2 = a * u;
  s2.backward();
  yell::poly<Deg> want = b0 + s2;
  if (e != want) {
    std::printf("MISMATCH add_product_of\n");
    return 1;
  }
  yell::poly<Deg> n = a0;
  n.negate();
  n += a0;
  for (size_t cm = 0; cm < NdM; ++cm)
    for (size_t i = 0; i < Deg; ++i)
      if (n(cm, i) != 0 && n(cm, i) != yell::params::P[cm]) {
        std::printf("MISMATCH negate\n");
        return 1;
      }
  std::printf("OK\n");
  return 0;
}
