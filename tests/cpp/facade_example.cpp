// The reference's call pattern (example.cpp / a.forward(); b.forward();
// c = a * b; c.backward()) compiled unchanged against the yell_gb300 facade.
// Checks the product against a schoolbook negacyclic product in __int128 and
// the add_product_of / forward_lazy path of example.cpp:36-57.  Prints "OK".
#include <cstdio>
#include <cstdint>
#include <vector>
#include "yell/poly.hpp"

constexpr size_t Deg = 1024;
constexpr size_t NdM = 3;

static uint64_t splitmix64(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static void fill(yell::poly<Deg>& a, uint64_t seed) {
  for (size_t cm = 0; cm < a.moduli_count(); ++cm)
    for (size_t i = 0; i < Deg; ++i) a(cm, i) = splitmix64(seed) % yell::params::P[cm];
}

static uint64_t schoolbook_coeff(const yell::poly<Deg>& a, const yell::poly<Deg>& b, size_t cm, size_t k) {
  using u128 = unsigned __int128;
  const uint64_t p = yell::params::P[cm];
  u128 pos = 0, neg = 0;
  for (size_t i = 0; i <= k; ++i) pos += ((u128)a(cm, i) * b(cm, k - i)) % p;
  for (size_t i = k + 1; i < Deg; ++i) neg += ((u128)a(cm, i) * b(cm, Deg + k - i)) % p;
  const uint64_t s = (uint64_t)(pos % p), d = (uint64_t)(neg % p);
  return s >= d ? s - d : s + (p - d);
}

int main() {
  yell::ntt<Deg>::init_ntt_tables(NdM);
  yell::poly<Deg> a(NdM), b(NdM);
  fill(a, 11);
  fill(b, 12);
  const yell::poly<Deg> a0 = a, b0 = b;
  a.forward();
  b.forward();
  yell::poly<Deg> c = a * b;
  c.backward();
  for (size_t cm = 0; cm < NdM; ++cm)
    for (size_t k = 0; k < Deg; k += 97)
      if (c(cm, k) != schoolbook_coeff(a0, b0, cm, k)) {
        std::printf("MISMATCH cm=%zu k=%zu\n", cm, k);
        return 1;
      }
  // example.cpp pattern: e.forward_lazy(); e.add_product_of(u, s); e.backward()
  yell::poly<Deg> e = b0, u = a0;
  u.forward();
  e.forward_lazy();
  e.add_product_of(u, a);  // a holds forward(a0)
  e.backward();
  yell::ops::mulmod mm;
  yell::poly<Deg> s2 = a * u;  // forward(a0) * forward(a0)
  s2.backward();
  yell::poly<Deg> want = b0 + s2;
  if (e != want) {
    std::printf("MISMATCH add_product_of path\n");
    return 1;
  }
  if (mm(3, 5, 0) != 15) return 1;
  // the largest degree of the reference (params::kMaxPolyDegree = 2^20): round trip
  constexpr size_t Big = yell::params::kMaxPolyDegree;
  yell::ntt<Big>::init_table(5);
  std::vector<uint64_t> x(Big), x0;
  uint64_t seed = 13;
  for (auto& v : x) v = splitmix64(seed) % yell::params::P[5];
  x0 = x;
  yell::ntt<Big>::forward(x.data(), 5);
  yell::ntt<Big>::backward(x.data(), 5);
  if (x != x0) {
    std::printf("MISMATCH round trip at N = 2^20\n");
    return 1;
  }
  std::printf("OK\n");
  return 0;
}
