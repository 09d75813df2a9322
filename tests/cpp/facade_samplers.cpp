// The reference's sampler and lifting calls (poly<N>(L, uniform{}),
// set(hwt_dist), set(ZO_dist), gmp::poly2mpz) compiled against the
// yell_gb300 facade and run on the GPU.  Checks ranges, Hamming weight, the
// same small integer in every limb, and that each lifted coefficient is
// congruent to its residues; then mul_sensitive_poly against the plain
// product, the stream format and recast_as_array.  Prints "OK".
#include <cstdio>
#include <cstdint>
#include <sstream>
#include <string>
#include "yell/gmp.hpp"
#include "yell/poly.hpp"

constexpr size_t Deg = 4096;
constexpr size_t NdM = 3;

static int fail(const char* what) {
  std::printf("FAIL %s\n", what);
  return 1;
}

// signed value of a residue known to be small
static long long centred(uint64_t v, uint64_t p) { return v > p / 2 ? (long long)v - (long long)p : (long long)v; }

int main() {
  using u128 = unsigned __int128;
  yell::set_sampler_seed(42);
  yell::poly<Deg> u(NdM, yell::uniform{});
  for (size_t cm = 0; cm < NdM; ++cm)
    for (size_t i = 0; i < Deg; ++i)
      if (u(cm, i) >= yell::params::P[cm]) return fail("uniform range");

  yell::poly<Deg> h(NdM);
  h.set(yell::hwt_dist(64));
  size_t weight = 0;
  for (size_t i = 0; i < Deg; ++i) {
    const long long e = centred(h(0, i), yell::params::P[0]);
    if (e != 0) ++weight;
    if (e < -1 || e > 1) return fail("hwt values");
    for (size_t cm = 1; cm < NdM; ++cm)
      if (centred(h(cm, i), yell::params::P[cm]) != e) return fail("hwt limbs");
  }
  if (weight != 64) return fail("hwt weight");

  yell::poly<Deg> z(NdM, yell::ZO_dist(0x7F));
  yell::poly<Deg> g(NdM, yell::gaussian_dist(3.2, 19));
  for (size_t i = 0; i < Deg; ++i)
    for (size_t cm = 0; cm < NdM; ++cm) {
      const long long ez = centred(z(cm, i), yell::params::P[cm]);
      const long long eg = centred(g(cm, i), yell::params::P[cm]);
      if (ez < -1 || ez > 1 || eg < -19 || eg > 19) return fail("zo / gaussian range");
      if (ez != centred(z(0, i), yell::params::P[0]) || eg != centred(g(0, i), yell::params::P[0]))
        return fail("zo / gaussian limbs");
    }

  // gmp::poly2mpz: the lifted u is congruent to its residues
  const uint32_t W = yell::gmp::words(NdM);
  const std::vector<uint64_t> x = yell::gmp::poly2words(u);
  for (size_t i = 0; i < Deg; i += 37)
    for (size_t cm = 0; cm < NdM; ++cm) {
      const uint64_t p = yell::params::P[cm];
      u128 r = 0;
      for (size_t w = W; w-- > 0;) r = ((r << 64) | x[i * W + w]) % p;
      if ((uint64_t)r != u(cm, i)) return fail("lift congruence");
    }
  // small signed integers lift to themselves modulo Q: g's lift is e or Q + e
  const std::vector<uint64_t> xg = yell::gmp::poly2words(g);
  for (size_t i = 0; i < Deg; ++i) {
    const long long e = centred(g(0, i), yell::params::P[0]);
    if (e >= 0) {
      if (xg[i * W] != (uint64_t)e) return fail("lift of a small integer");
      for (size_t w = 1; w < W; ++w)
        if (xg[i * W + w] != 0) return fail("lift of a small integer (high words)");
    }
  }
  // details/poly.hpp:135-149: a * s through a random split equals a * s
  {
    yell::poly<Deg> a(NdM, yell::uniform{}), s(NdM, yell::uniform{});
    yell::poly<Deg> want = a * s;
    a.mul_sensitive_poly(s);
    if (a != want) return fail("mul_sensitive_poly");
    a.check_vaild_range();
  }
  // include/yell/details/poly.hpp:336-354 stream format; include/yell/poly.hpp:150-161 recast_as_array
  {
    yell::poly<8> t(2);
    for (size_t cm = 0; cm < 2; ++cm)
      for (size_t i = 0; i < 8; ++i) t(cm, i) = 10 * cm + i;
    std::ostringstream os;
    os << t;
    if (os.str() != "{{0ULL, 1ULL, 2ULL, 3ULL, 4ULL, 5ULL, 6ULL, 7ULL}\n"
                    "{10ULL, 11ULL, 12ULL, 13ULL, 14ULL, 15ULL, 16ULL, 17ULL}}")
      return fail("stream format");
    auto arr = yell::recast_as_array(t, 1);
    if ((*arr)[3] != 13 || arr->size() != 8) return fail("recast_as_array");
  }
  std::printf("OK\n");
  return 0;
}
