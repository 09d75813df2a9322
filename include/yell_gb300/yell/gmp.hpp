// Drop-in for yell/gmp.hpp (include/yell/gmp.hpp:42-70, lib/gmp.cpp:6-51):
// gmp::poly2mpz lifts every coefficient of a poly over moduli 0 .. L-1 to
// the unique integer in [0, prod q_j), computed on the GPU
// (yell_poly_to_bigint).  poly2words returns the integers as little-endian
// 64-bit words, words() per coefficient; poly2mpz (when <gmp.h> is present)
// imports them into mpz_t like the reference returns them.
#pragma once
#include <array>
#include <cstdint>
#include <vector>
#include "yell/poly.hpp"
#if defined(__has_include)
#if __has_include(<gmp.h>)
#include <gmp.h>
#define YELL_GB300_HAVE_GMP 1
#endif
#endif

namespace yell {

struct gmp {
  // 64-bit words per lifted coefficient for L moduli.
  static uint32_t words(size_t nmoduli) {
    uint32_t w = 0;
    check_status(yell_crt_words((uint32_t)nmoduli, 0, &w), "crt_words");
    return w;
  }

  template <size_t degree_>
  static std::vector<uint64_t> poly2words(poly<degree_> const& op) {
    const uint32_t W = words(op.moduli_count());
    std::vector<uint64_t> out((size_t)degree_ * W);
    check_status(yell_poly_to_bigint(out.data(), op.raw_data(), (uint32_t)op.moduli_count(), poly<degree_>::logn),
                 "poly2mpz");
    return out;
  }

#ifdef YELL_GB300_HAVE_GMP
  template <size_t degree_>
  static std::array<mpz_t, degree_> poly2mpz(poly<degree_> const& op) {
    const uint32_t W = words(op.moduli_count());
    const std::vector<uint64_t> w = poly2words(op);
    std::array<mpz_t, degree_> rop;
    for (size_t i = 0; i < degree_; ++i) {
      mpz_init2(rop[i], 64 * W);
      mpz_import(rop[i], W, -1, sizeof(uint64_t), 0, 0, w.data() + i * W);
    }
    return rop;
  }
#endif
};

}  // namespace yell
