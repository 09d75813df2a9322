// Drop-in for yell/params.hpp (include/yell/params_64.hpp:6-40, and
// params_32.hpp:5-34 when built with -DYELL_USE_32BITS_MODULI, as in
// include/yell/params.hpp:2-6) over the yell_gb300 C ABI: the same names and
// meanings; the tables live in the library (regenerated from the rule the
// reference's headers state).
#pragma once
#include <cstddef>
#include <cstdint>
#include "yell_gb300.h"

namespace yell {

struct params {
  using uint128_t = unsigned __int128;
#ifdef YELL_USE_32BITS_MODULI
  using value_type = uint32_t;
  using signed_type = int32_t;
  using gt_value_type = uint64_t;
  using float_type = double;

  static constexpr unsigned int kMaxNbModuli = 291;
  static constexpr unsigned int kMaxPolyDegree = 32768;
  static constexpr unsigned int kModulusBitsize = 30;
  static constexpr unsigned int kModulusRepresentationBitsize = 32;

  struct prime_table {
    value_type operator[](size_t cm) const { return yell32_prime((uint32_t)cm); }
  };
  struct pn_table {
    value_type operator[](size_t cm) const { return yell32_prime_pn((uint32_t)cm); }
  };
  struct root_table {
    value_type operator[](size_t cm) const { return yell32_primitive_root((uint32_t)cm); }
  };
#else
  using value_type = uint64_t;
  using signed_type = int64_t;
  using gt_value_type = uint128_t;
  using float_type = double;

  static constexpr unsigned int kMaxNbModuli = 1000;
  static constexpr unsigned int kMaxPolyDegree = 1048576;
  static constexpr unsigned int kModulusBitsize = 62;
  static constexpr unsigned int kModulusRepresentationBitsize = 64;
  static constexpr unsigned int kMaxLazyReduction = 32;

  // params::P[cm], params::Pn[cm], params::primitive_roots[cm] keep their
  // subscript syntax; each reads the library's table.
  struct prime_table {
    value_type operator[](size_t cm) const { return yell_prime((uint32_t)cm); }
  };
  struct pn_table {
    value_type operator[](size_t cm) const { return yell_prime_pn((uint32_t)cm); }
  };
  struct root_table {
    value_type operator[](size_t cm) const { return yell_primitive_root((uint32_t)cm); }
  };
#endif
  static constexpr prime_table P{};
  static constexpr pn_table Pn{};
  static constexpr root_table primitive_roots{};
};

}  // namespace yell
