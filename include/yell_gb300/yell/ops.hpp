// Drop-in for yell/ops.hpp (include/yell/ops.hpp:43-158): the scalar modular
// functors with the reference's formulas, for single coefficients on the
// host.  Whole-polynomial arithmetic (poly<N>'s operators) runs on the GPU
// through the C ABI; these functors are the per-coefficient helpers only.
#pragma once
#include <cstddef>
#include <cstdint>
#include "yell/params.hpp"

namespace yell {
namespace ops {

// include/yell/ops.hpp:46-52
template <typename T>
static inline void mod_correct(T& a, const T p) {
  a -= (a >= p) ? p : T(0);
}

constexpr unsigned kWordBits = params::kModulusRepresentationBitsize;
constexpr unsigned kDelta = params::kModulusRepresentationBitsize - params::kModulusBitsize;

// lib/ops.cpp:5-21
inline void barret_reduction(params::gt_value_type* x, size_t cm) {
  if (!x) return;
  using T = params::value_type;
  using gT = params::gt_value_type;
  const gT xv = *x;
  const gT q = (gT)params::Pn[cm] * (T)(xv >> kWordBits) + (xv << kDelta);
  const T p = params::P[cm];
  T r = (T)xv - (T)(q >> kWordBits) * p;
  mod_correct(r, p);
  *x = r;
}

// lib/ops.cpp:23-27
inline params::value_type shoupify(params::value_type x, size_t cm) {
  return (params::value_type)(((params::gt_value_type)x << kWordBits) / params::P[cm]);
}

struct addmod {
  using T = params::value_type;
  T operator()(T x, T y, size_t cm) const { compute(x, y, cm); return x; }
  void compute(T& x, T y, size_t cm) const { x += y; mod_correct(x, params::P[cm]); }
};

struct submod {
  using T = params::value_type;
  T operator()(T x, T y, size_t cm) const { compute(x, y, cm); return x; }
  void compute(T& x, T y, size_t cm) const {
    const T p = params::P[cm];
    x += (p - y);
    mod_correct(x, p);
  }
};

struct mulmod {
  using T = params::value_type;
  T operator()(T x, T y, size_t cm) const { compute(x, y, cm); return x; }
  void compute(T& x, T y, size_t cm) const {
    params::gt_value_type r = (params::gt_value_type)x * y;
    barret_reduction(&r, cm);
    x = (T)r;
  }
};

struct mulmod_shoup {
  using T = params::value_type;
  T operator()(T x, T y, T yprime, size_t cm) const { compute(x, y, yprime, cm); return x; }
  void compute(T& x, T y, T yprime, size_t cm) const {
    const T p = params::P[cm];
    const T q = (T)(((params::gt_value_type)x * yprime) >> kWordBits) * p;
    x = x * y - q;
    mod_correct(x, p);
  }
};

struct muladd {
  using T = params::value_type;
  T operator()(T rop, T x, T y, size_t cm) const { compute(rop, x, y, cm); return rop; }
  void compute(T& rop, T x, T y, size_t cm) const {
    params::gt_value_type r = (params::gt_value_type)x * y;
    r += rop;
    barret_reduction(&r, cm);
    rop = (T)r;
  }
};

}  // namespace ops
}  // namespace yell
