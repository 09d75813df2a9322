// Drop-in for yell/poly.hpp (include/yell/poly.hpp:43-171 and
// include/yell/details/poly.hpp): yell::poly<N> keeps one host allocation per
// limb (raw_data() is the same uint64_t** the reference exposes) and every
// NTT, arithmetic and sampling member runs on the GPU through the yell_gb300
// C ABI.  The samplers take the reference's tag types (uniform, hwt_dist,
// ZO_dist); the reference's gaussian<> wraps an MPFR-built FastGaussianNoise,
// so the facade names the distribution instead (gaussian_dist).
#pragma once
#include <array>
#include <atomic>
#include <cassert>
#include <cstdlib>
#include <random>
#include <cstring>
#include <ostream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>
#include "yell/ntt.hpp"
#include "yell/ops.hpp"
#include "yell/params.hpp"

namespace yell {

// include/yell/poly.hpp:20-41
struct uniform {};
struct hwt_dist {
  uint32_t hwt;
  explicit hwt_dist(uint32_t hwt_) : hwt(hwt_) {}
};
struct ZO_dist {
  uint8_t rho;  // P(1) = P(-1) ~ (rho / 0xFF) / 2
  explicit ZO_dist(uint8_t rho_ = 0x7F) : rho(rho_) {}
};
// Discrete Gaussian exp(-e^2 / 2 sigma^2) on |e| <= tail, times amplifier.
struct gaussian_dist {
  double sigma;
  uint32_t tail;
  uint64_t amplifier;
  explicit gaussian_dist(double sigma_ = 3.2, uint32_t tail_ = 19, uint64_t amp = 1)
      : sigma(sigma_), tail(tail_), amplifier(amp) {}
};

namespace detail {
// The reference's samplers draw from an unseeded stream; here each sampling
// call takes the next seed of a process-wide counter that starts at a
// random_device value, or at the value given to set_sampler_seed().
inline std::atomic<uint64_t>& sampler_seed() {
  static std::atomic<uint64_t> s{((uint64_t)std::random_device{}() << 32) ^ std::random_device{}()};
  return s;
}
}  // namespace detail

inline void set_sampler_seed(uint64_t seed) { detail::sampler_seed().store(seed); }

namespace detail {
// poly<N> entry points of the word size the build selected.
using W = params::value_type;
#ifdef YELL_USE_32BITS_MODULI
inline int poly_forward(W* const* l, uint32_t L, uint32_t n) { return yell32_poly_forward(l, L, n); }
inline int poly_forward_lazy(W* const* l, uint32_t L, uint32_t n) { return yell32_poly_forward_lazy(l, L, n); }
inline int poly_backward(W* const* l, uint32_t L, uint32_t n) { return yell32_poly_backward(l, L, n); }
inline int poly_negate(W* const* l, uint32_t L, uint32_t n) { return yell32_poly_negate(l, L, n); }
inline int poly_mulmod(W* const* d, const W* const* a, const W* const* b, uint32_t L, uint32_t n) {
  return yell32_poly_mulmod(d, a, b, L, n);
}
inline int poly_addmod(W* const* d, const W* const* a, const W* const* b, uint32_t L, uint32_t n) {
  return yell32_poly_addmod(d, a, b, L, n);
}
inline int poly_submod(W* const* d, const W* const* a, const W* const* b, uint32_t L, uint32_t n) {
  return yell32_poly_submod(d, a, b, L, n);
}
inline int poly_add_product_of(W* const* d, const W* const* a, const W* const* b, uint32_t L, uint32_t n) {
  return yell32_poly_add_product_of(d, a, b, L, n);
}
#else
inline int poly_forward(W* const* l, uint32_t L, uint32_t n) { return yell_poly_forward(l, L, n); }
inline int poly_forward_lazy(W* const* l, uint32_t L, uint32_t n) { return yell_poly_forward_lazy(l, L, n); }
inline int poly_backward(W* const* l, uint32_t L, uint32_t n) { return yell_poly_backward(l, L, n); }
inline int poly_negate(W* const* l, uint32_t L, uint32_t n) { return yell_poly_negate(l, L, n); }
inline int poly_mulmod(W* const* d, const W* const* a, const W* const* b, uint32_t L, uint32_t n) {
  return yell_poly_mulmod(d, a, b, L, n);
}
inline int poly_addmod(W* const* d, const W* const* a, const W* const* b, uint32_t L, uint32_t n) {
  return yell_poly_addmod(d, a, b, L, n);
}
inline int poly_submod(W* const* d, const W* const* a, const W* const* b, uint32_t L, uint32_t n) {
  return yell_poly_submod(d, a, b, L, n);
}
inline int poly_add_product_of(W* const* d, const W* const* a, const W* const* b, uint32_t L, uint32_t n) {
  return yell_poly_add_product_of(d, a, b, L, n);
}
#endif
}  // namespace detail

template <size_t degree_>
class poly {
  static_assert(degree_ < params::kMaxPolyDegree, "");
  size_t nmoduli;
  std::vector<params::value_type*> _data;
  static constexpr uint32_t log_n = static_log2<degree_>::value;

  static params::value_type* alloc_limb() {
    void* p = nullptr;
    if (posix_memalign(&p, 64, degree_ * sizeof(params::value_type)) != 0) throw std::bad_alloc();
    std::memset(p, 0, degree_ * sizeof(params::value_type));
    return static_cast<params::value_type*>(p);
  }

 public:
  using value_type = params::value_type;
  using gt_value_type = params::gt_value_type;
  using signed_type = params::signed_type;
  using pointer_type = value_type*;
  using const_pointer_type = value_type const*;
  using iterator = pointer_type;
  using const_iterator = const_pointer_type;
  static constexpr size_t degree = degree_;
  static constexpr size_t logn = log_n;

  explicit poly(size_t nmoduli_) : nmoduli(nmoduli_) {
    assert(nmoduli <= params::kMaxNbModuli);
    for (size_t cm = 0; cm < nmoduli; ++cm) _data.push_back(alloc_limb());
  }
#ifndef YELL_USE_32BITS_MODULI
  // the device samplers fill 64-bit words; the 32-bit mode has none
  poly(size_t nmoduli_, uniform const& mode) : poly(nmoduli_) { set(mode); }
  poly(size_t nmoduli_, hwt_dist const& mode) : poly(nmoduli_) { set(mode); }
  poly(size_t nmoduli_, ZO_dist const& mode) : poly(nmoduli_) { set(mode); }
  poly(size_t nmoduli_, gaussian_dist const& mode) : poly(nmoduli_) { set(mode); }

  // details/poly.hpp:195-330, sampled on the device and copied into the limbs.
  void set(uniform const&) {
    sample([&](uint64_t* d, uint64_t seed) {
      return yell_dev_sample_uniform(d, 1, (uint32_t)nmoduli, log_n, 0, seed, nullptr);
    });
  }
  void set(hwt_dist const& mode) {
    sample([&](uint64_t* d, uint64_t seed) {
      return yell_dev_sample_hwt(d, 1, (uint32_t)nmoduli, log_n, 0, mode.hwt, seed, nullptr);
    });
  }
  void set(ZO_dist const& mode) {
    sample([&](uint64_t* d, uint64_t seed) {
      return yell_dev_sample_zo(d, 1, (uint32_t)nmoduli, log_n, 0, mode.rho, seed, nullptr);
    });
  }
  void set(gaussian_dist const& mode) {
    sample([&](uint64_t* d, uint64_t seed) {
      return yell_dev_sample_gaussian(d, 1, (uint32_t)nmoduli, log_n, 0, mode.sigma, mode.tail, mode.amplifier,
                                      seed, nullptr);
    });
  }
#endif
  ~poly() {
    for (auto& p : _data) std::free(p);
  }
  poly(poly const& oth) : poly(oth.nmoduli) {
    for (size_t cm = 0; cm < nmoduli; ++cm) std::memcpy(_data[cm], oth._data[cm], degree_ * sizeof(value_type));
  }
  poly(poly&& oth) : nmoduli(0) { swap(*this, oth); }
  poly& operator=(poly const& oth) {
    resize_moduli_count(oth.moduli_count());
    for (size_t cm = 0; cm < nmoduli; ++cm) std::memcpy(_data[cm], oth._data[cm], degree_ * sizeof(value_type));
    return *this;
  }

  iterator ptr_at(size_t cm) { return _data.at(cm); }
  iterator ptr_end(size_t cm) { return ptr_at(cm) + degree; }
  const_iterator cptr_at(size_t cm) const { return _data.at(cm); }
  const_iterator cptr_end(size_t cm) const { return cptr_at(cm) + degree; }

  bool operator==(poly const& oth) const {
    if (nmoduli != oth.nmoduli) return false;
    for (size_t cm = 0; cm < nmoduli; ++cm)
      if (std::memcmp(_data[cm], oth._data[cm], degree_ * sizeof(value_type)) != 0) return false;
    return true;
  }
  bool operator!=(poly const& oth) const { return !(*this == oth); }

  // details/poly.hpp:118-132: *this += op0 * op1 (ops::muladd per word).
  poly& add_product_of(const poly& op0, const poly& op1) {
    assert(nmoduli == op0.nmoduli && nmoduli == op1.nmoduli);
    check_status(detail::poly_add_product_of(_data.data(), op0._data.data(), op1._data.data(),
                                          (uint32_t)nmoduli, log_n),
                 "add_product_of");
    return *this;
  }
#ifndef YELL_USE_32BITS_MODULI
  // details/poly.hpp:135-149: a * s computed as a * r + a * (s - r) with a
  // fresh uniform r, so s never meets a in one product (NTT domain).
  poly& mul_sensitive_poly(const poly& sensitive_poly) {
    assert(nmoduli == sensitive_poly.nmoduli);
    poly r0(nmoduli, uniform{});
    poly r1 = sensitive_poly - r0;
    r1 *= *this;
    *this *= r0;
    *this += r1;
    r0.clear();
    r1.clear();
    return *this;
  }
#endif
  // details/poly.hpp:151-157
  void negate() { check_status(detail::poly_negate(_data.data(), (uint32_t)nmoduli, log_n), "negate"); }

  // details/poly.hpp:90-109
  void resize_moduli_count(size_t new_nmoduli) {
    assert(new_nmoduli <= params::kMaxNbModuli);
    while (_data.size() < new_nmoduli) _data.push_back(alloc_limb());
    while (_data.size() > new_nmoduli) {
      std::free(_data.back());
      _data.pop_back();
    }
    nmoduli = new_nmoduli;
  }

  value_type const& operator()(size_t cm, size_t i) const { return _data[cm][i]; }
  value_type& operator()(size_t cm, size_t i) { return _data[cm][i]; }

#ifndef YELL_USE_32BITS_MODULI
 private:
  template <class F>
  void sample(F&& fill) {
    if (nmoduli == 0) return;
    yell_dev_poly* h = nullptr;
    check_status(yell_dev_poly_alloc((uint32_t)nmoduli, log_n, 0, &h), "sample (alloc)");
    uint64_t* d = nullptr;
    int st = yell_dev_poly_info(h, &d, nullptr, nullptr, nullptr);
    if (st == YELL_OK) st = fill(d, detail::sampler_seed().fetch_add(1));
    if (st == YELL_OK) st = yell_dev_poly_download(h, _data.data());
    yell_dev_poly_free(h);
    check_status(st, "sample");
  }

 public:
#endif

  // details/poly.hpp:170-186, one GPU call over all limbs each.
  void forward() { check_status(detail::poly_forward(_data.data(), (uint32_t)nmoduli, log_n), "forward"); }
  void forward_lazy() {
    check_status(detail::poly_forward_lazy(_data.data(), (uint32_t)nmoduli, log_n), "forward_lazy");
  }
  void backward() { check_status(detail::poly_backward(_data.data(), (uint32_t)nmoduli, log_n), "backward"); }

  value_type get_modulus(size_t cm) { return params::P[cm]; }
  params::value_type** raw_data() { return _data.data(); }
  params::value_type* const* raw_data() const { return _data.data(); }
  friend void swap(poly& a, poly& b) {
    std::swap(a._data, b._data);
    std::swap(a.nmoduli, b.nmoduli);
  }
  void clear() {
    for (size_t cm = 0; cm < nmoduli; ++cm) std::memset(_data[cm], 0, degree_ * sizeof(value_type));
  }
  size_t moduli_count() const { return nmoduli; }
  // details/poly.hpp:357-368: every word below its modulus (debug builds only).
  void check_vaild_range() const {
#ifndef NDEBUG
    for (size_t cm = 0; cm < nmoduli; ++cm)
      for (size_t i = 0; i < degree_; ++i) assert(_data[cm][i] < params::P[cm]);
#endif
  }
};

// details/poly.hpp:336-354: {{w0ULL, w1ULL, ...}\n{...}}, one brace group per limb.
template <size_t Degree>
std::ostream& operator<<(std::ostream& os, poly<Degree> const& p) {
  os << "{";
  for (size_t cm = 0; cm < p.moduli_count(); ++cm) {
    os << "{";
    for (size_t i = 0; i < Degree; ++i) os << p(cm, i) << "ULL" << (i + 1 < Degree ? ", " : "}");
    if (cm + 1 < p.moduli_count()) os << "\n";
  }
  return os << "}";
}

// include/yell/poly.hpp:144-161: limb cm viewed as a std::array of N words.
template <typename value_type, size_t degree>
struct ArrayPointer {
  using T = std::array<value_type, degree>*;
  using cT = const T;
};
template <size_t degree>
typename ArrayPointer<params::value_type, degree>::T recast_as_array(poly<degree>& op, size_t cm) {
  assert(cm < op.moduli_count());
  return reinterpret_cast<typename ArrayPointer<params::value_type, degree>::T>(op.ptr_at(cm));
}

namespace detail {
template <size_t N, int (*FN)(W* const*, const W* const*, const W* const*, uint32_t, uint32_t)>
poly<N> binary_op(poly<N> const& a, poly<N> const& b, const char* name) {
  const size_t L = a.moduli_count() < b.moduli_count() ? a.moduli_count() : b.moduli_count();
  poly<N> r(L);
  check_status(FN(r.raw_data(), a.raw_data(), b.raw_data(), (uint32_t)L, poly<N>::logn), name);
  return r;
}
template <size_t N, int (*FN)(W* const*, const W* const*, const W* const*, uint32_t, uint32_t)>
poly<N>& self_op(poly<N>& a, poly<N> const& b, const char* name) {
  const size_t L = a.moduli_count() < b.moduli_count() ? a.moduli_count() : b.moduli_count();
  check_status(FN(a.raw_data(), a.raw_data(), b.raw_data(), (uint32_t)L, poly<N>::logn), name);
  return a;
}
}  // namespace detail

// include/yell/poly.hpp:163-168 (the YELL_BINARY_OPERATOR loops of ops.hpp:7-41).
template <size_t N> poly<N> operator*(poly<N> const& a, poly<N> const& b) { return detail::binary_op<N, detail::poly_mulmod>(a, b, "operator*"); }
template <size_t N> poly<N> operator+(poly<N> const& a, poly<N> const& b) { return detail::binary_op<N, detail::poly_addmod>(a, b, "operator+"); }
template <size_t N> poly<N> operator-(poly<N> const& a, poly<N> const& b) { return detail::binary_op<N, detail::poly_submod>(a, b, "operator-"); }
template <size_t N> poly<N>& operator*=(poly<N>& a, poly<N> const& b) { return detail::self_op<N, detail::poly_mulmod>(a, b, "operator*="); }
template <size_t N> poly<N>& operator+=(poly<N>& a, poly<N> const& b) { return detail::self_op<N, detail::poly_addmod>(a, b, "operator+="); }
template <size_t N> poly<N>& operator-=(poly<N>& a, poly<N> const& b) { return detail::self_op<N, detail::poly_submod>(a, b, "operator-="); }

}  // namespace yell
