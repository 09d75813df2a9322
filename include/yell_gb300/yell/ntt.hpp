// Drop-in for yell/ntt.hpp (include/yell/ntt.hpp:6-66): yell::ntt<N>'s static
// calls, each one a GPU call through the yell_gb300 C ABI on host memory.
// Failures (which the reference only asserts on) throw yell::gpu_error.
#pragma once
#include <cstddef>
#include <stdexcept>
#include <string>
#include "yell/params.hpp"
#include "yell_gb300.h"

namespace yell {

struct gpu_error : std::runtime_error {
  int status;
  gpu_error(int st, const char* fn)
      : std::runtime_error(std::string(fn) + ": " + yell_status_string(st) + " (" + yell_last_error() + ")"),
        status(st) {}
};

inline void check_status(int st, const char* fn) {
  if (st != YELL_OK) throw gpu_error(st, fn);
}

template <size_t N>
struct static_log2 {
  static_assert(N >= 2 && (N & (N - 1)) == 0, "degree must be a power of two");
  static constexpr uint32_t value = 1 + static_log2<N / 2>::value;
};
template <>
struct static_log2<1> {
  static constexpr uint32_t value = 0;
};

namespace detail {
// The C ABI entry points of the word size the build selected.
#ifdef YELL_USE_32BITS_MODULI
inline int ntt_init_table(uint32_t log_n, uint32_t cm) { return yell32_init_ntt_tables(log_n, cm, 1); }
inline int ntt_init_tables(uint32_t log_n, uint32_t K) { return yell32_init_ntt_tables(log_n, 0, K); }
inline int ntt_forward(uint32_t* op, uint32_t log_n, uint32_t cm) { return yell32_ntt_forward(op, log_n, cm); }
inline int ntt_forward_lazy(uint32_t* op, uint32_t log_n, uint32_t cm) { return yell32_ntt_forward_lazy(op, log_n, cm); }
inline int ntt_backward(uint32_t* op, uint32_t log_n, uint32_t cm) { return yell32_ntt_backward(op, log_n, cm); }
#else
inline int ntt_init_table(uint32_t log_n, uint32_t cm) { return yell_init_table(log_n, cm); }
inline int ntt_init_tables(uint32_t log_n, uint32_t K) { return yell_init_ntt_tables(log_n, K); }
inline int ntt_forward(uint64_t* op, uint32_t log_n, uint32_t cm) { return yell_ntt_forward(op, log_n, cm); }
inline int ntt_forward_lazy(uint64_t* op, uint32_t log_n, uint32_t cm) { return yell_ntt_forward_lazy(op, log_n, cm); }
inline int ntt_backward(uint64_t* op, uint32_t log_n, uint32_t cm) { return yell_ntt_backward(op, log_n, cm); }
#endif
}  // namespace detail

#ifndef YELL_USE_32BITS_MODULI
// include/yell/details/ntt.hpp:10-23: the runtime-N lazy loops with caller
// tables (forward: [0,4p) in and out; backward: all layers but m = 1).
inline void negacylic_forward_lazy(params::value_type* x, const size_t degree, const params::value_type* w,
                                   const params::value_type* wshoup, const params::value_type p) {
  check_status(yell_negacyclic_forward_lazy(x, degree, w, wshoup, p), "negacylic_forward_lazy");
}
inline void negacylic_backward_lazy(params::value_type* x, const size_t degree, const params::value_type* w,
                                    const params::value_type* wshoup, const params::value_type p) {
  check_status(yell_negacyclic_backward_lazy(x, degree, w, wshoup, p), "negacylic_backward_lazy");
}
#endif

template <size_t degree_>
class ntt {
  using T = params::value_type;
  static constexpr uint32_t log_n = static_log2<degree_>::value;

 public:
  static constexpr size_t degree = degree_;
  // include/yell/ntt.hpp:50: builds the table of modulus cm (on the GPU, kept for the process).
  static void init_table(size_t cm) { check_status(detail::ntt_init_table(log_n, (uint32_t)cm), "init_table"); }
  // include/yell/ntt.hpp:53-56
  static void init_ntt_tables(size_t K) {
    check_status(detail::ntt_init_tables(log_n, (uint32_t)K), "init_ntt_tables");
  }
  // include/yell/ntt.hpp:59: in place, bit-reversed output in [0, p).
  static void forward(T* op, size_t cm) { check_status(detail::ntt_forward(op, log_n, (uint32_t)cm), "forward"); }
  // include/yell/ntt.hpp:62: in place, output in [0, 4p).
  static void forward_lazy(T* op, size_t cm) {
    check_status(detail::ntt_forward_lazy(op, log_n, (uint32_t)cm), "forward_lazy");
  }
  // include/yell/ntt.hpp:65: in place, natural-order output in [0, p).
  static void backward(T* op, size_t cm) { check_status(detail::ntt_backward(op, log_n, (uint32_t)cm), "backward"); }
};

}  // namespace yell
