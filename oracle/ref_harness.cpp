// Harness around the reference's own hot-path sources (fionser/YELL).
//
// TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles this file together
// with the reference's unmodified lib/{ntt,ops,math,params}.cpp, where they
// lie in the reference checkout, into oracle/_ref/libyellref.so.  It exists
// only where the reference sources are present; it pins the C restatement in
// yell_oracle.c and produces the fixtures in tests/golden/.
//
// The reference's yell::poly<N> is not includable (yell/poly.hpp pulls in
// <gmp.h> and an MPFR sampler), so the element-wise entry points below call
// the yell::ops functors exactly as the YELL_BINARY_OPERATOR loop does
// (include/yell/ops.hpp:7-41).  N is a template parameter in the reference
// (include/yell/ntt.hpp:6-7); the switch below instantiates 2^2 .. 2^20.
#include <cstdint>
#include <cstring>
#include <chrono>
#include <thread>
#include <vector>
#include "yell/ntt.hpp"
#include "yell/ops.hpp"
#include "yell/params.hpp"

namespace {

template <size_t N>
struct ntt_entry {
  static void forward(uint64_t* x, size_t cm) { yell::ntt<N>::forward(x, cm); }
  static void forward_lazy(uint64_t* x, size_t cm) { yell::ntt<N>::forward_lazy(x, cm); }
  static void backward(uint64_t* x, size_t cm) { yell::ntt<N>::backward(x, cm); }
  static void tables(size_t cm, uint64_t* out, uint64_t* sc) {
    auto t = yell::ntt<N>::init_table(cm);
    std::memcpy(out, t->phiTbl, N * 8);
    std::memcpy(out + N, t->shoupPhiTbl, N * 8);
    std::memcpy(out + 2 * N, t->invphiTbl, N * 8);
    std::memcpy(out + 3 * N, t->shoupInvphiTbl, N * 8);
    sc[0] = t->invDegree;
    sc[1] = t->shoupInvDegree;
    sc[2] = t->invphiInvDegree;
    sc[3] = t->shoupInvphiInvDegree;
  }
};

enum class op_kind { fwd, fwd_lazy, bwd };

template <size_t N>
void run_one(op_kind k, uint64_t* x, size_t cm) {
  if (k == op_kind::fwd) ntt_entry<N>::forward(x, cm);
  else if (k == op_kind::fwd_lazy) ntt_entry<N>::forward_lazy(x, cm);
  else ntt_entry<N>::backward(x, cm);
}

#define YELL_REF_SWITCH(LOGN, CALL)            \
  switch (LOGN) {                              \
    case 2: CALL(4); break;                    \
    case 3: CALL(8); break;                    \
    case 4: CALL(16); break;                   \
    case 5: CALL(32); break;                   \
    case 6: CALL(64); break;                   \
    case 7: CALL(128); break;                  \
    case 8: CALL(256); break;                  \
    case 9: CALL(512); break;                  \
    case 10: CALL(1024); break;                \
    case 11: CALL(2048); break;                \
    case 12: CALL(4096); break;                \
    case 13: CALL(8192); break;                \
    case 14: CALL(16384); break;               \
    case 15: CALL(32768); break;               \
    case 16: CALL(65536); break;               \
    case 17: CALL(131072); break;              \
    case 18: CALL(262144); break;              \
    case 19: CALL(524288); break;              \
    case 20: CALL(1048576); break;             \
    default: return -1;                        \
  }

int dispatch(op_kind k, uint64_t* x, uint32_t log_n, uint32_t cm) {
  if (cm >= yell::params::kMaxNbModuli) return -1;
#define CALL_RUN(N) run_one<N>(k, x, cm)
  YELL_REF_SWITCH(log_n, CALL_RUN)
#undef CALL_RUN
  return 0;
}

// a.forward(); b.forward(); c = a * b; c.backward() on one limb.
template <size_t N>
void polymul_limb(uint64_t* c, const uint64_t* a, const uint64_t* b, uint64_t* tmp, size_t cm) {
  std::memcpy(c, a, N * 8);
  std::memcpy(tmp, b, N * 8);
  yell::ntt<N>::forward(c, cm);
  yell::ntt<N>::forward(tmp, cm);
  yell::ops::mulmod op;
  for (size_t i = 0; i < N; ++i) c[i] = op(c[i], tmp[i], cm);
  yell::ntt<N>::backward(c, cm);
}

template <size_t N>
double polymul_batch(uint64_t* c, const uint64_t* a, const uint64_t* b, uint32_t pairs,
                     uint32_t L, uint32_t threads) {
  yell::ntt<N>::init_ntt_tables(L);
  size_t units = (size_t)pairs * L;
  auto t0 = std::chrono::steady_clock::now();
  auto work = [&](uint32_t tid) {
    std::vector<uint64_t> tmp(N);
    for (size_t u = tid; u < units; u += threads)
      polymul_limb<N>(c + u * N, a + u * N, b + u * N, tmp.data(), u % L);
  };
  if (threads <= 1) {
    work(0);
  } else {
    std::vector<std::thread> th;
    for (uint32_t i = 0; i < threads; ++i) th.emplace_back(work, i);
    for (auto& t : th) t.join();
  }
  auto t1 = std::chrono::steady_clock::now();
  return std::chrono::duration<double>(t1 - t0).count();
}

}  // namespace

extern "C" {

uint64_t ref_prime(uint32_t cm) { return yell::params::P[cm]; }
uint64_t ref_pn(uint32_t cm) { return yell::params::Pn[cm]; }
uint64_t ref_primitive_root(uint32_t cm) { return yell::params::primitive_roots[cm]; }
uint32_t ref_max_moduli(void) { return yell::params::kMaxNbModuli; }

int ref_forward(uint64_t* x, uint32_t log_n, uint32_t cm) { return dispatch(op_kind::fwd, x, log_n, cm); }
int ref_forward_lazy(uint64_t* x, uint32_t log_n, uint32_t cm) { return dispatch(op_kind::fwd_lazy, x, log_n, cm); }
int ref_backward(uint64_t* x, uint32_t log_n, uint32_t cm) { return dispatch(op_kind::bwd, x, log_n, cm); }

int ref_ntt_tables(uint32_t log_n, uint32_t cm, uint64_t* out4n, uint64_t* scalars) {
  if (cm >= yell::params::kMaxNbModuli) return -1;
#define CALL_TAB(N) ntt_entry<N>::tables(cm, out4n, scalars)
  YELL_REF_SWITCH(log_n, CALL_TAB)
#undef CALL_TAB
  return 0;
}

uint64_t ref_barrett(uint64_t hi, uint64_t lo, uint32_t cm) {
  yell::params::gt_value_type x = ((yell::params::gt_value_type)hi << 64) | lo;
  yell::ops::barret_reduction(&x, cm);
  return (uint64_t)x;
}

uint64_t ref_shoupify(uint64_t x, uint32_t cm) { return yell::ops::shoupify(x, cm); }

void ref_mulmod_n(uint64_t* d, const uint64_t* a, const uint64_t* b, size_t n, uint32_t cm) {
  yell::ops::mulmod op;
  for (size_t i = 0; i < n; ++i) d[i] = op(a[i], b[i], cm);
}

void ref_addmod_n(uint64_t* d, const uint64_t* a, const uint64_t* b, size_t n, uint32_t cm) {
  yell::ops::addmod op;
  for (size_t i = 0; i < n; ++i) d[i] = op(a[i], b[i], cm);
}

void ref_submod_n(uint64_t* d, const uint64_t* a, const uint64_t* b, size_t n, uint32_t cm) {
  yell::ops::submod op;
  for (size_t i = 0; i < n; ++i) d[i] = op(a[i], b[i], cm);
}

void ref_muladd_n(uint64_t* rop, const uint64_t* a, const uint64_t* b, size_t n, uint32_t cm) {
  yell::ops::muladd op;
  for (size_t i = 0; i < n; ++i) op.compute(rop[i], a[i], b[i], cm);
}

void ref_mulmod_shoup_n(uint64_t* d, const uint64_t* a, uint64_t y, size_t n, uint32_t cm) {
  yell::ops::mulmod_shoup op;
  uint64_t yp = yell::ops::shoupify(y, cm);
  for (size_t i = 0; i < n; ++i) d[i] = op(a[i], y, yp, cm);
}

int ref_negacyclic_forward_lazy(uint64_t* x, uint64_t degree, const uint64_t* w, const uint64_t* ws, uint64_t p) {
  yell::negacylic_forward_lazy(x, (size_t)degree, w, ws, p);
  return 0;
}

int ref_negacyclic_backward_lazy(uint64_t* x, uint64_t degree, const uint64_t* w, const uint64_t* ws, uint64_t p) {
  yell::negacylic_backward_lazy(x, (size_t)degree, w, ws, p);
  return 0;
}

double ref_polymul_batch(uint64_t* c, const uint64_t* a, const uint64_t* b, uint32_t pairs,
                         uint32_t L, uint32_t log_n, uint32_t threads) {
  double t = -1.0;
#define CALL_PM(N) t = polymul_batch<N>(c, a, b, pairs, L, threads)
  switch (log_n) {
    case 10: CALL_PM(1024); break;
    case 12: CALL_PM(4096); break;
    case 13: CALL_PM(8192); break;
    case 14: CALL_PM(16384); break;
    case 16: CALL_PM(65536); break;
    default: return -1.0;
  }
#undef CALL_PM
  return t;
}

}  // extern "C"
