// Harness around the reference's own hot-path sources built in their 32-bit
// moduli mode (fionser/YELL, -DYELL_USE_32BITS_MODULI selects
// include/yell/params_32.hpp: 291 30-bit primes, uint32 words, uint64
// products, degrees up to kMaxPolyDegree = 2^15).
//
// TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles this file together with
// the reference's unmodified lib/{ntt,ops,math,params}.cpp into
// oracle/_ref/libyellref32.so where the reference checkout exists; it pins the
// 32-bit restatement in yell_oracle32.c and produces tests/golden fixtures.
#include <chrono>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>
#include "yell/ntt.hpp"
#include "yell/ops.hpp"
#include "yell/params.hpp"

static_assert(sizeof(yell::params::value_type) == 4, "build with -DYELL_USE_32BITS_MODULI");

namespace {

using word = uint32_t;

template <size_t N>
struct entry32 {
  static void forward(word* x, size_t cm) { yell::ntt<N>::forward(x, cm); }
  static void forward_lazy(word* x, size_t cm) { yell::ntt<N>::forward_lazy(x, cm); }
  static void backward(word* x, size_t cm) { yell::ntt<N>::backward(x, cm); }
  static void tables(size_t cm, word* out, word* sc) {
    auto t = yell::ntt<N>::init_table(cm);
    std::memcpy(out, t->phiTbl, N * 4);
    std::memcpy(out + N, t->shoupPhiTbl, N * 4);
    std::memcpy(out + 2 * N, t->invphiTbl, N * 4);
    std::memcpy(out + 3 * N, t->shoupInvphiTbl, N * 4);
    sc[0] = t->invDegree;
    sc[1] = t->shoupInvDegree;
    sc[2] = t->invphiInvDegree;
    sc[3] = t->shoupInvphiInvDegree;
  }
};

enum class op_kind { fwd, fwd_lazy, bwd };

template <size_t N>
void run_one(op_kind k, word* x, size_t cm) {
  if (k == op_kind::fwd) entry32<N>::forward(x, cm);
  else if (k == op_kind::fwd_lazy) entry32<N>::forward_lazy(x, cm);
  else entry32<N>::backward(x, cm);
}

#define YELL_REF32_SWITCH(LOGN, CALL) \
  switch (LOGN) {                     \
    case 2: CALL(4); break;           \
    case 3: CALL(8); break;           \
    case 4: CALL(16); break;          \
    case 5: CALL(32); break;          \
    case 6: CALL(64); break;          \
    case 7: CALL(128); break;         \
    case 8: CALL(256); break;         \
    case 9: CALL(512); break;         \
    case 10: CALL(1024); break;       \
    case 11: CALL(2048); break;       \
    case 12: CALL(4096); break;       \
    case 13: CALL(8192); break;       \
    case 14: CALL(16384); break;      \
    case 15: CALL(32768); break;      \
    default: return -1;               \
  }

template <size_t N>
void polymul_limb(word* c, const word* a, const word* b, word* tmp, size_t cm) {
  std::memcpy(c, a, N * 4);
  std::memcpy(tmp, b, N * 4);
  yell::ntt<N>::forward(c, cm);
  yell::ntt<N>::forward(tmp, cm);
  yell::ops::mulmod op;
  for (size_t i = 0; i < N; ++i) c[i] = op(c[i], tmp[i], cm);
  yell::ntt<N>::backward(c, cm);
}

template <size_t N>
double polymul_batch(word* c, const word* a, const word* b, uint32_t pairs, uint32_t L, uint32_t threads) {
  yell::ntt<N>::init_ntt_tables(L);
  const size_t units = (size_t)pairs * L;
  auto t0 = std::chrono::steady_clock::now();
  auto work = [&](uint32_t tid) {
    std::vector<word> tmp(N);
    for (size_t u = tid; u < units; u += threads) polymul_limb<N>(c + u * N, a + u * N, b + u * N, tmp.data(), u % L);
  };
  if (threads <= 1) {
    work(0);
  } else {
    std::vector<std::thread> th;
    for (uint32_t i = 0; i < threads; ++i) th.emplace_back(work, i);
    for (auto& t : th) t.join();
  }
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

extern "C" {

uint32_t ref32_prime(uint32_t cm) { return yell::params::P[cm]; }
uint32_t ref32_pn(uint32_t cm) { return yell::params::Pn[cm]; }
uint32_t ref32_primitive_root(uint32_t cm) { return yell::params::primitive_roots[cm]; }
uint32_t ref32_max_moduli(void) { return yell::params::kMaxNbModuli; }

static int dispatch(op_kind k, word* x, uint32_t log_n, uint32_t cm) {
  if (cm >= yell::params::kMaxNbModuli) return -1;
#define CALL_RUN(N) run_one<N>(k, x, cm)
  YELL_REF32_SWITCH(log_n, CALL_RUN)
#undef CALL_RUN
  return 0;
}

int ref32_forward(word* x, uint32_t log_n, uint32_t cm) { return dispatch(op_kind::fwd, x, log_n, cm); }
int ref32_forward_lazy(word* x, uint32_t log_n, uint32_t cm) { return dispatch(op_kind::fwd_lazy, x, log_n, cm); }
int ref32_backward(word* x, uint32_t log_n, uint32_t cm) { return dispatch(op_kind::bwd, x, log_n, cm); }

int ref32_ntt_tables(uint32_t log_n, uint32_t cm, word* out4n, word* scalars) {
  if (cm >= yell::params::kMaxNbModuli) return -1;
#define CALL_TAB(N) entry32<N>::tables(cm, out4n, scalars)
  YELL_REF32_SWITCH(log_n, CALL_TAB)
#undef CALL_TAB
  return 0;
}

uint32_t ref32_barrett(uint64_t x, uint32_t cm) {
  yell::params::gt_value_type v = x;
  yell::ops::barret_reduction(&v, cm);
  return (uint32_t)v;
}

uint32_t ref32_shoupify(uint32_t x, uint32_t cm) { return yell::ops::shoupify(x, cm); }

void ref32_mulmod_n(word* d, const word* a, const word* b, size_t n, uint32_t cm) {
  yell::ops::mulmod op;
  for (size_t i = 0; i < n; ++i) d[i] = op(a[i], b[i], cm);
}
void ref32_addmod_n(word* d, const word* a, const word* b, size_t n, uint32_t cm) {
  yell::ops::addmod op;
  for (size_t i = 0; i < n; ++i) d[i] = op(a[i], b[i], cm);
}
void ref32_submod_n(word* d, const word* a, const word* b, size_t n, uint32_t cm) {
  yell::ops::submod op;
  for (size_t i = 0; i < n; ++i) d[i] = op(a[i], b[i], cm);
}
void ref32_muladd_n(word* rop, const word* a, const word* b, size_t n, uint32_t cm) {
  yell::ops::muladd op;
  for (size_t i = 0; i < n; ++i) op.compute(rop[i], a[i], b[i], cm);
}
void ref32_mulmod_shoup_n(word* d, const word* a, word y, size_t n, uint32_t cm) {
  yell::ops::mulmod_shoup op;
  const word yp = yell::ops::shoupify(y, cm);
  for (size_t i = 0; i < n; ++i) d[i] = op(a[i], y, yp, cm);
}

double ref32_polymul_batch(word* c, const word* a, const word* b, uint32_t pairs, uint32_t L, uint32_t log_n,
                           uint32_t threads) {
  double t = -1.0;
#define CALL_PM(N) t = polymul_batch<N>(c, a, b, pairs, L, threads)
  switch (log_n) {
    case 10: CALL_PM(1024); break;
    case 12: CALL_PM(4096); break;
    case 14: CALL_PM(16384); break;
    case 15: CALL_PM(32768); break;
    default: return -1.0;
  }
#undef CALL_PM
  return t;
}

}  // extern "C"
