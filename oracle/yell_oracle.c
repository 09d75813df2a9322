/*
 * CPU oracle for the YELL RNS-polynomial hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: the parity tests, the
 * smoke check and the CPU-baseline leg of the benchmark load it.  No product
 * code path calls it, links it or falls back to it.
 *
 * It is a plain-C restatement of the reference algorithm (fionser/YELL), one
 * function per reference routine, each citing the file:line it follows:
 *   - prime table  : include/yell/params_64.hpp:19-38 (regenerated from its
 *                    stated rule, see orc_table_init below)
 *   - Barrett      : lib/ops.cpp:5-21
 *   - shoupify     : lib/ops.cpp:23-27
 *   - addmod/submod/mulmod/mulmod_shoup/muladd : include/yell/ops.hpp:46-158
 *   - twiddles     : include/yell/details/ntt.hpp:97-146
 *   - CT/GS butterflies, lazy NTT loops : lib/ntt.cpp:48-210
 *   - forward / forward_lazy / backward : include/yell/details/ntt.hpp:106-166
 *   - negate       : include/yell/details/poly.hpp:151-157
 *   - add_product_of : include/yell/details/poly.hpp:118-132
 * plus an independent schoolbook negacyclic product in unsigned __int128.
 *
 * Parity of this restatement is pinned against the reference itself (its own
 * lib/{ntt,ops,math,params}.cpp compiled by oracle/Makefile into
 * oracle/_ref/) and against the fixtures in tests/golden/ that were produced
 * from that build.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>
#include <time.h>

typedef unsigned __int128 u128;

#define ORC_MAX_MODULI 1000u      /* params_64.hpp:19 kMaxNbModuli            */
#define ORC_LOG_MAX_DEGREE 20u    /* params_64.hpp:21 kMaxPolyDegree = 2^20   */

/* ------------------------------------------------------------------------ */
/* Prime table.                                                              */
/*                                                                           */
/* params_64.hpp:16-17 states the rule: p = 2^62 - i*2*kMaxPolyDegree + 1 for */
/* increasing i, kept when prime; Pn (params_64.hpp:29-31) is the low word of */
/* floor(2^128/p); primitive_roots (params_64.hpp:33-34) are primitive        */
/* 2^21-th roots of unity, and in that table each one equals g^((p-1)/2^21)  */
/* for g the least primitive root mod p.  The oracle regenerates all three   */
/* with its own primality test and factoring, independently of the product. */
/* ------------------------------------------------------------------------ */

static uint64_t orc_P[ORC_MAX_MODULI];
static uint64_t orc_Pn[ORC_MAX_MODULI];
static uint64_t orc_root[ORC_MAX_MODULI];
static pthread_once_t orc_once = PTHREAD_ONCE_INIT;

static uint64_t mulmod_u128(uint64_t a, uint64_t b, uint64_t m) {
  return (uint64_t)(((u128)a * b) % m);
}

static uint64_t powmod_u128(uint64_t b, uint64_t e, uint64_t m) {
  uint64_t r = 1 % m;
  b %= m;
  while (e) {
    if (e & 1) r = mulmod_u128(r, b, m);
    b = mulmod_u128(b, b, m);
    e >>= 1;
  }
  return r;
}

/* Deterministic Miller-Rabin for n < 2^64 (first 12 prime bases). */
static int is_prime_u64(uint64_t n) {
  static const uint64_t bases[12] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37};
  if (n < 2) return 0;
  for (int i = 0; i < 12; ++i) {
    if (n == bases[i]) return 1;
    if (n % bases[i] == 0) return 0;
  }
  uint64_t d = n - 1;
  int s = 0;
  while ((d & 1) == 0) { d >>= 1; ++s; }
  for (int i = 0; i < 12; ++i) {
    uint64_t x = powmod_u128(bases[i], d, n);
    if (x == 1 || x == n - 1) continue;
    int comp = 1;
    for (int r = 1; r < s; ++r) {
      x = mulmod_u128(x, x, n);
      if (x == n - 1) { comp = 0; break; }
    }
    if (comp) return 0;
  }
  return 1;
}

/* Least primitive root of prime p, with p - 1 = 2^21 * m and m < 2^41. */
static uint64_t least_primitive_root(uint64_t p) {
  uint64_t factors[64];
  int nf = 0;
  uint64_t m = p - 1;
  while ((m & 1) == 0) m >>= 1;
  factors[nf++] = 2;
  for (uint64_t f = 3; f * f <= m; f += 2) {
    if (m % f == 0) {
      factors[nf++] = f;
      while (m % f == 0) m /= f;
    }
  }
  if (m > 1) factors[nf++] = m;
  for (uint64_t g = 2;; ++g) {
    int ok = 1;
    for (int i = 0; i < nf && ok; ++i)
      if (powmod_u128(g, (p - 1) / factors[i], p) == 1) ok = 0;
    if (ok) return g;
  }
}

static void orc_table_init(void) {
  uint32_t k = 0;
  for (uint64_t i = 1; k < ORC_MAX_MODULI; ++i) {
    uint64_t p = (1ull << 62) - i * (2ull << ORC_LOG_MAX_DEGREE) + 1;
    if (!is_prime_u64(p)) continue;
    orc_P[k] = p;
    orc_Pn[k] = (uint64_t)((~(u128)0) / p); /* floor((2^128-1)/p) == floor(2^128/p): p is odd */
    k++;
  }
}

/* Primitive roots are computed on demand (the factoring is the slow part). */
static pthread_mutex_t orc_root_mu = PTHREAD_MUTEX_INITIALIZER;

uint64_t orc_prime(uint32_t cm) {
  pthread_once(&orc_once, orc_table_init);
  return cm < ORC_MAX_MODULI ? orc_P[cm] : 0;
}

uint64_t orc_pn(uint32_t cm) {
  pthread_once(&orc_once, orc_table_init);
  return cm < ORC_MAX_MODULI ? orc_Pn[cm] : 0;
}

uint64_t orc_primitive_root(uint32_t cm) {
  pthread_once(&orc_once, orc_table_init);
  if (cm >= ORC_MAX_MODULI) return 0;
  pthread_mutex_lock(&orc_root_mu);
  if (orc_root[cm] == 0) {
    uint64_t p = orc_P[cm];
    uint64_t g = least_primitive_root(p);
    orc_root[cm] = powmod_u128(g, (p - 1) >> 21, p);
  }
  uint64_t r = orc_root[cm];
  pthread_mutex_unlock(&orc_root_mu);
  return r;
}

/* ------------------------------------------------------------------------ */
/* Modular operations (include/yell/ops.hpp, lib/ops.cpp).                    */
/* ------------------------------------------------------------------------ */

/* lib/ops.cpp:5-21.  q = Pn*(x>>64) + (x<<2) (wrapping u128), r = lo(x) -
 * hi(q)*p (wrapping u64), one conditional subtraction of p. */
static inline uint64_t barrett(u128 x, uint64_t p, uint64_t pn) {
  u128 q = (u128)pn * (uint64_t)(x >> 64) + (x << 2);
  uint64_t r = (uint64_t)x - (uint64_t)(q >> 64) * p;
  if (r >= p) r -= p;
  return r;
}

/* lib/ops.cpp:23-27 */
static inline uint64_t shoupify(uint64_t x, uint64_t p) {
  return (uint64_t)(((u128)x << 64) / p);
}

/* include/yell/ops.hpp:103-112 */
static inline uint64_t mulmod(uint64_t x, uint64_t y, uint64_t p, uint64_t pn) {
  return barrett((u128)x * y, p, pn);
}

/* include/yell/ops.hpp:122-132: x*y - hi(x*y')*p, then mod_correct. */
static inline uint64_t mulmod_shoup(uint64_t x, uint64_t y, uint64_t yp, uint64_t p) {
  uint64_t q = (uint64_t)(((u128)x * yp) >> 64) * p;
  uint64_t r = x * y - q;
  if (r >= p) r -= p;
  return r;
}

/* include/yell/ops.hpp:54-68 (mod_correct at :46-52). */
static inline uint64_t addmod(uint64_t x, uint64_t y, uint64_t p) {
  x += y;
  if (x >= p) x -= p;
  return x;
}

/* include/yell/ops.hpp:70-83 */
static inline uint64_t submod(uint64_t x, uint64_t y, uint64_t p) {
  x += (p - y);
  if (x >= p) x -= p;
  return x;
}

/* include/yell/ops.hpp:144-158 */
static inline uint64_t muladd(uint64_t rop, uint64_t x, uint64_t y, uint64_t p, uint64_t pn) {
  u128 res = (u128)x * y;
  res += rop;
  return barrett(res, p, pn);
}

uint64_t orc_barrett(uint64_t hi, uint64_t lo, uint32_t cm) {
  return barrett(((u128)hi << 64) | lo, orc_prime(cm), orc_pn(cm));
}

uint64_t orc_shoupify(uint64_t x, uint32_t cm) { return shoupify(x, orc_prime(cm)); }

/* Element-wise forms over one limb; dst may alias an operand. */
void orc_mulmod_n(uint64_t* dst, const uint64_t* a, const uint64_t* b, size_t n, uint32_t cm) {
  uint64_t p = orc_prime(cm), pn = orc_pn(cm);
  for (size_t i = 0; i < n; ++i) dst[i] = mulmod(a[i], b[i], p, pn);
}

void orc_addmod_n(uint64_t* dst, const uint64_t* a, const uint64_t* b, size_t n, uint32_t cm) {
  uint64_t p = orc_prime(cm);
  for (size_t i = 0; i < n; ++i) dst[i] = addmod(a[i], b[i], p);
}

void orc_submod_n(uint64_t* dst, const uint64_t* a, const uint64_t* b, size_t n, uint32_t cm) {
  uint64_t p = orc_prime(cm);
  for (size_t i = 0; i < n; ++i) dst[i] = submod(a[i], b[i], p);
}

void orc_muladd_n(uint64_t* rop, const uint64_t* a, const uint64_t* b, size_t n, uint32_t cm) {
  uint64_t p = orc_prime(cm), pn = orc_pn(cm);
  for (size_t i = 0; i < n; ++i) rop[i] = muladd(rop[i], a[i], b[i], p, pn);
}

/* include/yell/details/poly.hpp:151-157 */
void orc_negate_n(uint64_t* x, size_t n, uint32_t cm) {
  uint64_t p = orc_prime(cm);
  for (size_t i = 0; i < n; ++i) x[i] = p - x[i];
}

void orc_mulmod_shoup_n(uint64_t* dst, const uint64_t* a, uint64_t y, size_t n, uint32_t cm) {
  uint64_t p = orc_prime(cm);
  uint64_t yp = shoupify(y, p);
  for (size_t i = 0; i < n; ++i) dst[i] = mulmod_shoup(a[i], y, yp, p);
}

/* ------------------------------------------------------------------------ */
/* Twiddle tables: include/yell/details/ntt.hpp:97-146.                      */
/* ------------------------------------------------------------------------ */

/* include/yell/utils/math.hpp:29-43: in-place bit-reversal permutation. */
static void revbin_permute(uint64_t* a, size_t n) {
  if (n <= 2) return;
  for (size_t i = 1, j = 0; i < n; ++i) {
    size_t bit = n >> 1;
    for (; j >= bit; bit >>= 1) j -= bit;
    j += bit;
    if (i < j) { uint64_t t = a[i]; a[i] = a[j]; a[j] = t; }
  }
}

/* include/yell/utils/math.hpp:21-34: Fermat inverse with Barrett mulmod. */
static uint64_t inv_mod_prime(uint64_t a, uint64_t p, uint64_t pn) {
  uint64_t ret = 1, y = p - 2;
  while (y > 0) {
    if (y & 1) ret = mulmod(ret, a, p, pn);
    y >>= 1;
    a = mulmod(a, a, p, pn);
  }
  return ret;
}

typedef struct {
  uint32_t log_n;
  uint64_t p, pn;
  uint64_t *phi, *phi_s, *iphi, *iphi_s;          /* N words each, bit-reversed */
  uint64_t inv_n, inv_n_s, inv_n_iphi, inv_n_iphi_s;
} orc_tables;

static void tables_build(orc_tables* t, uint32_t log_n, uint32_t cm) {
  size_t n = (size_t)1 << log_n;
  uint64_t p = orc_prime(cm), pn = orc_pn(cm);
  t->log_n = log_n;
  t->p = p;
  t->pn = pn;
  t->phi = (uint64_t*)malloc(4 * n * sizeof(uint64_t));
  t->phi_s = t->phi + n;
  t->iphi = t->phi + 2 * n;
  t->iphi_s = t->phi + 3 * n;
  /* include/yell/details/ntt.hpp:39-43: square the 2^21-th root (20 - log2 N) times. */
  uint64_t phi = orc_primitive_root(cm);
  for (uint32_t i = 0; i < ORC_LOG_MAX_DEGREE - log_n; ++i) phi = mulmod(phi, phi, p, pn);
  /* include/yell/details/ntt.hpp:47-53 */
  uint64_t temp = 1;
  for (size_t i = 0; i < n; ++i) {
    t->phi[i] = temp;
    t->phi_s[i] = shoupify(temp, p);
    temp = mulmod(temp, phi, p, pn);
  }
  /* include/yell/details/ntt.hpp:57-65: phi^N * phi^(N-1) = phi^-1. */
  uint64_t invphi = mulmod(temp, t->phi[n - 1], p, pn);
  temp = 1;
  for (size_t i = 0; i < n; ++i) {
    t->iphi[i] = temp;
    t->iphi_s[i] = shoupify(temp, p);
    temp = mulmod(temp, invphi, p, pn);
  }
  /* include/yell/details/ntt.hpp:67-71 */
  revbin_permute(t->phi, n);
  revbin_permute(t->phi_s, n);
  revbin_permute(t->iphi, n);
  revbin_permute(t->iphi_s, n);
  /* include/yell/details/ntt.hpp:73-76 */
  t->inv_n = inv_mod_prime((uint64_t)n, p, pn);
  t->inv_n_iphi = mulmod(t->inv_n, t->iphi[1], p, pn);
  t->inv_n_s = shoupify(t->inv_n, p);
  t->inv_n_iphi_s = shoupify(t->inv_n_iphi, p);
}

static void tables_free(orc_tables* t) { free(t->phi); }

/* Exports the table for (log_n, cm): out4n holds phi, phi', invphi, invphi'
 * (N words each, bit-reversed); scalars[4] = N^-1, its Shoup form,
 * N^-1*invphi_brv[1], its Shoup form. */
int orc_ntt_tables(uint32_t log_n, uint32_t cm, uint64_t* out4n, uint64_t* scalars) {
  if (log_n < 1 || log_n > ORC_LOG_MAX_DEGREE || cm >= ORC_MAX_MODULI) return -1;
  orc_tables t;
  tables_build(&t, log_n, cm);
  memcpy(out4n, t.phi, 4 * ((size_t)1 << log_n) * sizeof(uint64_t));
  scalars[0] = t.inv_n;
  scalars[1] = t.inv_n_s;
  scalars[2] = t.inv_n_iphi;
  scalars[3] = t.inv_n_iphi_s;
  tables_free(&t);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* NTT loops: lib/ntt.cpp:34-210.                                            */
/* ------------------------------------------------------------------------ */

/* lib/ntt.cpp:69-83.  In/out [0,4p). */
static inline void ct_butterfly(uint64_t* x0, uint64_t* x1, uint64_t w, uint64_t wp,
                                uint64_t p, uint64_t p2) {
  uint64_t u0 = *x0, u1 = *x1;
  if (u0 >= p2) u0 -= p2;
  uint64_t q = (uint64_t)(((u128)u1 * wp) >> 64);
  uint64_t t = u1 * w - q * p;
  *x0 = u0 + t;
  *x1 = u0 - t + p2;
}

/* lib/ntt.cpp:47-63.  In/out [0,2p). */
static inline void gs_butterfly(uint64_t* x0, uint64_t* x1, uint64_t w, uint64_t wp,
                                uint64_t p, uint64_t p2) {
  uint64_t u0 = *x0, u1 = *x1;
  uint64_t t0 = u0 + u1;
  if (t0 >= p2) t0 -= p2;
  uint64_t t1 = u0 - u1 + p2;
  uint64_t q = (uint64_t)(((u128)t1 * wp) >> 64);
  *x0 = t0;
  *x1 = t1 * w - q * p;
}

/* lib/ntt.cpp:89-149.  Stage with m groups of half-size h (h*m = N/2) uses
 * twiddle w[m + r] for group r.  The reference splits out h=2 and h=1 only
 * to pick a constant-time selector; the values are the same as this loop. */
static void forward_lazy_loop(uint64_t* x, size_t n, const uint64_t* w, const uint64_t* ws,
                              uint64_t p) {
  uint64_t p2 = p << 1;
  for (size_t m = 1, h = n >> 1; h >= 1; m <<= 1, h >>= 1) {
    for (size_t r = 0; r < m; ++r) {
      uint64_t* x0 = x + 2 * h * r;
      uint64_t wr = w[m + r], wsr = ws[m + r];
      for (size_t i = 0; i < h; ++i) ct_butterfly(x0 + i, x0 + i + h, wr, wsr, p, p2);
    }
  }
}

/* lib/ntt.cpp:151-210.  Runs the first loop (m=N/2, h=1), the second loop
 * (m=N/4, h=2) unconditionally, then continues while m > 1, so the last
 * layer (m=1) is left to the caller for N >= 8.  At N = 4 the second loop
 * already is the m=1 layer, which the caller then applies again; that quirk
 * is kept here so the oracle reproduces the reference at every size. */
static void backward_lazy_loop(uint64_t* x, size_t n, const uint64_t* w, const uint64_t* ws,
                               uint64_t p) {
  uint64_t p2 = p << 1;
  size_t m = n >> 1, h = 1;
  for (size_t r = 0; r < m; ++r)
    gs_butterfly(x + 2 * r, x + 2 * r + 1, w[m + r], ws[m + r], p, p2);
  m >>= 1;
  h <<= 1;
  for (size_t r = 0; r < m; ++r) {
    uint64_t* x0 = x + 4 * r;
    gs_butterfly(x0, x0 + 2, w[m + r], ws[m + r], p, p2);
    gs_butterfly(x0 + 1, x0 + 3, w[m + r], ws[m + r], p, p2);
  }
  m >>= 1;
  h <<= 1;
  for (; m > 1; m >>= 1, h <<= 1) {
    for (size_t r = 0; r < m; ++r) {
      uint64_t* x0 = x + 2 * h * r;
      for (size_t i = 0; i < h; ++i) gs_butterfly(x0 + i, x0 + i + h, w[m + r], ws[m + r], p, p2);
    }
  }
}

/* The loops with caller tables: negacylic_forward_lazy / negacylic_backward_lazy
 * (include/yell/details/ntt.hpp:10-23). */
int orc_negacyclic_forward_lazy(uint64_t* x, uint64_t degree, const uint64_t* w, const uint64_t* ws, uint64_t p) {
  if (degree < 4 || (degree & (degree - 1))) return -1;
  forward_lazy_loop(x, (size_t)degree, w, ws, p);
  return 0;
}

int orc_negacyclic_backward_lazy(uint64_t* x, uint64_t degree, const uint64_t* w, const uint64_t* ws, uint64_t p) {
  if (degree < 4 || (degree & (degree - 1))) return -1;
  backward_lazy_loop(x, (size_t)degree, w, ws, p);
  return 0;
}

/* include/yell/details/ntt.hpp:125-134 */
static void forward_lazy_t(uint64_t* x, const orc_tables* t) {
  forward_lazy_loop(x, (size_t)1 << t->log_n, t->phi, t->phi_s, t->p);
}

/* include/yell/details/ntt.hpp:106-123: lazy forward, then v -= 2p*[v>=2p]; v -= p*[v>=p]. */
static void forward_t(uint64_t* x, const orc_tables* t) {
  size_t n = (size_t)1 << t->log_n;
  uint64_t p = t->p, p2 = p << 1;
  forward_lazy_t(x, t);
  for (size_t i = 0; i < n; ++i) {
    uint64_t v = x[i];
    if (v >= p2) v -= p2;
    if (v >= p) v -= p;
    x[i] = v;
  }
}

/* include/yell/details/ntt.hpp:136-166: lazy GS stages, then the fused last layer. */
static void backward_t(uint64_t* x, const orc_tables* t) {
  size_t n = (size_t)1 << t->log_n;
  uint64_t p = t->p, p2 = p << 1;
  backward_lazy_loop(x, n, t->iphi, t->iphi_s, p);
  for (size_t i = 0; i < n / 2; ++i) {
    uint64_t u = x[i], v = x[i + n / 2];
    x[i] = mulmod_shoup(u + v, t->inv_n, t->inv_n_s, p);
    x[i + n / 2] = mulmod_shoup(u - v + p2, t->inv_n_iphi, t->inv_n_iphi_s, p);
  }
}

/* Table cache: one table per (log_n, cm), built on first use. */
static orc_tables* orc_cache[ORC_LOG_MAX_DEGREE + 1][ORC_MAX_MODULI];
static pthread_mutex_t orc_cache_mu = PTHREAD_MUTEX_INITIALIZER;

static const orc_tables* tables_get(uint32_t log_n, uint32_t cm) {
  pthread_mutex_lock(&orc_cache_mu);
  orc_tables* t = orc_cache[log_n][cm];
  pthread_mutex_unlock(&orc_cache_mu);
  if (t) return t;
  orc_tables* fresh = (orc_tables*)malloc(sizeof(orc_tables));
  tables_build(fresh, log_n, cm);
  pthread_mutex_lock(&orc_cache_mu);
  if (!orc_cache[log_n][cm]) {
    orc_cache[log_n][cm] = fresh;
    fresh = NULL;
  }
  t = orc_cache[log_n][cm];
  pthread_mutex_unlock(&orc_cache_mu);
  if (fresh) { tables_free(fresh); free(fresh); }
  return t;
}

static int check_args(uint32_t log_n, uint32_t cm) {
  return (log_n >= 2 && log_n <= ORC_LOG_MAX_DEGREE && cm < ORC_MAX_MODULI) ? 0 : -1;
}

int orc_forward(uint64_t* x, uint32_t log_n, uint32_t cm) {
  if (check_args(log_n, cm)) return -1;
  forward_t(x, tables_get(log_n, cm));
  return 0;
}

int orc_forward_lazy(uint64_t* x, uint32_t log_n, uint32_t cm) {
  if (check_args(log_n, cm)) return -1;
  forward_lazy_t(x, tables_get(log_n, cm));
  return 0;
}

int orc_backward(uint64_t* x, uint32_t log_n, uint32_t cm) {
  if (check_args(log_n, cm)) return -1;
  backward_t(x, tables_get(log_n, cm));
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Schoolbook negacyclic product mod p in unsigned __int128: independent of  */
/* every NTT routine above.  c = a*b mod (X^N + 1, p).                        */
/* ------------------------------------------------------------------------ */
int orc_negacyclic_schoolbook(uint64_t* c, const uint64_t* a, const uint64_t* b,
                              uint32_t log_n, uint32_t cm) {
  if (log_n > 13 || cm >= ORC_MAX_MODULI) return -1;
  size_t n = (size_t)1 << log_n;
  uint64_t p = orc_prime(cm);
  for (size_t k = 0; k < n; ++k) {
    u128 pos = 0, neg = 0;
    for (size_t i = 0; i <= k; ++i) pos += ((u128)a[i] * b[k - i]) % p;
    for (size_t i = k + 1; i < n; ++i) neg += ((u128)a[i] * b[n + k - i]) % p;
    uint64_t s = (uint64_t)(pos % p), d = (uint64_t)(neg % p);
    c[k] = s >= d ? s - d : s + (p - d);
  }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Whole-poly and batch drivers.  A "poly" here is L limbs of N words laid   */
/* out limb-major; limb cm uses prime cm (details/poly.hpp:170-186).         */
/* ------------------------------------------------------------------------ */

/* One reference-style polymul on one limb, as user code writes it:
 * a.forward(); b.forward(); c = a * b; c.backward()  (details/poly.hpp:170-186,
 * ops.hpp:7-24).  a and b are copied so the inputs are left untouched. */
static void polymul_limb(uint64_t* c, const uint64_t* a, const uint64_t* b, uint64_t* tmp,
                         const orc_tables* t) {
  size_t n = (size_t)1 << t->log_n;
  memcpy(c, a, n * sizeof(uint64_t));
  memcpy(tmp, b, n * sizeof(uint64_t));
  forward_t(c, t);
  forward_t(tmp, t);
  for (size_t i = 0; i < n; ++i) c[i] = mulmod(c[i], tmp[i], t->p, t->pn);
  backward_t(c, t);
}

int orc_polymul(uint64_t* c, const uint64_t* a, const uint64_t* b, uint32_t L, uint32_t log_n,
                uint32_t cm0) {
  if (check_args(log_n, cm0) || cm0 + L > ORC_MAX_MODULI) return -1;
  size_t n = (size_t)1 << log_n;
  uint64_t* tmp = (uint64_t*)malloc(n * sizeof(uint64_t));
  for (uint32_t l = 0; l < L; ++l)
    polymul_limb(c + l * n, a + l * n, b + l * n, tmp, tables_get(log_n, cm0 + l));
  free(tmp);
  return 0;
}

/* Multi-threaded batch of polymuls with the same (N, L): pairs are laid out
 * pair-major, then limb-major.  Work units are (pair, limb) and are dealt
 * round-robin to `threads` POSIX threads, since the reference has no internal
 * parallelism and is safe per buffer.  Returns elapsed seconds. */
typedef struct {
  uint64_t *c;
  const uint64_t *a, *b;
  uint32_t pairs, L, log_n, cm0, tid, nthreads;
} polymul_job;

static void* polymul_worker(void* arg) {
  polymul_job* j = (polymul_job*)arg;
  size_t n = (size_t)1 << j->log_n;
  uint64_t* tmp = (uint64_t*)malloc(n * sizeof(uint64_t));
  size_t units = (size_t)j->pairs * j->L;
  for (size_t u = j->tid; u < units; u += j->nthreads) {
    uint32_t l = (uint32_t)(u % j->L);
    polymul_limb(j->c + u * n, j->a + u * n, j->b + u * n, tmp, tables_get(j->log_n, j->cm0 + l));
  }
  free(tmp);
  return NULL;
}

double orc_polymul_batch(uint64_t* c, const uint64_t* a, const uint64_t* b, uint32_t pairs,
                         uint32_t L, uint32_t log_n, uint32_t cm0, uint32_t threads) {
  if (check_args(log_n, cm0) || cm0 + L > ORC_MAX_MODULI || threads == 0) return -1.0;
  for (uint32_t l = 0; l < L; ++l) tables_get(log_n, cm0 + l); /* table warm-up, untimed */
  polymul_job* jobs = (polymul_job*)calloc(threads, sizeof(polymul_job));
  pthread_t* th = (pthread_t*)calloc(threads, sizeof(pthread_t));
  struct timespec t0, t1;
  clock_gettime(CLOCK_MONOTONIC, &t0);
  for (uint32_t i = 0; i < threads; ++i) {
    polymul_job jb = {c, a, b, pairs, L, log_n, cm0, i, threads};
    jobs[i] = jb;
    if (threads == 1) polymul_worker(&jobs[i]);
    else pthread_create(&th[i], NULL, polymul_worker, &jobs[i]);
  }
  if (threads > 1)
    for (uint32_t i = 0; i < threads; ++i) pthread_join(th[i], NULL);
  clock_gettime(CLOCK_MONOTONIC, &t1);
  free(jobs);
  free(th);
  return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}
