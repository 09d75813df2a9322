/*
 * CPU oracle for the 32-bit moduli mode of the YELL hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the parity tests load it as the checker; no
 * product code calls, links or falls back to it.
 *
 * The reference selects this mode at compile time (-DYELL_USE_32BITS_MODULI,
 * include/yell/params.hpp:2-6): words are uint32, products uint64, and the
 * same generic code runs with bit_width 32.  Restated here:
 *   - prime table  : include/yell/params_32.hpp:15-34 (291 primes
 *                    p = 2^30 - j*2^16 + 1 for increasing j, kept when prime;
 *                    Pn = low 32 bits of floor(2^64/p); primitive_roots[cm] =
 *                    g^((p-1)/2^16) for g the least primitive root; all three
 *                    regenerated here and checked against the reference build)
 *   - Barrett      : lib/ops.cpp:5-21 with shift 32, delta 2
 *   - shoupify     : lib/ops.cpp:23-27, floor(x * 2^32 / p)
 *   - twiddles     : include/yell/details/ntt.hpp:28-77 (kMaxPolyDegree 2^15)
 *   - butterflies and lazy loops : lib/ntt.cpp:34-210 at 32-bit words
 *   - forward / forward_lazy / backward : include/yell/details/ntt.hpp:107-166
 *   - ops functors : include/yell/ops.hpp:46-158
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define O32_MAX_MODULI 291u  /* params_32.hpp kMaxNbModuli  */
#define O32_LOG_MAX_DEGREE 15u /* kMaxPolyDegree = 2^15 */

static uint32_t o32_P[O32_MAX_MODULI], o32_Pn[O32_MAX_MODULI], o32_root[O32_MAX_MODULI];
static pthread_once_t o32_once = PTHREAD_ONCE_INIT;

static uint32_t pow_u64(uint64_t b, uint64_t e, uint32_t m) {
  uint64_t r = 1 % m;
  b %= m;
  while (e) {
    if (e & 1) r = r * b % m;
    b = b * b % m;
    e >>= 1;
  }
  return (uint32_t)r;
}

/* Deterministic Miller-Rabin for n < 2^32 (bases 2, 7, 61). */
static int is_prime_u32(uint32_t n) {
  static const uint32_t bases[3] = {2, 7, 61};
  if (n < 2) return 0;
  for (int i = 0; i < 3; ++i) {
    if (n == bases[i]) return 1;
    if (n % bases[i] == 0) return 0;
  }
  uint32_t d = n - 1;
  int s = 0;
  while ((d & 1) == 0) { d >>= 1; ++s; }
  for (int i = 0; i < 3; ++i) {
    uint64_t x = pow_u64(bases[i], d, n);
    if (x == 1 || x == n - 1) continue;
    int comp = 1;
    for (int r = 1; r < s; ++r) {
      x = x * x % n;
      if (x == n - 1) { comp = 0; break; }
    }
    if (comp) return 0;
  }
  return 1;
}

static uint32_t least_primitive_root(uint32_t p) {
  uint32_t f[32];
  int nf = 0;
  uint32_t m = p - 1;
  for (uint32_t q = 2; q * q <= m; ++q)
    if (m % q == 0) {
      f[nf++] = q;
      while (m % q == 0) m /= q;
    }
  if (m > 1) f[nf++] = m;
  for (uint32_t g = 2;; ++g) {
    int ok = 1;
    for (int i = 0; i < nf && ok; ++i)
      if (pow_u64(g, (p - 1) / f[i], p) == 1) ok = 0;
    if (ok) return g;
  }
}

static void o32_init(void) {
  uint32_t k = 0;
  for (uint32_t j = 1; k < O32_MAX_MODULI; ++j) {
    const uint32_t p = (1u << 30) - j * (1u << 16) + 1;
    if (!is_prime_u32(p)) continue;
    o32_P[k] = p;
    o32_Pn[k] = (uint32_t)(~0ull / p); /* low word of floor(2^64 / p): p odd */
    o32_root[k] = pow_u64(least_primitive_root(p), (p - 1) >> 16, p);
    ++k;
  }
}

uint32_t orc32_prime(uint32_t cm) {
  pthread_once(&o32_once, o32_init);
  return cm < O32_MAX_MODULI ? o32_P[cm] : 0;
}
uint32_t orc32_pn(uint32_t cm) {
  pthread_once(&o32_once, o32_init);
  return cm < O32_MAX_MODULI ? o32_Pn[cm] : 0;
}
uint32_t orc32_primitive_root(uint32_t cm) {
  pthread_once(&o32_once, o32_init);
  return cm < O32_MAX_MODULI ? o32_root[cm] : 0;
}
uint32_t orc32_max_moduli(void) { return O32_MAX_MODULI; }

/* lib/ops.cpp:5-21 at shift 32, delta 2. */
static uint32_t barrett32(uint64_t x, uint32_t p, uint32_t pn) {
  const uint64_t q = (uint64_t)pn * (x >> 32) + (x << 2);
  uint32_t r = (uint32_t)x - (uint32_t)(q >> 32) * p;
  if (r >= p) r -= p;
  return r;
}
static uint32_t shoupify32(uint32_t x, uint32_t p) { return (uint32_t)(((uint64_t)x << 32) / p); }
static uint32_t mulmod32(uint32_t x, uint32_t y, uint32_t p, uint32_t pn) { return barrett32((uint64_t)x * y, p, pn); }
static uint32_t mulmod_shoup32(uint32_t x, uint32_t y, uint32_t yp, uint32_t p) {
  const uint32_t q = (uint32_t)(((uint64_t)x * yp) >> 32) * p;
  uint32_t r = x * y - q;
  if (r >= p) r -= p;
  return r;
}

uint32_t orc32_barrett(uint64_t x, uint32_t cm) { return barrett32(x, orc32_prime(cm), orc32_pn(cm)); }
uint32_t orc32_shoupify(uint32_t x, uint32_t cm) { return shoupify32(x, orc32_prime(cm)); }

void orc32_mulmod_n(uint32_t* d, const uint32_t* a, const uint32_t* b, size_t n, uint32_t cm) {
  const uint32_t p = orc32_prime(cm), pn = orc32_pn(cm);
  for (size_t i = 0; i < n; ++i) d[i] = mulmod32(a[i], b[i], p, pn);
}
void orc32_addmod_n(uint32_t* d, const uint32_t* a, const uint32_t* b, size_t n, uint32_t cm) {
  const uint32_t p = orc32_prime(cm);
  for (size_t i = 0; i < n; ++i) {
    uint32_t x = a[i] + b[i];
    d[i] = x >= p ? x - p : x;
  }
}
void orc32_submod_n(uint32_t* d, const uint32_t* a, const uint32_t* b, size_t n, uint32_t cm) {
  const uint32_t p = orc32_prime(cm);
  for (size_t i = 0; i < n; ++i) {
    uint32_t x = a[i] + (p - b[i]);
    d[i] = x >= p ? x - p : x;
  }
}
void orc32_muladd_n(uint32_t* rop, const uint32_t* a, const uint32_t* b, size_t n, uint32_t cm) {
  const uint32_t p = orc32_prime(cm), pn = orc32_pn(cm);
  for (size_t i = 0; i < n; ++i) rop[i] = barrett32((uint64_t)a[i] * b[i] + rop[i], p, pn);
}
void orc32_negate_n(uint32_t* x, size_t n, uint32_t cm) {
  const uint32_t p = orc32_prime(cm);
  for (size_t i = 0; i < n; ++i) x[i] = p - x[i];
}
void orc32_mulmod_shoup_n(uint32_t* d, const uint32_t* a, uint32_t y, size_t n, uint32_t cm) {
  const uint32_t p = orc32_prime(cm), yp = shoupify32(y, p);
  for (size_t i = 0; i < n; ++i) d[i] = mulmod_shoup32(a[i], y, yp, p);
}

static void revbin32(uint32_t* a, size_t n) {
  if (n <= 2) return;
  for (size_t i = 1, j = 0; i < n; ++i) {
    size_t bit = n >> 1;
    for (; j >= bit; bit >>= 1) j -= bit;
    j += bit;
    if (i < j) { uint32_t t = a[i]; a[i] = a[j]; a[j] = t; }
  }
}

typedef struct {
  uint32_t log_n, p, pn;
  uint32_t *phi, *phi_s, *iphi, *iphi_s;
  uint32_t inv_n, inv_n_s, inv_n_iphi, inv_n_iphi_s;
} o32_tables;

/* details/ntt.hpp:28-77 */
static void tables32_build(o32_tables* t, uint32_t log_n, uint32_t cm) {
  const size_t n = (size_t)1 << log_n;
  const uint32_t p = orc32_prime(cm), pn = orc32_pn(cm);
  t->log_n = log_n;
  t->p = p;
  t->pn = pn;
  t->phi = (uint32_t*)malloc(4 * n * sizeof(uint32_t));
  t->phi_s = t->phi + n;
  t->iphi = t->phi + 2 * n;
  t->iphi_s = t->phi + 3 * n;
  uint32_t phi = orc32_primitive_root(cm);
  for (uint32_t i = 0; i < O32_LOG_MAX_DEGREE - log_n; ++i) phi = mulmod32(phi, phi, p, pn);
  uint32_t temp = 1;
  for (size_t i = 0; i < n; ++i) {
    t->phi[i] = temp;
    t->phi_s[i] = shoupify32(temp, p);
    temp = mulmod32(temp, phi, p, pn);
  }
  const uint32_t invphi = mulmod32(temp, t->phi[n - 1], p, pn);
  temp = 1;
  for (size_t i = 0; i < n; ++i) {
    t->iphi[i] = temp;
    t->iphi_s[i] = shoupify32(temp, p);
    temp = mulmod32(temp, invphi, p, pn);
  }
  revbin32(t->phi, n);
  revbin32(t->phi_s, n);
  revbin32(t->iphi, n);
  revbin32(t->iphi_s, n);
  /* math::inv_mod_prime: Fermat with Barrett mulmod */
  uint32_t a = (uint32_t)n, inv = 1, y = p - 2;
  while (y > 0) {
    if (y & 1) inv = mulmod32(inv, a, p, pn);
    y >>= 1;
    a = mulmod32(a, a, p, pn);
  }
  t->inv_n = inv;
  t->inv_n_iphi = mulmod32(inv, t->iphi[1], p, pn);
  t->inv_n_s = shoupify32(t->inv_n, p);
  t->inv_n_iphi_s = shoupify32(t->inv_n_iphi, p);
}

int orc32_ntt_tables(uint32_t log_n, uint32_t cm, uint32_t* out4n, uint32_t* scalars) {
  if (log_n < 1 || log_n > O32_LOG_MAX_DEGREE || cm >= O32_MAX_MODULI) return -1;
  o32_tables t;
  tables32_build(&t, log_n, cm);
  memcpy(out4n, t.phi, 4 * ((size_t)1 << log_n) * sizeof(uint32_t));
  scalars[0] = t.inv_n;
  scalars[1] = t.inv_n_s;
  scalars[2] = t.inv_n_iphi;
  scalars[3] = t.inv_n_iphi_s;
  free(t.phi);
  return 0;
}

/* lib/ntt.cpp:69-83 and 47-63 at 32-bit words */
static inline void ct32(uint32_t* x0, uint32_t* x1, uint32_t w, uint32_t wp, uint32_t p, uint32_t p2) {
  uint32_t u0 = *x0, u1 = *x1;
  if (u0 >= p2) u0 -= p2;
  const uint32_t q = (uint32_t)(((uint64_t)u1 * wp) >> 32);
  const uint32_t t = u1 * w - q * p;
  *x0 = u0 + t;
  *x1 = u0 - t + p2;
}
static inline void gs32(uint32_t* x0, uint32_t* x1, uint32_t w, uint32_t wp, uint32_t p, uint32_t p2) {
  const uint32_t u0 = *x0, u1 = *x1;
  uint32_t t0 = u0 + u1;
  if (t0 >= p2) t0 -= p2;
  const uint32_t t1 = u0 - u1 + p2;
  const uint32_t q = (uint32_t)(((uint64_t)t1 * wp) >> 32);
  *x0 = t0;
  *x1 = t1 * w - q * p;
}

static void fwd_lazy32(uint32_t* x, const o32_tables* t) {
  const size_t n = (size_t)1 << t->log_n;
  const uint32_t p = t->p, p2 = p << 1;
  for (size_t m = 1, h = n >> 1; h >= 1; m <<= 1, h >>= 1)
    for (size_t r = 0; r < m; ++r) {
      uint32_t* x0 = x + 2 * h * r;
      for (size_t i = 0; i < h; ++i) ct32(x0 + i, x0 + i + h, t->phi[m + r], t->phi_s[m + r], p, p2);
    }
}

/* lib/ntt.cpp:151-210 (first two layers unconditional, then while m > 1) */
static void bwd_lazy32(uint32_t* x, const o32_tables* t) {
  const size_t n = (size_t)1 << t->log_n;
  const uint32_t p = t->p, p2 = p << 1;
  const uint32_t *w = t->iphi, *ws = t->iphi_s;
  size_t m = n >> 1, h = 1;
  for (size_t r = 0; r < m; ++r) gs32(x + 2 * r, x + 2 * r + 1, w[m + r], ws[m + r], p, p2);
  m >>= 1;
  h <<= 1;
  for (size_t r = 0; r < m; ++r) {
    gs32(x + 4 * r, x + 4 * r + 2, w[m + r], ws[m + r], p, p2);
    gs32(x + 4 * r + 1, x + 4 * r + 3, w[m + r], ws[m + r], p, p2);
  }
  m >>= 1;
  h <<= 1;
  for (; m > 1; m >>= 1, h <<= 1)
    for (size_t r = 0; r < m; ++r) {
      uint32_t* x0 = x + 2 * h * r;
      for (size_t i = 0; i < h; ++i) gs32(x0 + i, x0 + i + h, w[m + r], ws[m + r], p, p2);
    }
}

static void fwd32(uint32_t* x, const o32_tables* t) {
  const size_t n = (size_t)1 << t->log_n;
  const uint32_t p = t->p, p2 = p << 1;
  fwd_lazy32(x, t);
  for (size_t i = 0; i < n; ++i) {
    uint32_t v = x[i];
    if (v >= p2) v -= p2;
    if (v >= p) v -= p;
    x[i] = v;
  }
}

static void bwd32(uint32_t* x, const o32_tables* t) {
  const size_t n = (size_t)1 << t->log_n;
  const uint32_t p = t->p, p2 = p << 1;
  bwd_lazy32(x, t);
  for (size_t i = 0; i < n / 2; ++i) {
    const uint32_t u = x[i], v = x[i + n / 2];
    x[i] = mulmod_shoup32(u + v, t->inv_n, t->inv_n_s, p);
    x[i + n / 2] = mulmod_shoup32(u - v + p2, t->inv_n_iphi, t->inv_n_iphi_s, p);
  }
}

static o32_tables* o32_cache[O32_LOG_MAX_DEGREE + 1][O32_MAX_MODULI];
static pthread_mutex_t o32_mu = PTHREAD_MUTEX_INITIALIZER;

static const o32_tables* tables32_get(uint32_t log_n, uint32_t cm) {
  pthread_mutex_lock(&o32_mu);
  o32_tables* t = o32_cache[log_n][cm];
  if (!t) {
    t = (o32_tables*)malloc(sizeof(o32_tables));
    tables32_build(t, log_n, cm);
    o32_cache[log_n][cm] = t;
  }
  pthread_mutex_unlock(&o32_mu);
  return t;
}

static int bad32(uint32_t log_n, uint32_t cm) {
  return !(log_n >= 2 && log_n <= O32_LOG_MAX_DEGREE && cm < O32_MAX_MODULI);
}

int orc32_forward(uint32_t* x, uint32_t log_n, uint32_t cm) {
  if (bad32(log_n, cm)) return -1;
  fwd32(x, tables32_get(log_n, cm));
  return 0;
}
int orc32_forward_lazy(uint32_t* x, uint32_t log_n, uint32_t cm) {
  if (bad32(log_n, cm)) return -1;
  fwd_lazy32(x, tables32_get(log_n, cm));
  return 0;
}
int orc32_backward(uint32_t* x, uint32_t log_n, uint32_t cm) {
  if (bad32(log_n, cm)) return -1;
  bwd32(x, tables32_get(log_n, cm));
  return 0;
}

/* a.forward(); b.forward(); c = a * b; c.backward() per limb, limb l under cm0 + l */
int orc32_polymul(uint32_t* c, const uint32_t* a, const uint32_t* b, uint32_t L, uint32_t log_n, uint32_t cm0) {
  if (bad32(log_n, cm0) || cm0 + L > O32_MAX_MODULI) return -1;
  const size_t n = (size_t)1 << log_n;
  uint32_t* tmp = (uint32_t*)malloc(n * sizeof(uint32_t));
  for (uint32_t l = 0; l < L; ++l) {
    const o32_tables* t = tables32_get(log_n, cm0 + l);
    memcpy(c + l * n, a + l * n, n * 4);
    memcpy(tmp, b + l * n, n * 4);
    fwd32(c + l * n, t);
    fwd32(tmp, t);
    for (size_t i = 0; i < n; ++i) c[l * n + i] = mulmod32(c[l * n + i], tmp[i], t->p, t->pn);
    bwd32(c + l * n, t);
  }
  free(tmp);
  return 0;
}
