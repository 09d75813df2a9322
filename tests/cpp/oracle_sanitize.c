/* Drives every oracle entry point (64-bit, 32-bit, samplers) on edge sizes
 * and edge values; built with AddressSanitizer and UndefinedBehaviorSanitizer
 * by tests/test_cpu_sanitizers.py, so any out-of-bounds access, overflow of a
 * signed type or misaligned access in the oracle aborts the run.  Prints OK. */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

uint64_t orc_prime(uint32_t cm);
int orc_ntt_tables(uint32_t log_n, uint32_t cm, uint64_t* out4n, uint64_t* scalars);
int orc_forward(uint64_t* x, uint32_t log_n, uint32_t cm);
int orc_forward_lazy(uint64_t* x, uint32_t log_n, uint32_t cm);
int orc_backward(uint64_t* x, uint32_t log_n, uint32_t cm);
int orc_negacyclic_forward_lazy(uint64_t* x, uint64_t degree, const uint64_t* w, const uint64_t* ws, uint64_t p);
int orc_negacyclic_backward_lazy(uint64_t* x, uint64_t degree, const uint64_t* w, const uint64_t* ws, uint64_t p);
int orc_negacyclic_schoolbook(uint64_t* c, const uint64_t* a, const uint64_t* b, uint32_t log_n, uint32_t cm);
int orc_polymul(uint64_t* c, const uint64_t* a, const uint64_t* b, uint32_t L, uint32_t log_n, uint32_t cm0);
double orc_polymul_batch(uint64_t* c, const uint64_t* a, const uint64_t* b, uint32_t pairs, uint32_t L,
                         uint32_t log_n, uint32_t cm0, uint32_t threads);
void orc_mulmod_n(uint64_t* dst, const uint64_t* a, const uint64_t* b, size_t n, uint32_t cm);
void orc_addmod_n(uint64_t* dst, const uint64_t* a, const uint64_t* b, size_t n, uint32_t cm);
void orc_submod_n(uint64_t* dst, const uint64_t* a, const uint64_t* b, size_t n, uint32_t cm);
void orc_muladd_n(uint64_t* rop, const uint64_t* a, const uint64_t* b, size_t n, uint32_t cm);
void orc_negate_n(uint64_t* x, size_t n, uint32_t cm);
void orc_mulmod_shoup_n(uint64_t* dst, const uint64_t* a, uint64_t y, size_t n, uint32_t cm);
void orc_sample_uniform(uint64_t* out, uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0, uint64_t seed);
void orc_sample_zo(uint64_t* out, uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0, uint32_t rho,
                   uint64_t seed);
int orc_sample_hwt(uint64_t* out, uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0, uint32_t h,
                   uint64_t seed);
uint32_t orc_gaussian_cdt(double sigma, uint32_t tail, uint64_t* out);
void orc_sample_gaussian(uint64_t* out, uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0,
                         const uint64_t* cdt, uint32_t len, uint32_t tail, uint64_t amplifier, uint64_t seed);
uint32_t orc32_prime(uint32_t cm);
int orc32_forward(uint32_t* x, uint32_t log_n, uint32_t cm);
int orc32_forward_lazy(uint32_t* x, uint32_t log_n, uint32_t cm);
int orc32_backward(uint32_t* x, uint32_t log_n, uint32_t cm);
int orc32_polymul(uint32_t* c, const uint32_t* a, const uint32_t* b, uint32_t L, uint32_t log_n, uint32_t cm0);
void orc32_mulmod_n(uint32_t* d, const uint32_t* a, const uint32_t* b, size_t n, uint32_t cm);
void orc32_addmod_n(uint32_t* d, const uint32_t* a, const uint32_t* b, size_t n, uint32_t cm);
void orc32_submod_n(uint32_t* d, const uint32_t* a, const uint32_t* b, size_t n, uint32_t cm);
void orc32_muladd_n(uint32_t* rop, const uint32_t* a, const uint32_t* b, size_t n, uint32_t cm);
void orc32_negate_n(uint32_t* x, size_t n, uint32_t cm);

static uint64_t state = 0x1234567887654321ull;
static uint64_t next(void) {
  uint64_t z = (state += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static void fill(uint64_t* x, size_t n, uint64_t bound) {
  for (size_t i = 0; i < n; ++i) x[i] = bound ? next() % bound : next();
}
static int fail(const char* what, unsigned a) {
  printf("FAIL %s %u\n", what, a);
  return 1;
}

int main(void) {
  const uint32_t cms[3] = {0, 17, 999};
  /* 64-bit transforms at every degree up to 2^16, round trip through [0, p) */
  for (uint32_t log_n = 2; log_n <= 16; ++log_n) {
    const size_t n = (size_t)1 << log_n;
    uint64_t* x = malloc(n * 8);
    uint64_t* y = malloc(n * 8);
    for (int k = 0; k < 3; ++k) {
      const uint64_t p = orc_prime(cms[k]);
      fill(x, n, p);
      memcpy(y, x, n * 8);
      if (orc_forward(y, log_n, cms[k]) || orc_backward(y, log_n, cms[k])) return fail("forward/backward", log_n);
      if (log_n > 2 && memcmp(x, y, n * 8)) return fail("round trip", log_n);
      fill(y, n, 4 * p);
      if (orc_forward_lazy(y, log_n, cms[k])) return fail("forward_lazy", log_n);
      for (size_t i = 0; i < n; ++i) y[i] = 4 * p - 1;  /* top of the lazy range */
      if (orc_forward_lazy(y, log_n, cms[k])) return fail("forward_lazy edge", log_n);
    }
    free(x);
    free(y);
  }
  /* the runtime-N free functions with the reference's tables */
  for (uint32_t log_n = 2; log_n <= 12; log_n += 5) {
    const size_t n = (size_t)1 << log_n;
    uint64_t* t = malloc(4 * n * 8);
    uint64_t sc[4];
    uint64_t* x = malloc(n * 8);
    if (orc_ntt_tables(log_n, 3, t, sc)) return fail("tables", log_n);
    const uint64_t p = orc_prime(3);
    fill(x, n, 4 * p);
    if (orc_negacyclic_forward_lazy(x, n, t, t + n, p)) return fail("free forward", log_n);
    for (size_t i = 0; i < n; ++i) x[i] %= 2 * p;
    if (orc_negacyclic_backward_lazy(x, n, t + 2 * n, t + 3 * n, p)) return fail("free backward", log_n);
    free(t);
    free(x);
  }
  /* polymul against the schoolbook product, batch with threads */
  {
    const uint32_t log_n = 9, L = 3, pairs = 3;
    const size_t n = (size_t)1 << log_n, w = (size_t)L * n;
    uint64_t* a = malloc(pairs * w * 8);
    uint64_t* b = malloc(pairs * w * 8);
    uint64_t* c = malloc(pairs * w * 8);
    uint64_t* s = malloc(n * 8);
    for (uint32_t l = 0; l < pairs * L; ++l) {
      fill(a + l * n, n, orc_prime(l % L));
      fill(b + l * n, n, orc_prime(l % L));
    }
    if (orc_polymul(c, a, b, L, log_n, 0)) return fail("polymul", log_n);
    if (orc_negacyclic_schoolbook(s, a, b, log_n, 0) || memcmp(s, c, n * 8)) return fail("schoolbook", log_n);
    if (orc_polymul_batch(c, a, b, pairs, L, log_n, 0, 2) < 0) return fail("polymul_batch", log_n);
    free(a);
    free(b);
    free(c);
    free(s);
  }
  /* element-wise ops on full-range words, odd lengths */
  {
    const size_t n = 513;
    uint64_t *a = malloc(n * 8), *b = malloc(n * 8), *d = malloc(n * 8);
    fill(a, n, 0);
    fill(b, n, 0);
    fill(d, n, 0);
    orc_mulmod_n(d, a, b, n, 999);
    orc_addmod_n(d, a, b, n, 0);
    orc_submod_n(d, a, b, n, 5);
    orc_muladd_n(d, a, b, n, 7);
    orc_negate_n(d, n, 11);
    orc_mulmod_shoup_n(d, a, orc_prime(2) - 1, n, 2);
    free(a);
    free(b);
    free(d);
  }
  /* samplers, smallest and a mid degree */
  for (uint32_t log_n = 3; log_n <= 10; log_n += 7) {
    const uint32_t count = 2, L = 3;
    const size_t n = (size_t)1 << log_n;
    uint64_t* out = malloc(count * L * n * 8);
    uint64_t cdt[2 * 64 + 1];
    orc_sample_uniform(out, count, L, log_n, 997, 5);
    orc_sample_zo(out, count, L, log_n, 0, 255, 6);
    orc_sample_zo(out, count, L, log_n, 0, 0, 6);
    if (orc_sample_hwt(out, count, L, log_n, 0, 1, 7) || orc_sample_hwt(out, count, L, log_n, 0, (uint32_t)n, 7))
      return fail("hwt", log_n);
    const uint32_t len = orc_gaussian_cdt(3.2, 19, cdt);
    orc_sample_gaussian(out, count, L, log_n, 0, cdt, len, 19, 1, 8);
    free(out);
  }
  /* 32-bit mode */
  for (uint32_t log_n = 3; log_n <= 15; ++log_n) {
    const size_t n = (size_t)1 << log_n;
    uint32_t *x = malloc(n * 4), *y = malloc(n * 4), *c = malloc(n * 4);
    const uint32_t p = orc32_prime(290);
    for (size_t i = 0; i < n; ++i) x[i] = (uint32_t)(next() % p);
    memcpy(y, x, n * 4);
    if (orc32_forward(y, log_n, 290) || orc32_backward(y, log_n, 290) || memcmp(x, y, n * 4))
      return fail("32-bit round trip", log_n);
    for (size_t i = 0; i < n; ++i) y[i] = 4 * p - 1;
    if (orc32_forward_lazy(y, log_n, 290)) return fail("32-bit forward_lazy", log_n);
    if (orc32_polymul(c, x, x, 1, log_n, 290)) return fail("32-bit polymul", log_n);
    orc32_mulmod_n(c, x, x, n, 290);
    orc32_addmod_n(c, x, x, n, 290);
    orc32_submod_n(c, x, x, n, 290);
    orc32_muladd_n(c, x, x, n, 290);
    orc32_negate_n(c, n, 290);
    free(x);
    free(y);
    free(c);
  }
  /* invalid arguments are refused, not read past */
  {
    uint64_t x[8] = {0};
    if (orc_forward(x, 21, 0) != -1 || orc_forward(x, 3, 1000) != -1) return fail("invalid 64-bit", 0);
    uint32_t z[8] = {0};
    if (orc32_forward(z, 16, 0) != -1 || orc32_forward(z, 3, 291) != -1) return fail("invalid 32-bit", 0);
  }
  printf("OK\n");
  return 0;
}
