/*
 * Declarations-only stand-in for <mpfr.h> (TEST INFRASTRUCTURE ONLY).
 *
 * The reference's FastGaussianNoise (include/yell/prng/FastGaussianNoise.hpp)
 * builds its tables with MPFR.  The runtime (libmpfr.so.6) is installed in
 * this container, its development header is not; the harness that runs the
 * reference's sampler compiles against this file.  It declares only the
 * functions the reference calls, written from the MPFR manual's function
 * descriptions, with the library's exported names and its documented mpfr_t
 * layout (precision, sign, exponent, limb pointer; 64-bit precision and
 * exponent types).  mpfr_init_set_d and mpfr_init_set are the manual's
 * "initialise, then set" combinations.  Every call goes to libmpfr.so.6.
 */
#ifndef YELL_ORACLE_SHIM_MPFR_H
#define YELL_ORACLE_SHIM_MPFR_H

#include "gmp.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef long mpfr_prec_t;
typedef int mpfr_sign_t;
typedef long mpfr_exp_t;

typedef struct {
  mpfr_prec_t _mpfr_prec;
  mpfr_sign_t _mpfr_sign;
  mpfr_exp_t _mpfr_exp;
  mp_limb_t* _mpfr_d;
} __mpfr_struct;

typedef __mpfr_struct mpfr_t[1];
typedef __mpfr_struct* mpfr_ptr;
typedef const __mpfr_struct* mpfr_srcptr;

/* Rounding modes; MPFR_RNDN (to nearest) is the only one the reference uses. */
typedef enum { MPFR_RNDN = 0, MPFR_RNDZ, MPFR_RNDU, MPFR_RNDD, MPFR_RNDA } mpfr_rnd_t;

void mpfr_init(mpfr_ptr);
void mpfr_init2(mpfr_ptr, mpfr_prec_t);
void mpfr_inits2(mpfr_prec_t, mpfr_ptr, ...);
void mpfr_clear(mpfr_ptr);
void mpfr_clears(mpfr_ptr, ...);
void mpfr_free_cache(void);
int mpfr_set(mpfr_ptr, mpfr_srcptr, mpfr_rnd_t);
int mpfr_set_d(mpfr_ptr, double, mpfr_rnd_t);
int mpfr_set_si(mpfr_ptr, long, mpfr_rnd_t);
int mpfr_set_ui(mpfr_ptr, unsigned long, mpfr_rnd_t);
double mpfr_get_d(mpfr_srcptr, mpfr_rnd_t);
int mpfr_get_z(mpz_ptr, mpfr_srcptr, mpfr_rnd_t);
int mpfr_add(mpfr_ptr, mpfr_srcptr, mpfr_srcptr, mpfr_rnd_t);
int mpfr_sub(mpfr_ptr, mpfr_srcptr, mpfr_srcptr, mpfr_rnd_t);
int mpfr_mul(mpfr_ptr, mpfr_srcptr, mpfr_srcptr, mpfr_rnd_t);
int mpfr_sqr(mpfr_ptr, mpfr_srcptr, mpfr_rnd_t);
int mpfr_neg(mpfr_ptr, mpfr_srcptr, mpfr_rnd_t);
int mpfr_exp(mpfr_ptr, mpfr_srcptr, mpfr_rnd_t);
int mpfr_mul_ui(mpfr_ptr, mpfr_srcptr, unsigned long, mpfr_rnd_t);
int mpfr_sub_ui(mpfr_ptr, mpfr_srcptr, unsigned long, mpfr_rnd_t);
int mpfr_ui_div(mpfr_ptr, unsigned long, mpfr_srcptr, mpfr_rnd_t);
int mpfr_pow_ui(mpfr_ptr, mpfr_srcptr, unsigned long, mpfr_rnd_t);

#ifdef __cplusplus
}
#endif

#define mpfr_init_set_d(x, d, rnd) (mpfr_init(x), mpfr_set_d((x), (d), (rnd)))
#define mpfr_init_set(x, y, rnd) (mpfr_init(x), mpfr_set((x), (y), (rnd)))

#endif
