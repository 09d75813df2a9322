/*
 * Declarations-only stand-in for <gmp.h> (TEST INFRASTRUCTURE ONLY).
 *
 * The reference's CRT lifting (include/yell/gmp.hpp, lib/gmp.cpp) and its
 * Gaussian sampler include <gmp.h>.  The GMP runtime (libgmp.so.10) is
 * installed in this container but its development header is not, so the
 * harness that runs the reference's own code against the oracle compiles
 * against this file instead.  It declares only what the reference calls,
 * written from the GNU MP manual's descriptions of the integer functions
 * ("Integer Functions"), with the library's exported link names (__gmpz_*)
 * and its documented mpz_t layout.  Nothing here is implemented: every call
 * goes to the installed libgmp.so.10.
 */
#ifndef YELL_ORACLE_SHIM_GMP_H
#define YELL_ORACLE_SHIM_GMP_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef unsigned long mp_limb_t;
typedef unsigned long mp_bitcnt_t;
typedef long mp_size_t;

/* An integer: allocated limbs, signed used-limb count, limb array. */
typedef struct {
  int _mp_alloc;
  int _mp_size;
  mp_limb_t* _mp_d;
} __mpz_struct;

typedef __mpz_struct mpz_t[1];
typedef __mpz_struct* mpz_ptr;
typedef const __mpz_struct* mpz_srcptr;

void __gmpz_init(mpz_ptr);
void __gmpz_init2(mpz_ptr, mp_bitcnt_t);
void __gmpz_inits(mpz_ptr, ...);
void __gmpz_init_set_ui(mpz_ptr, unsigned long);
void __gmpz_clear(mpz_ptr);
void __gmpz_clears(mpz_ptr, ...);
void __gmpz_set(mpz_ptr, mpz_srcptr);
void __gmpz_set_ui(mpz_ptr, unsigned long);
void __gmpz_add(mpz_ptr, mpz_srcptr, mpz_srcptr);
void __gmpz_sub(mpz_ptr, mpz_srcptr, mpz_srcptr);
void __gmpz_mul(mpz_ptr, mpz_srcptr, mpz_srcptr);
void __gmpz_mul_ui(mpz_ptr, mpz_srcptr, unsigned long);
void __gmpz_addmul_ui(mpz_ptr, mpz_srcptr, unsigned long);
void __gmpz_submul(mpz_ptr, mpz_srcptr, mpz_srcptr);
void __gmpz_tdiv_q(mpz_ptr, mpz_srcptr, mpz_srcptr);
void __gmpz_tdiv_q_2exp(mpz_ptr, mpz_srcptr, mp_bitcnt_t);
void __gmpz_divexact(mpz_ptr, mpz_srcptr, mpz_srcptr);
int __gmpz_invert(mpz_ptr, mpz_srcptr, mpz_srcptr);
void __gmpz_ui_pow_ui(mpz_ptr, unsigned long, unsigned long);
int __gmpz_cmp(mpz_srcptr, mpz_srcptr);
size_t __gmpz_sizeinbase(mpz_srcptr, int);
unsigned long __gmpz_get_ui(mpz_srcptr);
void* __gmpz_export(void*, size_t*, int, size_t, int, size_t, mpz_srcptr);

#ifdef __cplusplus
}
#endif

#define mpz_init __gmpz_init
#define mpz_init2 __gmpz_init2
#define mpz_inits __gmpz_inits
#define mpz_init_set_ui __gmpz_init_set_ui
#define mpz_clear __gmpz_clear
#define mpz_clears __gmpz_clears
#define mpz_set __gmpz_set
#define mpz_set_ui __gmpz_set_ui
#define mpz_add __gmpz_add
#define mpz_sub __gmpz_sub
#define mpz_mul __gmpz_mul
#define mpz_mul_ui __gmpz_mul_ui
#define mpz_addmul_ui __gmpz_addmul_ui
#define mpz_submul __gmpz_submul
#define mpz_tdiv_q __gmpz_tdiv_q
#define mpz_tdiv_q_2exp __gmpz_tdiv_q_2exp
#define mpz_divexact __gmpz_divexact
#define mpz_invert __gmpz_invert
#define mpz_ui_pow_ui __gmpz_ui_pow_ui
#define mpz_cmp __gmpz_cmp
#define mpz_sizeinbase __gmpz_sizeinbase
#define mpz_get_ui __gmpz_get_ui
#define mpz_export __gmpz_export

#endif
