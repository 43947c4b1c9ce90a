/*  gmp.h -- minimal declarations of the GNU MP 6.x public ABI used by this project.

    Neither this container nor the GPU hosts ship GMP's development header; both ship the
    runtime library libgmp.so.10 (GMP 6.x).  This header declares only the documented
    public interface that the project calls: the mpz_t / gmp_randstate_t types (layout per
    the GMP manual, "Integer Internals") and the functions below, bound to the exported
    __gmpz_* / __gmp_* symbol names.  It is used only when the system has no <gmp.h>
    (the build puts this directory on the include path in that case) and is linked with
    -l:libgmp.so.10.
*/
#ifndef MODGCD_GMP_DECL_H
#define MODGCD_GMP_DECL_H

#include <stddef.h>
#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef unsigned long mp_limb_t;   /* 64-bit limbs on LP64 (x86_64 and aarch64) */
typedef long mp_size_t;
typedef unsigned long mp_bitcnt_t;

typedef struct
{
  int _mp_alloc;     /* number of limbs allocated at _mp_d */
  int _mp_size;      /* |_mp_size| limbs in use; the sign of _mp_size is the sign of the value */
  mp_limb_t *_mp_d;  /* least significant limb first */
} __mpz_struct;

typedef __mpz_struct mpz_t[1];
typedef __mpz_struct *mpz_ptr;
typedef const __mpz_struct *mpz_srcptr;

/* Random state: only ever handled through pointers, so it is declared with ample,
   aligned storage rather than its internal fields. */
typedef struct { long long _mp_opaque[8]; } __gmp_randstate_struct;
typedef __gmp_randstate_struct gmp_randstate_t[1];

extern const char *const __gmp_version;
#define gmp_version __gmp_version

void   __gmpz_init(mpz_ptr);
void   __gmpz_init_set_ui(mpz_ptr, unsigned long);
void   __gmpz_clear(mpz_ptr);
void   __gmpz_set(mpz_ptr, mpz_srcptr);
void   __gmpz_set_ui(mpz_ptr, unsigned long);
void   __gmpz_set_si(mpz_ptr, long);
void   __gmpz_swap(mpz_ptr, mpz_ptr);
int    __gmpz_cmp(mpz_srcptr, mpz_srcptr);
int    __gmpz_cmp_ui(mpz_srcptr, unsigned long);
size_t __gmpz_sizeinbase(mpz_srcptr, int);
size_t __gmpz_size(mpz_srcptr);
void  *__gmpz_export(void *, size_t *, int, size_t, int, size_t, mpz_srcptr);
void   __gmpz_import(mpz_ptr, size_t, int, size_t, int, size_t, const void *);
void   __gmpz_add(mpz_ptr, mpz_srcptr, mpz_srcptr);
void   __gmpz_add_ui(mpz_ptr, mpz_srcptr, unsigned long);
void   __gmpz_sub(mpz_ptr, mpz_srcptr, mpz_srcptr);
void   __gmpz_sub_ui(mpz_ptr, mpz_srcptr, unsigned long);
void   __gmpz_mul(mpz_ptr, mpz_srcptr, mpz_srcptr);
void   __gmpz_mul_ui(mpz_ptr, mpz_srcptr, unsigned long);
void   __gmpz_mul_2exp(mpz_ptr, mpz_srcptr, mp_bitcnt_t);
void   __gmpz_pow_ui(mpz_ptr, mpz_srcptr, unsigned long);
void   __gmpz_abs(mpz_ptr, mpz_srcptr);
void   __gmpz_neg(mpz_ptr, mpz_srcptr);
void   __gmpz_gcd(mpz_ptr, mpz_srcptr, mpz_srcptr);
unsigned long __gmpz_fdiv_q_ui(mpz_ptr, mpz_srcptr, unsigned long);
void   __gmpz_cdiv_q(mpz_ptr, mpz_srcptr, mpz_srcptr);
void   __gmpz_tdiv_r(mpz_ptr, mpz_srcptr, mpz_srcptr);
void   __gmpz_urandomb(mpz_ptr, __gmp_randstate_struct *, mp_bitcnt_t);
char  *__gmpz_get_str(char *, int, mpz_srcptr);
int    __gmpz_set_str(mpz_ptr, const char *, int);
size_t __gmpz_out_str(FILE *, int, mpz_srcptr);
size_t __gmpz_inp_str(mpz_ptr, FILE *, int);
void   __gmp_randinit_mt(__gmp_randstate_struct *);
void   __gmp_randseed_ui(__gmp_randstate_struct *, unsigned long);
void   __gmp_randclear(__gmp_randstate_struct *);

#define mpz_init        __gmpz_init
#define mpz_init_set_ui __gmpz_init_set_ui
#define mpz_clear       __gmpz_clear
#define mpz_set         __gmpz_set
#define mpz_set_ui      __gmpz_set_ui
#define mpz_set_si      __gmpz_set_si
#define mpz_swap        __gmpz_swap
#define mpz_cmp         __gmpz_cmp
#define mpz_cmp_ui      __gmpz_cmp_ui
#define mpz_sizeinbase  __gmpz_sizeinbase
#define mpz_size        __gmpz_size
#define mpz_export      __gmpz_export
#define mpz_import      __gmpz_import
#define mpz_add         __gmpz_add
#define mpz_add_ui      __gmpz_add_ui
#define mpz_sub         __gmpz_sub
#define mpz_sub_ui      __gmpz_sub_ui
#define mpz_mul         __gmpz_mul
#define mpz_mul_ui      __gmpz_mul_ui
#define mpz_mul_2exp    __gmpz_mul_2exp
#define mpz_pow_ui      __gmpz_pow_ui
#define mpz_abs         __gmpz_abs
#define mpz_neg         __gmpz_neg
#define mpz_gcd         __gmpz_gcd
#define mpz_fdiv_q_ui   __gmpz_fdiv_q_ui
#define mpz_cdiv_q      __gmpz_cdiv_q
#define mpz_tdiv_r      __gmpz_tdiv_r
#define mpz_urandomb    __gmpz_urandomb
#define mpz_get_str     __gmpz_get_str
#define mpz_set_str     __gmpz_set_str
#define mpz_out_str     __gmpz_out_str
#define mpz_inp_str     __gmpz_inp_str
#define gmp_randinit_mt __gmp_randinit_mt
#define gmp_randseed_ui __gmp_randseed_ui
#define gmp_randclear   __gmp_randclear

/* Sign of an mpz, read from the documented _mp_size field. */
#define mpz_sgn(z) ((z)->_mp_size < 0 ? -1 : (z)->_mp_size > 0)

#ifdef __cplusplus
}
#endif

#endif /* MODGCD_GMP_DECL_H */
