/* Declarations of the documented GMP 6.x API subset (LP64 ABI) used by the
 * host-side reference-orbit builder. Build images ship libgmp.so.10 without
 * development headers, so the library declares the entry points it needs and
 * links the runtime library by path. */
#ifndef MBX_GMP_ABI_H
#define MBX_GMP_ABI_H
#include <stddef.h>
#include <stdio.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef unsigned long int mp_limb_t;
typedef long int mp_limb_signed_t;
typedef unsigned long int mp_bitcnt_t;
typedef long int mp_size_t;
typedef long int mp_exp_t;
typedef mp_limb_t* mp_ptr;
typedef const mp_limb_t* mp_srcptr;
typedef struct { int _mp_alloc; int _mp_size; mp_limb_t* _mp_d; } __mpz_struct;
typedef __mpz_struct mpz_t[1];
typedef __mpz_struct* mpz_ptr;
typedef const __mpz_struct* mpz_srcptr;
typedef struct { int _mp_prec; int _mp_size; mp_exp_t _mp_exp; mp_limb_t* _mp_d; } __mpf_struct;
typedef __mpf_struct mpf_t[1];
typedef __mpf_struct* mpf_ptr;
typedef const __mpf_struct* mpf_srcptr;

#define mpf_sgn(F) ((F)->_mp_size < 0 ? -1 : (F)->_mp_size > 0)

void __gmpf_init(mpf_ptr);
void __gmpf_init2(mpf_ptr, mp_bitcnt_t);
void __gmpf_inits(mpf_ptr, ...);
void __gmpf_clear(mpf_ptr);
void __gmpf_clears(mpf_ptr, ...);
void __gmpf_set(mpf_ptr, mpf_srcptr);
void __gmpf_set_ui(mpf_ptr, unsigned long int);
void __gmpf_set_si(mpf_ptr, long int);
void __gmpf_set_d(mpf_ptr, double);
void __gmpf_set_z(mpf_ptr, mpz_srcptr);
int __gmpf_set_str(mpf_ptr, const char*, int);
void __gmpf_init_set(mpf_ptr, mpf_srcptr);
void __gmpf_init_set_ui(mpf_ptr, unsigned long int);
void __gmpf_init_set_d(mpf_ptr, double);
int __gmpf_init_set_str(mpf_ptr, const char*, int);
void __gmpf_set_prec(mpf_ptr, mp_bitcnt_t);
void __gmpf_set_default_prec(mp_bitcnt_t);
mp_bitcnt_t __gmpf_get_prec(mpf_srcptr);
mp_bitcnt_t __gmpf_get_default_prec(void);
void __gmpf_add(mpf_ptr, mpf_srcptr, mpf_srcptr);
void __gmpf_add_ui(mpf_ptr, mpf_srcptr, unsigned long int);
void __gmpf_sub(mpf_ptr, mpf_srcptr, mpf_srcptr);
void __gmpf_sub_ui(mpf_ptr, mpf_srcptr, unsigned long int);
void __gmpf_mul(mpf_ptr, mpf_srcptr, mpf_srcptr);
void __gmpf_mul_ui(mpf_ptr, mpf_srcptr, unsigned long int);
void __gmpf_mul_2exp(mpf_ptr, mpf_srcptr, mp_bitcnt_t);
void __gmpf_div(mpf_ptr, mpf_srcptr, mpf_srcptr);
void __gmpf_div_ui(mpf_ptr, mpf_srcptr, unsigned long int);
void __gmpf_div_2exp(mpf_ptr, mpf_srcptr, mp_bitcnt_t);
void __gmpf_sqrt(mpf_ptr, mpf_srcptr);
void __gmpf_neg(mpf_ptr, mpf_srcptr);
void __gmpf_abs(mpf_ptr, mpf_srcptr);
int __gmpf_cmp(mpf_srcptr, mpf_srcptr);
int __gmpf_cmp_d(mpf_srcptr, double);
int __gmpf_cmp_ui(mpf_srcptr, unsigned long int);
int __gmpf_cmp_si(mpf_srcptr, long int);
double __gmpf_get_d(mpf_srcptr);
double __gmpf_get_d_2exp(long int*, mpf_srcptr);
char* __gmpf_get_str(char*, mp_exp_t*, int, size_t, mpf_srcptr);
void __gmpz_init(mpz_ptr);
void __gmpz_clear(mpz_ptr);
void __gmpz_set_f(mpz_ptr, mpf_srcptr);
void __gmpz_import(mpz_ptr, size_t, int, size_t, int, size_t, const void*);
void* __gmpz_export(void*, size_t*, int, size_t, int, size_t, mpz_srcptr);
void __gmpn_mul_n(mp_ptr, mp_srcptr, mp_srcptr, mp_size_t);
void __gmpn_sqr(mp_ptr, mp_srcptr, mp_size_t);
mp_limb_t __gmpn_addmul_1(mp_ptr, mp_srcptr, mp_size_t, mp_limb_t);

#define mpf_init __gmpf_init
#define mpf_init2 __gmpf_init2
#define mpf_inits __gmpf_inits
#define mpf_clear __gmpf_clear
#define mpf_clears __gmpf_clears
#define mpf_set __gmpf_set
#define mpf_set_ui __gmpf_set_ui
#define mpf_set_si __gmpf_set_si
#define mpf_set_d __gmpf_set_d
#define mpf_set_z __gmpf_set_z
#define mpf_set_str __gmpf_set_str
#define mpf_init_set __gmpf_init_set
#define mpf_init_set_ui __gmpf_init_set_ui
#define mpf_init_set_d __gmpf_init_set_d
#define mpf_init_set_str __gmpf_init_set_str
#define mpf_set_prec __gmpf_set_prec
#define mpf_set_default_prec __gmpf_set_default_prec
#define mpf_get_prec __gmpf_get_prec
#define mpf_get_default_prec __gmpf_get_default_prec
#define mpf_add __gmpf_add
#define mpf_add_ui __gmpf_add_ui
#define mpf_sub __gmpf_sub
#define mpf_sub_ui __gmpf_sub_ui
#define mpf_mul __gmpf_mul
#define mpf_mul_ui __gmpf_mul_ui
#define mpf_mul_2exp __gmpf_mul_2exp
#define mpf_div __gmpf_div
#define mpf_div_ui __gmpf_div_ui
#define mpf_div_2exp __gmpf_div_2exp
#define mpf_sqrt __gmpf_sqrt
#define mpf_neg __gmpf_neg
#define mpf_abs __gmpf_abs
#define mpf_cmp __gmpf_cmp
#define mpf_cmp_d __gmpf_cmp_d
#define mpf_cmp_ui __gmpf_cmp_ui
#define mpf_cmp_si __gmpf_cmp_si
#define mpf_get_d __gmpf_get_d
#define mpf_get_d_2exp __gmpf_get_d_2exp
#define mpf_get_str __gmpf_get_str
#define mpz_init __gmpz_init
#define mpz_clear __gmpz_clear
#define mpz_set_f __gmpz_set_f
#define mpz_import __gmpz_import
#define mpz_export __gmpz_export
#define mpn_mul_n __gmpn_mul_n
#define mpn_sqr __gmpn_sqr
#define mpn_addmul_1 __gmpn_addmul_1
#ifdef __cplusplus
}
#endif
#endif
