/* Types-only stand-in for <mpfr.h>: the reference engine headers name MPFR
 * types in declarations of expression-engine functions that the Mandelbrot
 * path never calls. Oracle build support only. */
#ifndef MBX_COMPAT_MPFR_H
#define MBX_COMPAT_MPFR_H
#include "gmp.h"
#ifdef __cplusplus
extern "C" {
#endif
typedef long mpfr_prec_t;
typedef int mpfr_sign_t;
typedef long mpfr_exp_t;
typedef enum { MPFR_RNDN = 0, MPFR_RNDZ, MPFR_RNDU, MPFR_RNDD, MPFR_RNDA, MPFR_RNDF, MPFR_RNDNA = -1 } mpfr_rnd_t;
typedef struct { mpfr_prec_t _mpfr_prec; mpfr_sign_t _mpfr_sign; mpfr_exp_t _mpfr_exp; mp_limb_t* _mpfr_d; } __mpfr_struct;
typedef __mpfr_struct mpfr_t[1];
typedef __mpfr_struct* mpfr_ptr;
typedef const __mpfr_struct* mpfr_srcptr;
#ifdef __cplusplus
}
#endif
#endif
