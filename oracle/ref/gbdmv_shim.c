/*
 * Oracle test infrastructure: the reference's general-bandwidth diagonally
 * scaled band matvec with GBD_K = 1..5 diagonals (the FUNCTION bodies of
 * suzerain/blas_et_al/gbdmv.def, gbddmv.def, gbdddmv.def, gbddddmv.def and
 * gbdddddmv.def), instantiated as suzerain/blas_et_al/blasext.c's z*_d_z
 * and z*_d_d wrappers use them: real diagonals and band, complex
 * coefficients and output, complex (dzz) or real (ddz) x.  Exported as
 * oracle_ref_gbd<K>mv_{dzz,ddz}, returning the argument position the
 * reference hands to xerbla.  The Makefile compiles this file once per
 * arity, because every .def defines its own index helpers.  The fixed
 * bandwidth variants that suzerain/blas_et_al/gbd*mv.c generate for
 * kl == ku <= 15 evaluate the same sums.
 *
 * Nothing in the product links this file: it exists so tests can check the
 * oracle's formula for these operators against the reference's own code.
 */
#include <suzerain/common.h>
#include <suzerain/blas_et_al.h>

#if GBD_K == 1
#define GBD_DEF <suzerain/blas_et_al/gbdmv.def>
#elif GBD_K == 2
#define GBD_DEF <suzerain/blas_et_al/gbddmv.def>
#elif GBD_K == 3
#define GBD_DEF <suzerain/blas_et_al/gbdddmv.def>
#elif GBD_K == 4
#define GBD_DEF <suzerain/blas_et_al/gbddddmv.def>
#elif GBD_K == 5
#define GBD_DEF <suzerain/blas_et_al/gbdddddmv.def>
#else
#error "GBD_K must be 1..5"
#endif

#define GBD_CAT(a, b, c) a##b##c
#define GBD_NAME(k, sfx) GBD_CAT(oracle_ref_gbd, k, sfx)

#define STATIC   /*exported*/
#define FUNCTION GBD_NAME(GBD_K, mv_dzz)
#define TYPE_D   double
#define TYPE_A   double
#define TYPE_X   complex_double
#define TYPE_Y   complex_double
#define KL       const int kl,
#define KU       const int ku,
#include GBD_DEF

#define STATIC   /*exported*/
#define FUNCTION GBD_NAME(GBD_K, mv_ddz)
#define TYPE_D   double
#define TYPE_A   double
#define TYPE_X   double
#define TYPE_Y   complex_double
#define KL       const int kl,
#define KU       const int ku,
#include GBD_DEF

/* The same body once more under the reference's own name of the
 * general-bandwidth routine (real diagonals and band, complex x and y),
 * which suzerain/blas_et_al/blasext.c's zgb<d..>mv_d_z wrappers call; the
 * reference build of suzerain/rholut_imexop.c reaches it through them. */
#if GBD_K == 1
#define GBD_REF_NAME suzerain_gbdmv_dzz
#elif GBD_K == 2
#define GBD_REF_NAME suzerain_gbddmv_dzz
#elif GBD_K == 3
#define GBD_REF_NAME suzerain_gbdddmv_dzz
#elif GBD_K == 4
#define GBD_REF_NAME suzerain_gbddddmv_dzz
#else
#define GBD_REF_NAME suzerain_gbdddddmv_dzz
#endif
#define STATIC   /*exported*/
#define FUNCTION GBD_REF_NAME
#define TYPE_D   double
#define TYPE_A   double
#define TYPE_X   complex_double
#define TYPE_Y   complex_double
#define KL       const int kl,
#define KU       const int ku,
#include GBD_DEF
