/* Minimal stand-in for GSL's B-spline header: the reference's bsplineop.h
 * names gsl_bspline_workspace only in prototypes of functions the oracle's
 * reference build does not compile (it builds rholut_imexop.c, which reads
 * an already-formed suzerain_bsplineop_workspace).  GSL is not installed
 * here. */
#ifndef ORACLE_REF_GSL_BSPLINE_H
#define ORACLE_REF_GSL_BSPLINE_H
#ifdef __cplusplus
extern "C" {
#endif
typedef struct gsl_bspline_workspace gsl_bspline_workspace;
#ifdef __cplusplus
}
#endif
#endif
