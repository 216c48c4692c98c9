/* Minimal stand-in for GSL's permutation type: the two public members that
 * the reference's bsmbsm.c touches (size, data) plus alloc/free.  Only the
 * oracle's reference build uses it; GSL itself is not installed here. */
#ifndef ORACLE_REF_GSL_PERMUTATION_H
#define ORACLE_REF_GSL_PERMUTATION_H
#include <stddef.h>
#include <stdlib.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef struct { size_t size; size_t *data; } gsl_permutation;
gsl_permutation *gsl_permutation_alloc(size_t n);
void gsl_permutation_free(gsl_permutation *p);
#ifdef __cplusplus
}
#endif
#endif
