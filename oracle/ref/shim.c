/*
 * Oracle test infrastructure: link shim for building the reference's own C
 * sources of the banded-solve path without Intel MKL, GSL or Boost.
 *
 * The reference wraps BLAS/LAPACK behind suzerain_blas_* / suzerain_lapack_*
 * (suzerain/blas_et_al/blas.c, suzerain/blas_et_al/lapack.c) and requires MKL
 * (suzerain/blas_et_al/lapack.c:40-51).  Here the same entry points forward to
 * the LAPACK/BLAS symbols exported by SciPy's bundled OpenBLAS (scipy_*_),
 * resolved at link time.  The general-bandwidth banded matvec is compiled
 * from the reference's suzerain/blas_et_al/gbmv.def itself; the fixed
 * bandwidth specialisations of suzerain/blas_et_al/gbmv.c:346-366 only apply
 * to kl == ku <= 15 and compute the same sums.
 *
 * Nothing in the product links this file: it exists so tests can check the
 * oracle restatement against the reference's own code.
 */
#include <suzerain/common.h>
#include <suzerain/blas_et_al.h>
#include <suzerain/blas_et_al/gbmv.h>
#include <gsl/gsl_permutation.h>

/* ---- SciPy OpenBLAS (Fortran ABI, hidden character lengths last) ------- */
typedef int fint;
extern void scipy_zgbtrf_(const fint*, const fint*, const fint*, const fint*,
                          complex_double*, const fint*, fint*, fint*);
extern void scipy_cgbtrf_(const fint*, const fint*, const fint*, const fint*,
                          complex_float*, const fint*, fint*, fint*);
extern void scipy_dgbtrf_(const fint*, const fint*, const fint*, const fint*,
                          double*, const fint*, fint*, fint*);
extern void scipy_sgbtrf_(const fint*, const fint*, const fint*, const fint*,
                          float*, const fint*, fint*, fint*);
extern void scipy_zgbtrs_(const char*, const fint*, const fint*, const fint*,
                          const fint*, const complex_double*, const fint*,
                          const fint*, complex_double*, const fint*, fint*,
                          size_t);
extern void scipy_cgbtrs_(const char*, const fint*, const fint*, const fint*,
                          const fint*, const complex_float*, const fint*,
                          const fint*, complex_float*, const fint*, fint*,
                          size_t);
extern void scipy_dgbtrs_(const char*, const fint*, const fint*, const fint*,
                          const fint*, const double*, const fint*,
                          const fint*, double*, const fint*, fint*, size_t);
extern void scipy_sgbtrs_(const char*, const fint*, const fint*, const fint*,
                          const fint*, const float*, const fint*,
                          const fint*, float*, const fint*, fint*, size_t);
extern double scipy_zlangb_(const char*, const fint*, const fint*, const fint*,
                            const complex_double*, const fint*, double*,
                            size_t);
extern double scipy_dlangb_(const char*, const fint*, const fint*, const fint*,
                            const double*, const fint*, double*, size_t);
extern double scipy_dlamch_(const char*, size_t);
extern double scipy_dznrm2_(const fint*, const complex_double*, const fint*);
extern double scipy_dnrm2_(const fint*, const double*, const fint*);
extern void scipy_zlacpy_(const char*, const fint*, const fint*,
                          const complex_double*, const fint*,
                          complex_double*, const fint*, size_t);
extern void scipy_dlacpy_(const char*, const fint*, const fint*,
                          const double*, const fint*, double*, const fint*,
                          size_t);
extern void scipy_openblas_set_num_threads(int);

/* Errors only counted: the reference's xerbla prints via MKL and returns. */
int oracle_ref_xerbla_count = 0;
int suzerain_blas_xerbla(const char *srname, const int info)
{
    (void) srname;
    ++oracle_ref_xerbla_count;
    return info;
}

void oracle_ref_single_thread(void) { scipy_openblas_set_num_threads(1); }

gsl_permutation *gsl_permutation_alloc(size_t n)
{
    gsl_permutation *p = malloc(sizeof(*p));
    if (!p) return NULL;
    p->size = n;
    p->data = malloc(n * sizeof(size_t));
    if (!p->data) { free(p); return NULL; }
    return p;
}

void gsl_permutation_free(gsl_permutation *p)
{
    if (p) { free(p->data); free(p); }
}

/* ---- LAPACK wrappers (suzerain/blas_et_al/lapack.c semantics) ---------- */
#define GBTRF(P, T)                                                         \
int suzerain_lapack_##P##gbtrf(const int m, const int n, const int kl,      \
                               const int ku, T *ab, const int ldab,         \
                               int *ipiv)                                   \
{                                                                           \
    fint info = 0;                                                          \
    scipy_##P##gbtrf_(&m, &n, &kl, &ku, ab, &ldab, ipiv, &info);            \
    return info;                                                            \
}
GBTRF(z, complex_double)
GBTRF(c, complex_float)
GBTRF(d, double)
GBTRF(s, float)

#define GBTRS(P, T)                                                         \
int suzerain_lapack_##P##gbtrs(const char trans, const int n, const int kl, \
                               const int ku, const int nrhs, const T *ab,   \
                               const int ldab, const int *ipiv, T *b,       \
                               const int ldb)                               \
{                                                                           \
    fint info = 0;                                                          \
    scipy_##P##gbtrs_(&trans, &n, &kl, &ku, &nrhs, ab, &ldab, ipiv, b,      \
                      &ldb, &info, 1);                                      \
    return info;                                                            \
}
GBTRS(z, complex_double)
GBTRS(c, complex_float)
GBTRS(d, double)
GBTRS(s, float)

double suzerain_lapack_zlangb(const char norm, const int n, const int kl,
                              const int ku, const complex_double *ab,
                              const int ldab, double *work)
{
    double dummy = 0;
    return scipy_zlangb_(&norm, &n, &kl, &ku, ab, &ldab,
                         work ? work : &dummy, 1);
}

double suzerain_lapack_dlangb(const char norm, const int n, const int kl,
                              const int ku, const double *ab, const int ldab,
                              double *work)
{
    double dummy = 0;
    return scipy_dlangb_(&norm, &n, &kl, &ku, ab, &ldab,
                         work ? work : &dummy, 1);
}

double suzerain_lapack_dlamch(char cmach) { return scipy_dlamch_(&cmach, 1); }

void suzerain_lapack_zlacpy(char uplo, const int m, const int n,
                            const complex_double *a, const int lda,
                            complex_double *b, const int ldb)
{
    scipy_zlacpy_(&uplo, &m, &n, a, &lda, b, &ldb, 1);
}

void suzerain_lapack_dlacpy(char uplo, const int m, const int n,
                            const double *a, const int lda, double *b,
                            const int ldb)
{
    scipy_dlacpy_(&uplo, &m, &n, a, &lda, b, &ldb, 1);
}

/* ---- BLAS level 1 (plain loops; unit semantics of the BLAS) ------------ */
void suzerain_blas_zcopy(const int n, const complex_double *x, const int incx,
                         complex_double *y, const int incy)
{
    int ix = incx < 0 ? (1 - n) * incx : 0, iy = incy < 0 ? (1 - n) * incy : 0;
    for (int i = 0; i < n; ++i, ix += incx, iy += incy) y[iy] = x[ix];
}

void suzerain_blas_dcopy(const int n, const double *x, const int incx,
                         double *y, const int incy)
{
    int ix = incx < 0 ? (1 - n) * incx : 0, iy = incy < 0 ? (1 - n) * incy : 0;
    for (int i = 0; i < n; ++i, ix += incx, iy += incy) y[iy] = x[ix];
}

void suzerain_blas_zaxpy(const int n, const complex_double alpha,
                         const complex_double *x, const int incx,
                         complex_double *y, const int incy)
{
    int ix = incx < 0 ? (1 - n) * incx : 0, iy = incy < 0 ? (1 - n) * incy : 0;
    for (int i = 0; i < n; ++i, ix += incx, iy += incy) y[iy] += alpha * x[ix];
}

void suzerain_blas_zscal(const int n, const complex_double alpha,
                         complex_double *x, const int incx)
{
    for (int i = 0; i < n; ++i) x[i * incx] *= alpha;
}

/* The reference's MKL configuration: scale y by beta (unless beta == 1),
 * then y += alpha x (suzerain/blas_et_al/blas.c:636-657). */
void suzerain_blas_zaxpby(const int n, const complex_double alpha,
                          const complex_double *x, const int incx,
                          const complex_double beta, complex_double *y,
                          const int incy)
{
    if (beta != 1.0) suzerain_blas_zscal(n, beta, y, incy);
    suzerain_blas_zaxpy(n, alpha, x, incx, y, incy);
}

void suzerain_blas_daxpy(const int n, const double alpha, const double *x,
                         const int incx, double *y, const int incy)
{
    int ix = incx < 0 ? (1 - n) * incx : 0, iy = incy < 0 ? (1 - n) * incy : 0;
    for (int i = 0; i < n; ++i, ix += incx, iy += incy) y[iy] += alpha * x[ix];
}

double suzerain_blas_dznrm2(const int n, const complex_double *x,
                            const int incx)
{
    return scipy_dznrm2_(&n, x, &incx);
}

double suzerain_blas_dnrm2(const int n, const double *x, const int incx)
{
    return scipy_dnrm2_(&n, x, &incx);
}

/* blasext demote/promote come from the reference's own blasext.c, which
 * the reference build compiles too. */

/* ---- banded matvec: general-bandwidth code from the reference's gbmv.def */
#define STATIC   static
#define FUNCTION oracle_ref_gbmv_internal_z
#define TYPE_A   complex_double
#define TYPE_X   complex_double
#define TYPE_Y   complex_double
#define KL       const int kl,
#define KU       const int ku,
#include <suzerain/blas_et_al/gbmv.def>

#define STATIC   static
#define FUNCTION oracle_ref_gbmv_internal_d
#define TYPE_A   double
#define TYPE_X   double
#define TYPE_Y   double
#define KL       const int kl,
#define KU       const int ku,
#include <suzerain/blas_et_al/gbmv.def>

int suzerain_blas_zgbmv(const char trans, const int m, const int n,
                        const int kl, const int ku,
                        const complex_double alpha, const complex_double *a,
                        const int lda, const complex_double *x, const int incx,
                        const complex_double beta, complex_double *y,
                        const int incy)
{
    const int info = oracle_ref_gbmv_internal_z(trans, m, n, kl, ku, alpha, a,
                                                lda, x, incx, beta, y, incy);
    if (info) suzerain_blas_xerbla(__func__, info);
    return info;
}

int suzerain_blas_dgbmv(const char trans, const int m, const int n,
                        const int kl, const int ku, const double alpha,
                        const double *a, const int lda, const double *x,
                        const int incx, const double beta, double *y,
                        const int incy)
{
    const int info = oracle_ref_gbmv_internal_d(trans, m, n, kl, ku, alpha, a,
                                                lda, x, incx, beta, y, incy);
    if (info) suzerain_blas_xerbla(__func__, info);
    return info;
}
