/*
 * Oracle test infrastructure: what the reference build of
 * suzerain/rholut_imexop.c and suzerain/blas_et_al/blasext.c needs beyond
 * the other objects of libsuzref.so.
 *
 *   suzerain_blas_zgb_acc_d   the reference's MKL configuration of it
 *                             (suzerain/blas_et_al/blas.c:1408-1421): a
 *                             diagonal scaling by one through
 *                             suzerain_blasext_zgb_diag_scale_acc_d
 *   suzerain_blas_zgbmv_d_z   real band times complex vector through the
 *                             reference's general-bandwidth gbmv.def
 *                             (suzerain/blas_et_al/blas.c:1081-1100)
 *   suzerain_blas_zaxpy_d,    complex scalar times real vector (the plain
 *   suzerain_blas_zaxpby_d    loops of the reference's MKL configuration)
 *   suzerain_blas_malloc/free plain malloc and free
 *   the remaining symbols     blasext.c's other routines reference BLAS
 *                             wrappers and fixed-bandwidth kernels that the
 *                             reference generates with Boost.Preprocessor;
 *                             nothing on the rholut_imexop path calls them:
 *                             imexop_stubs.c stands in for each.
 *
 * Nothing in the product links this file.
 */
#include <stdio.h>
#include <stdlib.h>
#include <suzerain/common.h>
#include <suzerain/blas_et_al.h>

#define STATIC   static
#define FUNCTION oracle_ref_gbmv_internal_dzz
#define TYPE_A   double
#define TYPE_X   complex_double
#define TYPE_Y   complex_double
#define KL       const int kl,
#define KU       const int ku,
#include <suzerain/blas_et_al/gbmv.def>

int suzerain_blas_zgbmv_d_z(const char trans, const int m, const int n,
                            const int kl, const int ku, const complex_double alpha,
                            const double *a, const int lda, const complex_double *x,
                            const int incx, const complex_double beta,
                            complex_double *y, const int incy)
{
    const int info = oracle_ref_gbmv_internal_dzz(trans, m, n, kl, ku, alpha, a, lda,
                                                  x, incx, beta, y, incy);
    if (info) suzerain_blas_xerbla(__func__, info);
    return info;
}

int suzerain_blas_zgb_acc_d(const int m, const int n, const int kl, const int ku,
                            const complex_double alpha, const double *a, const int lda,
                            const complex_double beta, complex_double *b, const int ldb)
{
    const double one = 1.0;
    return suzerain_blasext_zgb_diag_scale_acc_d('R', m, n, kl, ku, alpha, &one, 0,
                                                 a, 1, lda, beta, b, 1, ldb);
}

/* y <- alpha x + y and y <- alpha x + beta y for complex alpha, beta, y and
 * real x: the reference's MKL configuration computes these with plain loops
 * (suzerain/blas_et_al/blas.c:534-564, :661-713), which this restates. */
void suzerain_blas_zaxpy_d(const int n, const complex_double alpha, const double *x,
                           const int incx, complex_double *y, const int incy)
{
    int ix = (incx < 0) ? (1 - n) * incx : 0;
    int iy = (incy < 0) ? (1 - n) * incy : 0;
    for (int i = 0; i < n; ++i, ix += incx, iy += incy) y[iy] += alpha * x[ix];
}

void suzerain_blas_zaxpby_d(const int n, const complex_double alpha, const double *x,
                            const int incx, const complex_double beta, complex_double *y,
                            const int incy)
{
    int ix = (incx < 0) ? (1 - n) * incx : 0;
    int iy = (incy < 0) ? (1 - n) * incy : 0;
    for (int i = 0; i < n; ++i, ix += incx, iy += incy) {
        if (beta == 0) {
            y[iy] = alpha * x[ix];
        } else {
            y[iy] *= beta;
            y[iy] += alpha * x[ix];
        }
    }
}

void *suzerain_blas_malloc(size_t size) { return malloc(size); }
void suzerain_blas_free(void *ptr) { free(ptr); }
