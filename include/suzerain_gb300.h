/*
 * suzerain_gb300 -- GB300-native batched BSMBSM implicit solve.
 *
 * Two layers, both plain C ABI (pointers, sizes, no torch types):
 *
 *  1. Drop-in replacements for the reference's entry points on the
 *     per-wavenumber implicit-solve path, with the reference's names,
 *     signatures, argument meaning and error conventions.  Each is cited
 *     beside its declaration.  Pointers may be host or device memory; host
 *     data is staged through device memory and every computation runs on the
 *     GPU (there is no CPU fallback: without a usable device the calls return
 *     an error).
 *
 *  2. The batched device API (prefix sgb_) that one call per substep drives
 *     thousands of (kx, kz) systems through: explicit operator apply, complex
 *     band LU (complex128, or complex64 with FP64 refinement and complex128
 *     fallback), solve, permutation.  Device pointers, a cudaStream_t
 *     (passed as void*), caller-owned memory.
 *
 * Complex scalars are C99 double _Complex / float _Complex in C and
 * std::complex<double> / std::complex<float> in C++ (layout compatible, as
 * suzerain/complex.h:28-45 arranges for the reference).
 */
#ifndef SUZERAIN_GB300_H
#define SUZERAIN_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
#include <complex>
typedef std::complex<double> sgb_complex_double;
typedef std::complex<float>  sgb_complex_float;
extern "C" {
#else
#include <complex.h>
typedef double _Complex sgb_complex_double;
typedef float _Complex  sgb_complex_float;
#endif

/* ======================================================================== */
/* 1. Drop-in replacements                                                  */
/* ======================================================================== */

/** BSMBSM geometry; same fields and meaning as suzerain/bsmbsm.h:104-116. */
typedef struct suzerain_bsmbsm {
    int S, n, kl, ku, ld, N, KL, KU, LD;
} suzerain_bsmbsm;

/** suzerain/bsmbsm.h:130-149 (static inline there; exported here). */
suzerain_bsmbsm suzerain_bsmbsm_construct(int S, int n, int kl, int ku);
/** q(i) = (i mod S) n + floor(i / S); suzerain/bsmbsm.h:162-169. */
int suzerain_bsmbsm_q(int S, int n, int i);
/** q^{-1}(i) = q with S and n exchanged; suzerain/bsmbsm.h:182-186. */
int suzerain_bsmbsm_qinv(int S, int n, int i);

/** Same layout as gsl_permutation (size, then the index array). */
typedef struct sgb_permutation {
    size_t size;
    size_t *data;
} sgb_permutation;
/** q as a permutation of S n indices; suzerain/bsmbsm.h:294,
 *  suzerain/bsmbsm.c:109-124.  Both blocks come from malloc, so
 *  gsl_permutation_free (or sgb_permutation_free) releases the result;
 *  NULL for S <= 0, n <= 0 or on allocation failure. */
sgb_permutation *suzerain_bsmbsm_permutation(int S, int n);
void sgb_permutation_free(sgb_permutation *p);

/** y <- alpha P x + beta y ('N') or alpha P^T x + beta y ('T');
 *  suzerain/bsmbsm.h:208-257, suzerain/bsmbsm_aPxpby_complex.def:36-329.
 *  Returns 0, or the positive BLAS argument position of a bad argument
 *  (1 trans, 2 S, 3 n, 58 x aliases y). */
int suzerain_bsmbsm_saPxpby(char trans, int S, int n, const float alpha,
                            const float *x, int incx, const float beta,
                            float *y, int incy);
int suzerain_bsmbsm_daPxpby(char trans, int S, int n, const double alpha,
                            const double *x, int incx, const double beta,
                            double *y, int incy);
int suzerain_bsmbsm_caPxpby(char trans, int S, int n,
                            const sgb_complex_float alpha,
                            const sgb_complex_float *x, int incx,
                            const sgb_complex_float beta,
                            sgb_complex_float *y, int incy);
int suzerain_bsmbsm_zaPxpby(char trans, int S, int n,
                            const sgb_complex_double alpha,
                            const sgb_complex_double *x, int incx,
                            const sgb_complex_double beta,
                            sgb_complex_double *y, int incy);

/** Pack alpha B^{ihat,jhat} into band storage of P A P^T, zeroing the
 *  block's positions outside B's band; suzerain/bsmbsm.h:338-381,
 *  suzerain/bsmbsm_pack.def:36-122.  Returns 0 or the positive argument
 *  position (511 when b aliases papt). */
int suzerain_bsmbsm_spack(int S, int n, int ihat, int jhat, int kl, int ku,
                          const float alpha, const float *b, int ldb,
                          int KL, int KU, float *papt, int ldpapt);
int suzerain_bsmbsm_dpack(int S, int n, int ihat, int jhat, int kl, int ku,
                          const double alpha, const double *b, int ldb,
                          int KL, int KU, double *papt, int ldpapt);
int suzerain_bsmbsm_cpack(int S, int n, int ihat, int jhat, int kl, int ku,
                          const sgb_complex_float alpha,
                          const sgb_complex_float *b, int ldb, int KL, int KU,
                          sgb_complex_float *papt, int ldpapt);
int suzerain_bsmbsm_cspack(int S, int n, int ihat, int jhat, int kl, int ku,
                           const sgb_complex_float alpha, const float *b,
                           int ldb, int KL, int KU, sgb_complex_float *papt,
                           int ldpapt);
int suzerain_bsmbsm_zpack(int S, int n, int ihat, int jhat, int kl, int ku,
                          const sgb_complex_double alpha,
                          const sgb_complex_double *b, int ldb, int KL, int KU,
                          sgb_complex_double *papt, int ldpapt);
int suzerain_bsmbsm_zdpack(int S, int n, int ihat, int jhat, int kl, int ku,
                           const sgb_complex_double alpha, const double *b,
                           int ldb, int KL, int KU, sgb_complex_double *papt,
                           int ldpapt);
/** packc / packf conveniences; suzerain/bsmbsm.h:407-468, :543-610. */
int suzerain_bsmbsm_zpackc(const suzerain_bsmbsm *A, int ihat, int jhat,
                           const sgb_complex_double alpha,
                           const sgb_complex_double *b,
                           sgb_complex_double *papt);
int suzerain_bsmbsm_zpackf(const suzerain_bsmbsm *A, int ihat, int jhat,
                           const sgb_complex_double alpha,
                           const sgb_complex_double *b,
                           sgb_complex_double *papt);
int suzerain_bsmbsm_zdpackc(const suzerain_bsmbsm *A, int ihat, int jhat,
                            const sgb_complex_double alpha, const double *b,
                            sgb_complex_double *papt);
int suzerain_bsmbsm_zdpackf(const suzerain_bsmbsm *A, int ihat, int jhat,
                            const sgb_complex_double alpha, const double *b,
                            sgb_complex_double *papt);
int suzerain_bsmbsm_spackc(const suzerain_bsmbsm *A, int ihat, int jhat,
                           const float alpha, const float *b, float *papt);
int suzerain_bsmbsm_spackf(const suzerain_bsmbsm *A, int ihat, int jhat,
                           const float alpha, const float *b, float *papt);
int suzerain_bsmbsm_dpackc(const suzerain_bsmbsm *A, int ihat, int jhat,
                           const double alpha, const double *b, double *papt);
int suzerain_bsmbsm_dpackf(const suzerain_bsmbsm *A, int ihat, int jhat,
                           const double alpha, const double *b, double *papt);
int suzerain_bsmbsm_cpackc(const suzerain_bsmbsm *A, int ihat, int jhat,
                           const sgb_complex_float alpha,
                           const sgb_complex_float *b, sgb_complex_float *papt);
int suzerain_bsmbsm_cpackf(const suzerain_bsmbsm *A, int ihat, int jhat,
                           const sgb_complex_float alpha,
                           const sgb_complex_float *b, sgb_complex_float *papt);
int suzerain_bsmbsm_cspackc(const suzerain_bsmbsm *A, int ihat, int jhat,
                            const sgb_complex_float alpha, const float *b,
                            sgb_complex_float *papt);
int suzerain_bsmbsm_cspackf(const suzerain_bsmbsm *A, int ihat, int jhat,
                            const sgb_complex_float alpha, const float *b,
                            sgb_complex_float *papt);

/** Partial-pivot band LU, LAPACK zgbtrf/cgbtrf semantics and storage
 *  ((2kl+ku+1) x n, 1-based ipiv, info > 0 at the first zero pivot);
 *  wraps of suzerain/blas_et_al/lapack.c:185-198. */
int suzerain_lapack_zgbtrf(const int m, const int n, const int kl,
                           const int ku, sgb_complex_double *ab,
                           const int ldab, int *ipiv);
int suzerain_lapack_cgbtrf(const int m, const int n, const int kl,
                           const int ku, sgb_complex_float *ab,
                           const int ldab, int *ipiv);
/** Band solve with a zgbtrf/cgbtrf factor, trans 'N', 'T' or 'C';
 *  suzerain/blas_et_al/lapack.c:261-279. */
int suzerain_lapack_zgbtrs(const char trans, const int n, const int kl,
                           const int ku, const int nrhs,
                           const sgb_complex_double *ab, const int ldab,
                           const int *ipiv, sgb_complex_double *b,
                           const int ldb);
int suzerain_lapack_cgbtrs(const char trans, const int n, const int kl,
                           const int ku, const int nrhs,
                           const sgb_complex_float *ab, const int ldab,
                           const int *ipiv, sgb_complex_float *b,
                           const int ldb);
/** LAPACK ZGBCON on a gbtrf factor (suzerain/blas_et_al/lapack.c): the
 *  reciprocal condition number in the 1-norm ('1' / 'O') or the
 *  infinity-norm ('I') by Higham's estimator; -i argument errors; work and
 *  rwork unused (may be NULL).  The estimator's triangular solves are plain
 *  solves (ZLATBS's rescaling against overflow is not reproduced). */
int suzerain_lapack_zgbcon(const char norm, const int n, const int kl, const int ku,
                           const sgb_complex_double *ab, const int ldab, const int *ipiv,
                           const double anorm, double *rcond, sgb_complex_double *work,
                           double *rwork);

/** LAPACK's expert driver zgbsvx (equilibration for fact 'E', factor for
 *  'N'/'E', a given factor for 'F', reciprocal condition number, solve,
 *  iterative refinement with forward and backward error bounds, unscaling;
 *  info = n+1 when rcond < eps); suzerain/blas_et_al/lapack.c:548-574 and
 *  lapack.h:601-626, as called by suzerain/bsmbsm_solver.cpp:252-291.  Same
 *  23 arguments; work is not used and rwork[0] receives the reciprocal pivot
 *  growth.  The condition estimate's triangular solves do not rescale
 *  against overflow (zlatbs with scale < 1). */
int suzerain_lapack_zgbsvx(const char fact, const char trans, const int n,
                           const int kl, const int ku, const int nrhs,
                           sgb_complex_double *ab, const int ldab,
                           sgb_complex_double *afb, const int ldafb,
                           int *ipiv, char *equed, double *r, double *c,
                           sgb_complex_double *b, const int ldb,
                           sgb_complex_double *x, const int ldx,
                           double *rcond, double *ferr, double *berr,
                           sgb_complex_double *work, double *rwork);

/** Factor when *fact == 'N' (then *fact = 'F'), solve;
 *  suzerain/blas_et_al/lapackext.c:127-147. */
int suzerain_lapackext_zgbsv(char *const fact, const char trans, const int n,
                             const int kl, const int ku, const int nrhs,
                             sgb_complex_double *ab, const int ldab, int *ipiv,
                             sgb_complex_double *b, const int ldb);
int suzerain_lapackext_cgbsv(char *const fact, const char trans, const int n,
                             const int kl, const int ku, const int nrhs,
                             sgb_complex_float *ab, const int ldab, int *ipiv,
                             sgb_complex_float *b, const int ldb);
/** Real forms (suzerain/blas_et_al/lapackext.h:66-95): the complex kernels
 *  on the band promoted with zero imaginary parts. */
int suzerain_lapackext_dgbsv(char *const fact, const char trans, const int n,
                             const int kl, const int ku, const int nrhs,
                             double *ab, const int ldab, int *ipiv,
                             double *b, const int ldb);
int suzerain_lapackext_sgbsv(char *const fact, const char trans, const int n,
                             const int kl, const int ku, const int nrhs,
                             float *ab, const int ldab, int *ipiv,
                             float *b, const int ldb);

/** Complex64 LU with FP64 iterative refinement and complex128 fallback;
 *  suzerain/blas_et_al/lapackext.h:258-299,
 *  suzerain/blas_et_al/dsgbsvx.def:70-313.  Same 18 arguments.  ab must be
 *  contiguous (ldab = kl+ku+1); afb returns the factor in LAPACK storage
 *  (ldafb = 2kl+ku+1), complex64 packed at its start when *fact == 'S'.
 *  The residual uses the reference gbmv's convention for trans 'C'
 *  (suzerain/blas_et_al/gbmv.def:161-196 treats 'C' as 'T'). */
int suzerain_lapackext_zcgbsvx(char *const fact, int *const apprx,
                               const int aiter, char trans, const int n,
                               const int kl, const int ku,
                               sgb_complex_double *const ab,
                               double *const afrob,
                               sgb_complex_double *const afb, int *const ipiv,
                               sgb_complex_double *const b,
                               sgb_complex_double *const x, int *const siter,
                               int *const diter, double *const tolsc,
                               sgb_complex_double *const r, double *const res);
/** The real form (same 18 arguments, suzerain/blas_et_al/lapackext.h:258-277):
 *  zcgbsvx on the promoted band; afb returns the float32 factor at its start
 *  for fact 'S' (the in-place demotion), the float64 one for 'D'. */
int suzerain_lapackext_dsgbsvx(char *const fact, int *const apprx,
                               const int aiter, char trans, const int n,
                               const int kl, const int ku, double *const ab,
                               double *const afrob, double *const afb,
                               int *const ipiv, double *const b,
                               double *const x, int *const siter,
                               int *const diter, double *const tolsc,
                               double *const r, double *const res);

/** y <- alpha op(A) x + beta y for a band A; suzerain/blas_et_al/blas.c:1035-1054
 *  over suzerain/blas_et_al/gbmv.def ('C' takes the 'T' branch unconjugated). */
int suzerain_blas_zgbmv(const char trans, const int m, const int n,
                        const int kl, const int ku,
                        const sgb_complex_double alpha,
                        const sgb_complex_double *a, const int lda,
                        const sgb_complex_double *x, const int incx,
                        const sgb_complex_double beta, sgb_complex_double *y,
                        const int incy);

/** B-spline collocation operators; workspace layout of
 *  suzerain/bsplineop.h:125-180 (transposed bands D_T). */
enum suzerain_bsplineop_method {
    SUZERAIN_BSPLINEOP_COLLOCATION_GREVILLE = 1,
    SUZERAIN_BSPLINEOP_GALERKIN_L2
};
typedef struct suzerain_bsplineop_workspace {
    enum suzerain_bsplineop_method method;
    int k, n, nderiv;
    int *kl, *ku;
    int max_kl, max_ku, ld;
    double **D_T;
} suzerain_bsplineop_workspace;
/** Replaces suzerain_bsplineop_alloc(gsl_bspline_workspace*, nderiv,
 *  COLLOCATION_GREVILLE) (suzerain/bsplineop.c:102-202): the GSL workspace
 *  argument becomes its defining data (order k and the breakpoints). */
suzerain_bsplineop_workspace *
sgb_bsplineop_alloc_breakpoints(int k, int nbreak, const double *breakpts,
                                int nderiv);
/** suzerain/bsplineop.c:205-219. */
void suzerain_bsplineop_free(suzerain_bsplineop_workspace *w);
/** y <- alpha D^nderiv x + beta y per right-hand side (complex x, y, alpha,
 *  beta); suzerain/bsplineop.c:261-298. */
int suzerain_bsplineop_accumulate_complex(int nderiv, int nrhs,
                                          const sgb_complex_double alpha,
                                          const sgb_complex_double *x,
                                          int incx, int ldx,
                                          const sgb_complex_double beta,
                                          sgb_complex_double *y, int incy,
                                          int ldy,
                                          const suzerain_bsplineop_workspace *w);

/** x <- alpha D^nderiv x in place (real and complex coefficients, real
 *  alpha) and y <- alpha D^nderiv x + beta y (real), per right-hand side;
 *  suzerain/bsplineop.c:222-400.  Argument errors return SUZERAIN_EINVAL (4)
 *  (the reference's code after its error handler); increments must be
 *  positive. */
int suzerain_bsplineop_apply(int nderiv, int nrhs, double alpha, double *x, int incx, int ldx,
                             const suzerain_bsplineop_workspace *w);
int suzerain_bsplineop_accumulate(int nderiv, int nrhs, double alpha, const double *x, int incx,
                                  int ldx, double beta, double *y, int incy, int ldy,
                                  const suzerain_bsplineop_workspace *w);
int suzerain_bsplineop_apply_complex(int nderiv, int nrhs, double alpha, sgb_complex_double *x,
                                     int incx, int ldx, const suzerain_bsplineop_workspace *w);

/** Operator workspaces of suzerain/bsplineop.h:455-990: the transpose of a
 *  linear combination of the D^m in LAPACK gbtrf storage (A_T + kl is the
 *  unfactored band, ld = 2 kl + ku + 1), its pivots, and the state flag
 *  ipiv[0] < 0 (not factored; -ipiv[0] counts accumulations).  Host memory,
 *  as the reference allocates it; the operations run on the GPU.  Codes:
 *  0, SUZERAIN_EINVAL (4) for bad arguments or call order, SUZERAIN_ESANITY
 *  (7) when the factor, norm or estimate reports an error, SUZERAIN_ENOMEM
 *  (8).  The real workspace factors, estimates and solves in complex
 *  arithmetic with zero imaginary parts. */
typedef struct suzerain_bsplineop_lu_workspace {
    int n, kl, ku, ld;
    int *ipiv;
    double *A_T;
} suzerain_bsplineop_lu_workspace;
typedef struct suzerain_bsplineop_luz_workspace {
    int n, kl, ku, ld;
    int *ipiv;
    sgb_complex_double *A_T;
} suzerain_bsplineop_luz_workspace;

suzerain_bsplineop_lu_workspace *suzerain_bsplineop_lu_alloc(const suzerain_bsplineop_workspace *w);
void suzerain_bsplineop_lu_free(suzerain_bsplineop_lu_workspace *luw);
int suzerain_bsplineop_lu_opaccumulate(int ncoefficients, const double *coefficients,
                                       const suzerain_bsplineop_workspace *w, const double scale,
                                       suzerain_bsplineop_lu_workspace *luw);
int suzerain_bsplineop_lu_opnorm(const suzerain_bsplineop_lu_workspace *luw, double *norm);
int suzerain_bsplineop_lu_factor(suzerain_bsplineop_lu_workspace *luw);
int suzerain_bsplineop_lu_rcond(const double norm, double *rcond,
                                const suzerain_bsplineop_lu_workspace *luw);
int suzerain_bsplineop_lu_solve(int nrhs, double *B, int incb, int ldb,
                                const suzerain_bsplineop_lu_workspace *luw);
int suzerain_bsplineop_lu_opform(int ncoefficients, const double *coefficients,
                                 const suzerain_bsplineop_workspace *w,
                                 suzerain_bsplineop_lu_workspace *luw);
int suzerain_bsplineop_lu_opform_mass(const suzerain_bsplineop_workspace *w,
                                      suzerain_bsplineop_lu_workspace *luw);
int suzerain_bsplineop_lu_factor_mass(const suzerain_bsplineop_workspace *w,
                                      suzerain_bsplineop_lu_workspace *luw);

suzerain_bsplineop_luz_workspace *suzerain_bsplineop_luz_alloc(const suzerain_bsplineop_workspace *w);
void suzerain_bsplineop_luz_free(suzerain_bsplineop_luz_workspace *luzw);
int suzerain_bsplineop_luz_opaccumulate(int ncoefficients, const sgb_complex_double *coefficients,
                                        const suzerain_bsplineop_workspace *w,
                                        const sgb_complex_double scale,
                                        suzerain_bsplineop_luz_workspace *luzw);
int suzerain_bsplineop_luz_opnorm(const suzerain_bsplineop_luz_workspace *luzw, double *norm);
int suzerain_bsplineop_luz_factor(suzerain_bsplineop_luz_workspace *luzw);
int suzerain_bsplineop_luz_rcond(const double norm, double *rcond,
                                 const suzerain_bsplineop_luz_workspace *luzw);
int suzerain_bsplineop_luz_solve(int nrhs, sgb_complex_double *B, int incb, int ldb,
                                 const suzerain_bsplineop_luz_workspace *luzw);
int suzerain_bsplineop_luz_opform(int ncoefficients, const sgb_complex_double *coefficients,
                                  const suzerain_bsplineop_workspace *w,
                                  suzerain_bsplineop_luz_workspace *luzw);
int suzerain_bsplineop_luz_opform_mass(const suzerain_bsplineop_workspace *w,
                                       suzerain_bsplineop_luz_workspace *luzw);
int suzerain_bsplineop_luz_factor_mass(const suzerain_bsplineop_workspace *w,
                                       suzerain_bsplineop_luz_workspace *luzw);

/** Non-transposed collocation matrices d^m B_j(xi_i), m = 0..nderiv, as
 *  LAPACK bands with the common trimmed kl/ku; bands may be NULL to query
 *  n/kl/ku.  bands[(m*n + j)*ld + ku + i - j], ld = kl+1+ku. */
int sgb_bspline_collocation_bands(int k, int nbreak, const double *breakpts,
                                  int nderiv, int *n, int *kl, int *ku,
                                  double *bands, double *abscissae);

/* ---- Band assembly helpers (suzerain/blas_et_al/blasext.h, blas.h) ----- */

/** B <- A (alpha D) + beta B (side 'R') or (alpha D) A + beta B (side 'L')
 *  for a real band A (kl, ku; element (i, j) at a[(ku+i-j) inca + j lda]),
 *  a real diagonal D (stride ldd, 0 for a constant) and a complex band B;
 *  returns the reference's positive argument position on error;
 *  suzerain/blas_et_al/blasext.h:1525-1540, blasext.c:2070-2141. */
int suzerain_blasext_zgb_diag_scale_acc_d(
    char side, int m, int n, int kl, int ku, const sgb_complex_double alpha, const double *d,
    int ldd, const double *a, int inca, int lda, const sgb_complex_double beta,
    sgb_complex_double *b, int incb, int ldb);
/** The two- to five-diagonal forms, sum_k alpha_k D_k;
 *  suzerain/blas_et_al/blasext.h:1576-1800, blasext.c:2143-2500. */
int suzerain_blasext_zgb_ddiag_scale_acc_d(
    char side, int m, int n, int kl, int ku, const sgb_complex_double alpha0, const double *d0,
    int ldd0, const sgb_complex_double alpha1, const double *d1, int ldd1, const double *a,
    int inca, int lda, const sgb_complex_double beta, sgb_complex_double *b, int incb, int ldb);
int suzerain_blasext_zgb_dddiag_scale_acc_d(
    char side, int m, int n, int kl, int ku, const sgb_complex_double alpha0, const double *d0,
    int ldd0, const sgb_complex_double alpha1, const double *d1, int ldd1,
    const sgb_complex_double alpha2, const double *d2, int ldd2, const double *a, int inca,
    int lda, const sgb_complex_double beta, sgb_complex_double *b, int incb, int ldb);
int suzerain_blasext_zgb_ddddiag_scale_acc_d(
    char side, int m, int n, int kl, int ku, const sgb_complex_double alpha0, const double *d0,
    int ldd0, const sgb_complex_double alpha1, const double *d1, int ldd1,
    const sgb_complex_double alpha2, const double *d2, int ldd2,
    const sgb_complex_double alpha3, const double *d3, int ldd3, const double *a, int inca,
    int lda, const sgb_complex_double beta, sgb_complex_double *b, int incb, int ldb);
int suzerain_blasext_zgb_dddddiag_scale_acc_d(
    char side, int m, int n, int kl, int ku, const sgb_complex_double alpha0, const double *d0,
    int ldd0, const sgb_complex_double alpha1, const double *d1, int ldd1,
    const sgb_complex_double alpha2, const double *d2, int ldd2,
    const sgb_complex_double alpha3, const double *d3, int ldd3,
    const sgb_complex_double alpha4, const double *d4, int ldd4, const double *a, int inca,
    int lda, const sgb_complex_double beta, sgb_complex_double *b, int incb, int ldb);
/** B <- alpha A + beta B for a real band A and complex band B;
 *  suzerain/blas_et_al/blas.c:1408-1421. */
int suzerain_blas_zgb_acc_d(int m, int n, int kl, int ku, const sgb_complex_double alpha,
                            const double *a, int lda, const sgb_complex_double beta,
                            sgb_complex_double *b, int ldb);
/** In-place complex128 -> complex64 (demote) and back (promote), and the
 *  real forms; suzerain/blas_et_al/blasext.c:2780-2866. */
int suzerain_blasext_zdemote(const int n, void *x);
int suzerain_blasext_zpromote(const int n, void *x);
int suzerain_blasext_ddemote(const int n, void *x);
int suzerain_blasext_dpromote(const int n, void *x);
/** Maximum column sum of |a_ij| over an m x n complex band;
 *  suzerain/blas_et_al/blasext.c:2741-2778. */
int suzerain_blasext_zgbnorm1(const int m, const int n, const int kl, const int ku,
                              const sgb_complex_double *a, const int lda, double *norm1);
/** The real form, dgbnorm1 (suzerain/blas_et_al/blasext.c:2659-2700). */
int suzerain_blasext_dgbnorm1(const int m, const int n, const int kl, const int ku,
                              const double *a, const int lda, double *norm1);

/* ---- The production implicit operator (suzerain/rholut_imexop.h) ------ */

/** suzerain/rholut_imexop.h:67-74. */
typedef struct suzerain_rholut_imexop_scenario {
    double Re, Pr, Ma, alpha, gamma;
} suzerain_rholut_imexop_scenario;
/** Wall-normal reference profiles; suzerain/rholut_imexop.h:77-104. */
typedef struct suzerain_rholut_imexop_ref {
    double *ux, *uy, *uz, *u2, *uxux, *uxuy, *uxuz, *uyuy, *uyuz, *uzuz;
    double *nu, *nuux, *nuuy, *nuuz, *nuu2, *nuuxux, *nuuxuy, *nuuxuz, *nuuyuy, *nuuyuz,
           *nuuzuz;
    double *ex_gradrho, *ey_gradrho, *ez_gradrho, *e_divm, *e_deltarho;
} suzerain_rholut_imexop_ref;
/** Strides of the profiles; suzerain/rholut_imexop.h:107-134. */
typedef struct suzerain_rholut_imexop_refld {
    int ux, uy, uz, u2, uxux, uxuy, uxuz, uyuy, uyuz, uzuz;
    int nu, nuux, nuuy, nuuz, nuu2, nuuxux, nuuxuy, nuuxuz, nuuyuy, nuuyuz, nuuzuz;
    int ex_gradrho, ey_gradrho, ez_gradrho, e_divm, e_deltarho;
} suzerain_rholut_imexop_refld;

/** y <- (M + phi L) x + beta y for one wavenumber pair (km, kn), equations
 *  E, u, v, w, rho (a NULL input and output pair omits an equation), with
 *  the optional non-reflecting upper boundary matrices a, b, c;
 *  suzerain/rholut_imexop.h:175-198, suzerain/rholut_imexop.c:43-545.
 *  Inputs and outputs are stride-one vectors of w->n, host or device. */
void suzerain_rholut_imexop_accumulate(
    const sgb_complex_double phi, const double km, const double kn,
    const suzerain_rholut_imexop_scenario *s, const suzerain_rholut_imexop_ref *r,
    const suzerain_rholut_imexop_refld *ld, const suzerain_bsplineop_workspace *w,
    const sgb_complex_double *in_rho_E, const sgb_complex_double *in_rho_u,
    const sgb_complex_double *in_rho_v, const sgb_complex_double *in_rho_w,
    const sgb_complex_double *in_rho, const sgb_complex_double beta,
    sgb_complex_double *out_rho_E, sgb_complex_double *out_rho_u,
    sgb_complex_double *out_rho_v, sgb_complex_double *out_rho_w,
    sgb_complex_double *out_rho, const double *a, const double *b, const double *c);
/** The km = kn = 0 form; suzerain/rholut_imexop.h:207-225. */
void suzerain_rholut_imexop_accumulate00(
    const sgb_complex_double phi, const suzerain_rholut_imexop_scenario *s,
    const suzerain_rholut_imexop_ref *r, const suzerain_rholut_imexop_refld *ld,
    const suzerain_bsplineop_workspace *w,
    const sgb_complex_double *in_rho_E, const sgb_complex_double *in_rho_u,
    const sgb_complex_double *in_rho_v, const sgb_complex_double *in_rho_w,
    const sgb_complex_double *in_rho, const sgb_complex_double beta,
    sgb_complex_double *out_rho_E, sgb_complex_double *out_rho_u,
    sgb_complex_double *out_rho_v, sgb_complex_double *out_rho_w,
    sgb_complex_double *out_rho, const double *c);
/** P (M + phi L)^T P^T into packc storage (A_T->LD x A_T->N) for gbmv and
 *  gbsvx; rho_E .. rho are the equations' positions (negative omits one);
 *  buf is not needed (the reference's working storage);
 *  suzerain/rholut_imexop.h:291-310, suzerain/rholut_imexop.def:41-594. */
void suzerain_rholut_imexop_packc(
    const sgb_complex_double phi, const double km, const double kn,
    const suzerain_rholut_imexop_scenario *s, const suzerain_rholut_imexop_ref *r,
    const suzerain_rholut_imexop_refld *ld, const suzerain_bsplineop_workspace *w,
    const int rho_E, const int rho_u, const int rho_v, const int rho_w, const int rho,
    sgb_complex_double *buf, suzerain_bsmbsm *A_T, sgb_complex_double *patpt,
    const double *a, const double *b, const double *c);
/** suzerain/rholut_imexop.h:324-340. */
void suzerain_rholut_imexop_packc00(
    const sgb_complex_double phi, const suzerain_rholut_imexop_scenario *s,
    const suzerain_rholut_imexop_ref *r, const suzerain_rholut_imexop_refld *ld,
    const suzerain_bsplineop_workspace *w,
    const int rho_E, const int rho_u, const int rho_v, const int rho_w, const int rho,
    sgb_complex_double *buf, suzerain_bsmbsm *A_T, sgb_complex_double *patpt,
    const double *c);
/** The same into packf storage ((A_T->LD + A_T->KL) x A_T->N, the band
 *  from row A_T->KL; the rows above it are left as they were) for gbtrf;
 *  suzerain/rholut_imexop.h:406-425. */
void suzerain_rholut_imexop_packf(
    const sgb_complex_double phi, const double km, const double kn,
    const suzerain_rholut_imexop_scenario *s, const suzerain_rholut_imexop_ref *r,
    const suzerain_rholut_imexop_refld *ld, const suzerain_bsplineop_workspace *w,
    const int rho_E, const int rho_u, const int rho_v, const int rho_w, const int rho,
    sgb_complex_double *buf, suzerain_bsmbsm *A_T, sgb_complex_double *patpt,
    const double *a, const double *b, const double *c);
/** suzerain/rholut_imexop.h:439-455. */
void suzerain_rholut_imexop_packf00(
    const sgb_complex_double phi, const suzerain_rholut_imexop_scenario *s,
    const suzerain_rholut_imexop_ref *r, const suzerain_rholut_imexop_refld *ld,
    const suzerain_bsplineop_workspace *w,
    const int rho_E, const int rho_u, const int rho_v, const int rho_w, const int rho,
    sgb_complex_double *buf, suzerain_bsmbsm *A_T, sgb_complex_double *patpt,
    const double *c);

/** 0.5 (1 + tanh(delta (x/L - 1/2)) / tanh(delta/2)); suzerain/htstretch.c:112-125. */
double suzerain_htstretch2(const double delta, const double L, const double x);
/** Signed wavenumber of in-order index i; suzerain/inorder.h:92-96. */
int suzerain_inorder_wavenumber(const int N, const int i);

/** Scale complex wave-space field x (Ny x Nx x Nz, column-major, Y fastest)
 *  by alpha (i kx)^dxcnt (i kz)^dzcnt, zeroing dealiased and Nyquist modes;
 *  suzerain/diffwave.h:90-97, suzerain/diffwave.c:66-131. */
int suzerain_diffwave_apply(const int dxcnt, const int dzcnt,
                            const sgb_complex_double alpha,
                            sgb_complex_double *x, const double Lx,
                            const double Lz, const int Ny, const int Nx,
                            const int dNx, const int dkbx, const int dkex,
                            const int Nz, const int dNz, const int dkbz,
                            const int dkez);

/** y <- alpha (i kx)^dxcnt (i kz)^dzcnt x + beta y on the same layout, with
 *  y <- beta y on dealiased and Nyquist modes; x and y must not alias
 *  (returns -1, where the reference asserts); suzerain/diffwave.h:142-151,
 *  suzerain/diffwave.c:132-198. */
int suzerain_diffwave_accumulate(const int dxcnt, const int dzcnt,
                                 const sgb_complex_double alpha,
                                 const sgb_complex_double *x,
                                 const sgb_complex_double beta, sgb_complex_double *y,
                                 const double Lx, const double Lz, const int Ny,
                                 const int Nx, const int dNx, const int dkbx,
                                 const int dkex, const int Nz, const int dNz,
                                 const int dkbz, const int dkez);

/** Diagonally scaled band matvecs of the explicit operator,
 *  y <- (alpha0 D0 + ... ) op(A) x + beta y with one to five real diagonals
 *  (entry i of D_t at d_t[i*ldd_t], ldd_t >= 0), a real n x n band A in BLAS
 *  band storage (lda > kl + ku), x complex (_d_z) or real (_d_d), alpha_t,
 *  beta and y complex; op(A) = A for 'N', A^T for 'T' and 'C'.  Argument
 *  errors return the position the reference reports to xerbla (ldd_t at
 *  7 + 3t, then lda, incx, incy); suzerain/blas_et_al/blasext.h:202-1000,
 *  suzerain/blas_et_al/gbdmv.def ... gbdddddmv.def.  Host or device
 *  pointers; the computation runs on the GPU. */
int suzerain_blasext_zgbdmv_d_z(const char trans, const int n, const int kl, const int ku,
    const sgb_complex_double alpha0, const double *d0, const int ldd0,
    const double *a, const int lda, const sgb_complex_double *x, const int incx,
    const sgb_complex_double beta, sgb_complex_double *y, const int incy);
int suzerain_blasext_zgbdmv_d_d(const char trans, const int n, const int kl, const int ku,
    const sgb_complex_double alpha0, const double *d0, const int ldd0,
    const double *a, const int lda, const double *x, const int incx,
    const sgb_complex_double beta, sgb_complex_double *y, const int incy);
int suzerain_blasext_zgbddmv_d_z(const char trans, const int n, const int kl, const int ku,
    const sgb_complex_double alpha0, const double *d0, const int ldd0, const sgb_complex_double alpha1, const double *d1, const int ldd1,
    const double *a, const int lda, const sgb_complex_double *x, const int incx,
    const sgb_complex_double beta, sgb_complex_double *y, const int incy);
int suzerain_blasext_zgbddmv_d_d(const char trans, const int n, const int kl, const int ku,
    const sgb_complex_double alpha0, const double *d0, const int ldd0, const sgb_complex_double alpha1, const double *d1, const int ldd1,
    const double *a, const int lda, const double *x, const int incx,
    const sgb_complex_double beta, sgb_complex_double *y, const int incy);
int suzerain_blasext_zgbdddmv_d_z(const char trans, const int n, const int kl, const int ku,
    const sgb_complex_double alpha0, const double *d0, const int ldd0, const sgb_complex_double alpha1, const double *d1, const int ldd1, const sgb_complex_double alpha2, const double *d2, const int ldd2,
    const double *a, const int lda, const sgb_complex_double *x, const int incx,
    const sgb_complex_double beta, sgb_complex_double *y, const int incy);
int suzerain_blasext_zgbdddmv_d_d(const char trans, const int n, const int kl, const int ku,
    const sgb_complex_double alpha0, const double *d0, const int ldd0, const sgb_complex_double alpha1, const double *d1, const int ldd1, const sgb_complex_double alpha2, const double *d2, const int ldd2,
    const double *a, const int lda, const double *x, const int incx,
    const sgb_complex_double beta, sgb_complex_double *y, const int incy);
int suzerain_blasext_zgbddddmv_d_z(const char trans, const int n, const int kl, const int ku,
    const sgb_complex_double alpha0, const double *d0, const int ldd0, const sgb_complex_double alpha1, const double *d1, const int ldd1, const sgb_complex_double alpha2, const double *d2, const int ldd2, const sgb_complex_double alpha3, const double *d3, const int ldd3,
    const double *a, const int lda, const sgb_complex_double *x, const int incx,
    const sgb_complex_double beta, sgb_complex_double *y, const int incy);
int suzerain_blasext_zgbddddmv_d_d(const char trans, const int n, const int kl, const int ku,
    const sgb_complex_double alpha0, const double *d0, const int ldd0, const sgb_complex_double alpha1, const double *d1, const int ldd1, const sgb_complex_double alpha2, const double *d2, const int ldd2, const sgb_complex_double alpha3, const double *d3, const int ldd3,
    const double *a, const int lda, const double *x, const int incx,
    const sgb_complex_double beta, sgb_complex_double *y, const int incy);
int suzerain_blasext_zgbdddddmv_d_z(const char trans, const int n, const int kl, const int ku,
    const sgb_complex_double alpha0, const double *d0, const int ldd0, const sgb_complex_double alpha1, const double *d1, const int ldd1, const sgb_complex_double alpha2, const double *d2, const int ldd2, const sgb_complex_double alpha3, const double *d3, const int ldd3, const sgb_complex_double alpha4, const double *d4, const int ldd4,
    const double *a, const int lda, const sgb_complex_double *x, const int incx,
    const sgb_complex_double beta, sgb_complex_double *y, const int incy);
int suzerain_blasext_zgbdddddmv_d_d(const char trans, const int n, const int kl, const int ku,
    const sgb_complex_double alpha0, const double *d0, const int ldd0, const sgb_complex_double alpha1, const double *d1, const int ldd1, const sgb_complex_double alpha2, const double *d2, const int ldd2, const sgb_complex_double alpha3, const double *d3, const int ldd3, const sgb_complex_double alpha4, const double *d4, const int ldd4,
    const double *a, const int lda, const double *x, const int incx,
    const sgb_complex_double beta, sgb_complex_double *y, const int incy);

/** Solver specification (suzerain/specification_zgbsv.hpp:44-140): the
 *  method and the zcgbsvx refinement parameters.  Defaults (empty string):
 *  zcgbsvx, equil = reuse = false, aiter = 1, siter = -1, diter = 5,
 *  tolsc = 0 (suzerain/specification_zgbsv.cpp:46-54). */
enum { SGB_METHOD_ZGBSV = 1, SGB_METHOD_ZGBSVX = 2, SGB_METHOD_ZCGBSVX = 3 };
typedef struct sgb_solver_spec {
    int method, equil, reuse, aiter, siter, diter;
    double tolsc;
} sgb_solver_spec;
void sgb_solver_spec_default(sgb_solver_spec *s);
/** Parse "zgbsv" | "zgbsvx[,equil=B]" | "zcgbsvx[,reuse=B][,aiter=I][,siter=I]
 *  [,diter=I][,tolsc=D]" (options in any order, each once; keywords
 *  case-insensitive; whitespace anywhere between tokens), the grammar of
 *  suzerain/specification_zgbsv.cpp:56-104.  Returns 0, or -1 with the
 *  reference's message ("... invalid beginning with '...'") in err. */
int sgb_solver_spec_parse(const char *spec, sgb_solver_spec *out, char *err, size_t errlen);
/** The reference's canonical string (suzerain/specification_zgbsv.cpp:128-155). */
int sgb_solver_spec_format(const sgb_solver_spec *s, char *buf, size_t len);

/* ======================================================================== */
/* 2. Batched device API                                                    */
/* ======================================================================== */

/** Last error message of this thread (static storage). */
const char *sgb_last_error(void);
/** 0 when a CUDA device of compute capability 10.3 is usable. */
int sgb_device_ok(void);

/** Complex elements of one system's row-panel LU factor:
 *  N rows of U (KL+KU+1 each) then N columns of L (KL each). */
long long sgb_factor_elems(int N, int KL, int KU);

/** Batched partial-pivot LU of nsys packed bands (complex128, LAPACK packc
 *  layout, ldab >= KL+KU+1 rows, system s at ab + s*ab_stride).  prec 'Z'
 *  factors in complex128, 'C' in complex64 (the band is demoted on load).
 *  fac: nsys * sgb_factor_elems complex of prec; ipiv nsys*N (1-based);
 *  info nsys (zgbtrf semantics). */
int sgb_gbtrf_batched(char prec, int nsys, int N, int KL, int KU,
                      const void *ab, int ldab, long long ab_stride,
                      void *fac, int *ipiv, int *info, void *stream);

/** sgb_gbtrf_batched with the kernel chosen explicitly: variant 0 is the
 *  blocked kernel with panel width nb (4, 8 or 16) and nw warps per system
 *  (1, 2 or 4; KL <= 52, 56, 63 respectively; N < 65536; nw 3 for complex64
 *  with nb 4, KL = KU = 24 or 34 and N a multiple of 4), variant 2 its
 *  lookahead form (nw 2 or 4: the next panel is factored while the other
 *  warps apply the previous panel's update), variant 1 the unblocked kernel
 *  (nb, nw ignored).  nb or nw 0 takes the shape recorded by
 *  sgb_gbtrf_set_shape for (prec, N, KL, KU), else the built-in default.
 *  Every shape produces zgbtf2's pivots and factor, bit for bit. */
int sgb_gbtrf_batched_ex(char prec, int nsys, int N, int KL, int KU,
                         const void *ab, int ldab, long long ab_stride,
                         void *fac, int *ipiv, int *info, int variant, int nb,
                         int nw, void *stream);

/** Diagnostics: the blocked factor with cycle counters.  cycles_dev (10
 *  device uint64, accumulated) receives the clock cycles the first warp of
 *  every system spent in initial load, panel, interchanges+U12, GEMM, U
 *  output, retire/load (waits at the phase barriers included), then inside
 *  the panel: pivot search, reciprocal + scale + L store, rank-1 update and
 *  loop; nw < 0 selects the lookahead form with -nw warps. */
int sgb_gbtrf_phase_cycles(char prec, int nsys, int N, int KL, int KU,
                           const void *ab, int ldab, long long ab_stride,
                           void *fac, int *ipiv, int *info, int nb, int nw,
                           unsigned long long *cycles_dev, void *stream);

/** Diagnostics: pipe-throughput microbenchmarks of the current device (the
 *  denominators the factor and residual kernels are compared with).  out
 *  (7 host doubles) receives FP64 FMA TFLOP/s, FP32 FMA TFLOP/s, packed
 *  two-lane FP32 FMA TFLOP/s, shared-memory load bandwidth TB/s, the same in
 *  bytes per SM per clock at the device's reported maximum SM clock, that
 *  clock in MHz, and the SM count. */
int sgb_measure_peaks(double *out, void *stream);

/** Process-wide shape table of the blocked factor, keyed (prec, N, KL, KU):
 *  set records (nb, nw) for every later factorization of that geometry (the
 *  plan and the refinement driver included); get reports the shape in force.
 *  nw = -2 or -4 records the lookahead form.  The tuner
 *  (suzerain_gb300.tune) times the candidates and calls set. */
int sgb_gbtrf_set_shape(char prec, int N, int KL, int KU, int nb, int nw);
int sgb_gbtrf_get_shape(char prec, int N, int KL, int KU, int *nb, int *nw);

/** Batched solve op(A) x = b with row-panel factors; b, x complex128
 *  (nsys x N, stride N).  x may equal b. */
int sgb_gbtrs_batched(char prec, char trans, int nsys, int N, int KL, int KU,
                      const void *fac, const int *ipiv, const void *b,
                      void *x, void *stream);

/** sgb_gbtrs_batched with caller scratch: ywork (nsys x N complex of prec,
 *  device memory) lets trans 'N' run the four-lanes-per-system sweeps (eight
 *  systems per warp).  Same result up to the summation order of the row dot
 *  products; other trans values ignore ywork. */
int sgb_gbtrs_batched_ws(char prec, char trans, int nsys, int N, int KL, int KU,
                         const void *fac, const int *ipiv, const void *b,
                         void *x, void *ywork, void *stream);

/** One row-panel factor (fac, ipiv of one system) solved for nrhs
 *  right-hand sides in one launch: column r of b (complex128, leading
 *  dimension ldb >= N) gives column r of x (ldx >= N); x may equal b when
 *  ldx == ldb.  ywork (nrhs x N complex of prec, or NULL) enables the
 *  four-lanes-per-system sweeps for trans 'N'.  Replaces the per-column
 *  zgbtrs loop of a bsmbsm_solver with nrhs > 1 and a reused factor
 *  (suzerain/bsmbsm_solver.cpp:80-102, :155-182; the wavenumber-independent
 *  operator of apps/perfect/operator_hybrid_isothermal.cpp:691-760). */
int sgb_gbtrs_shared(char prec, char trans, int nrhs, int N, int KL, int KU,
                     const void *fac, const int *ipiv, const void *b, long long ldb,
                     void *x, long long ldx, void *ywork, void *stream);

/** Batched zgbsvx: nsys systems of one geometry, one right-hand side each,
 *  every pointer on the device (rcond, ferr, berr, rpvgrw may also be host
 *  memory).  Per system: ab (ld ldab, stride ab_stride; overwritten by the
 *  equilibrated band), afb (LAPACK gbtrf storage, ld ldafb, stride
 *  afb_stride; input for fact 'F', output otherwise, may be null unless
 *  'F'), ipiv / r / c / b / x of n entries, equed / info of one.  Returns 0
 *  or a negative argument index; per-system results follow zgbsvx. */
int sgb_zgbsvx_batched(char fact, char trans, int nsys, int n, int kl, int ku,
                       sgb_complex_double *ab, int ldab, long long ab_stride,
                       sgb_complex_double *afb, int ldafb, long long afb_stride,
                       int *ipiv, char *equed, double *r, double *c,
                       sgb_complex_double *b, sgb_complex_double *x,
                       double *rcond, double *ferr, double *berr, double *rpvgrw,
                       int *info, void *stream);

/** Records in flight per system of the quad-lane solves (trans 'N' with a
 *  y workspace): 2, 4, 8 or 16 for the forward and the backward sweep (0
 *  keeps the current value; defaults 2 and 2).  Returns -1 for other values.
 *  Process-wide; results do not depend on it. */
int sgb_gbtrs_set_quad_depth(int fwd, int bwd);
/** Backward quad-lane solve, rows per factor record: 2 (the default), 4 or
 *  8 consecutive U rows arrive by one bulk copy (1-D TMA, completion on an
 *  mbarrier) per record and system; 0 or 1: one row by 16-byte cp.async
 *  spread over the system's four lanes.  Results are identical. */
int sgb_gbtrs_set_quad_bulk(int rows);
/** Complex64 blocked factor: instances with the bandwidths fixed at compile
 *  time (KL = KU = 24 or 34 with N a multiple of 4, the geometries of S = 5
 *  or 7 equations at B-spline order 6 or 8 whose window leaves room for 8
 *  systems per SM) on (1, the default) or off (0: every geometry takes the
 *  generic instance).  Process-wide; the factors are bit-identical either
 *  way. */
int sgb_gbtrf_set_specialized(int on);
/** Kernels that wait on asynchronous copies bound every wait; one whose
 *  wait ran out records a fault (its results are invalid).  Returns the
 *  number recorded since the last call (0 or 1) and clears the record; -1
 *  if the device cannot be read. */
int sgb_async_faults(void);

/** Row-panel factor -> LAPACK gbtrf storage ((2KL+KU+1) x N per system). */
int sgb_factor_to_lapack(char prec, int nsys, int N, int KL, int KU,
                         const void *fac, void *ab, void *stream);

/** Refinement controls, the parameters of the zcgbsvx spec string. */
typedef struct sgb_refine_spec {
    int aiter, siter, diter;
    double tolsc;
} sgb_refine_spec;

/** Per-system outputs of the mixed-precision driver (device pointers, any
 *  may be NULL). fact: 'S' or 'D' per system. */
typedef struct sgb_refine_report {
    int *info, *siter, *diter;
    double *res, *tolsc;
    char *fact;
} sgb_refine_report;

/** Batched zcgbsvx over packed complex128 bands: b, x permuted complex128
 *  (nsys x N).  Allocates its workspace internally on first use. */
int sgb_zcgbsvx_batched(int nsys, int N, int KL, int KU, char trans,
                        const void *ab, int ldab, long long ab_stride,
                        const void *b, void *x, const sgb_refine_spec *spec,
                        const sgb_refine_report *report, void *stream);

/** sgb_zcgbsvx_batched for callers that cannot allocate device memory
 *  (hosts that reserve all of HBM in their own arena, or solver loops that
 *  must not enter the driver's allocator once stepping has begun).  Same
 *  arguments and results; no counterpart in the reference.  It calls no
 *  cudaMalloc/cudaFree and no allocating library routine: its scratch is a
 *  fixed 64 MiB __device__ array inside this library, which every GPU that
 *  loads the library holds until process exit.  Problems whose scratch
 *  exceeds 64 MiB are rejected with an error naming both sizes: at N = 960,
 *  KL = KU = 34 the scratch is 6.3 MB for four complex128 fallback slots
 *  (fallback systems pass through them four at a time) plus 0.82 MB per
 *  system, so up to 74 systems per call.  Argument errors return the codes
 *  of sgb_zcgbsvx_batched.  The first call on a device
 *  looks up the array's device address (cudaGetSymbolAddress) with that
 *  device current; make that first call before any stream capture.  All
 *  calls share the one array: calls that overlap on the GPU (different
 *  streams without synchronization) race; the kernels initialise every
 *  value they read, so one call's leftovers never affect the next. */
int sgb_zcgbsvx_batched_static(int nsys, int N, int KL, int KU, char trans,
                               const void *ab, int ldab, long long ab_stride,
                               const void *b, void *x,
                               const sgb_refine_spec *spec,
                               const sgb_refine_report *report, void *stream);

/** One synthetic case (see sgb_case in the model header): bands and
 *  coefficients.  For sgb_plan_create the pointers are HOST pointers. */
typedef struct sgb_case {
    int S, n, kl, ku, ld;
    const double *M, *D1, *D2;
    const double *a, *b, *c, *g;
    unsigned dirichlet_mask;
    int pad_;
} sgb_case;

/** A resident batch: one case, nsys wavenumber pairs, device workspace. */
typedef struct sgb_plan sgb_plan;

sgb_plan *sgb_plan_create(const sgb_case *host_case, int nsys,
                          const double *kx, const double *kz,
                          int max_double_slots);
int sgb_plan_destroy(sgb_plan *p);
/** Device bytes the plan will hold after its first substep of method
 *  ('M', 'Z', or 0 for both), computed without allocating: admission
 *  control against a memory budget. */
size_t sgb_plan_estimate_bytes(const sgb_case *host_case, int nsys, int max_double_slots,
                               char method);
/** Device bytes the plan holds. */
size_t sgb_plan_device_bytes(const sgb_plan *p);
/** Plans draw device memory from a stream-ordered pool that keeps freed
 *  blocks for the next plan; this returns cached blocks beyond keep_bytes
 *  to the device. */
int sgb_plan_pool_trim(size_t keep_bytes);

/** One implicit substep for every system of the plan:
 *    y = P (M + phi_exp L) u          (explicit operator, Dirichlet rows 0)
 *    (M + phi_imp L) x = y            method 'Z': complex128 LU (zgbsv)
 *                                     method 'M': complex64 LU + FP64 refine
 *    u_out = P^T x
 *  u_in/u_out: device, nsys x N complex128, natural (unpermuted) order.
 *  phi_exp == 0 skips the explicit apply and uses u_in as y (P applied). */
int sgb_plan_substep(sgb_plan *p, char method, double phi_exp, double phi_imp,
                     const void *u_in, void *u_out,
                     const sgb_refine_spec *spec, void *stream);

/** sgb_plan_substep in a form that can be recorded into a CUDA graph: no
 *  host synchronization, allocation or host-to-device copy.  Call
 *  sgb_plan_substep once with the same method first (it allocates the
 *  workspace; sgb_plan_prepare does the allocation alone).  Method 'M' runs
 *  the reference's bounds: up to siter + 1 complex64 correction solves and,
 *  for systems that leave for complex128, up to diter + 2 corrections;
 *  every launch of the loop is issued and its grid is bounded by a
 *  device-side count, so once every system has converged the remaining
 *  launches exit at once.  The complex128 fallback runs one chunk of at
 *  most max_double_slots systems.  sgb_plan_unserved reports, after the work has
 *  run, how many fallback systems did not fit the chunk (their solution is
 *  the complex64 one, flagged fact = 'S' with tolsc > 1). */
int sgb_plan_substep_capturable(sgb_plan *plan, char method, double phi_exp,
                                double phi_imp, const void *u_in, void *u_out,
                                const sgb_refine_spec *spec, void *stream);
int sgb_plan_unserved(sgb_plan *plan, int *count);
/** Allocate what the first substep of method ('M', 'Z', or 0 for both)
 *  would, so that every substep can then take the capturable form. */
int sgb_plan_prepare(sgb_plan *plan, char method);

/** The capturable mixed substep (method 'M', siter >= 0) in two stages
 *  around an external complex64 factor: stage 1 runs the explicit operator
 *  and the refinement's initial state, stage 2 everything after the factor.
 *  Stage 1 of every plan of a ragged batch, sgb_ragged_factor, then stage 2
 *  of every plan give sgb_plan_substep_capturable's results bit for bit.
 *  Replaces, for a batch of wavenumber sets, the per-set factor loop of the
 *  reference's implicit solve (suzerain/bsmbsm_solver.cpp:443 and
 *  suzerain/bsmbsm_solver.cpp:1009, zgbtrf of each set's packed band). */
int sgb_plan_substep_stage(sgb_plan *plan, int stage, char method, double phi_exp,
                           double phi_imp, const void *u_in, void *u_out,
                           const sgb_refine_spec *spec, void *stream);

/** A ragged batch: the complex64 factors of several plans' mixed substeps
 *  (each plan at its own phi_imp, up to KL = 56, S <= 8) as one launch per
 *  row-tile class (KL <= 40, KL <= 56), the systems of the largest plans
 *  first.  Every plan needs its mixed workspace (one
 *  sgb_plan_substep with 'M', or sgb_plan_prepare) before creation; the
 *  batch reads the plans' workspaces, so the plans outlive it. */
typedef struct sgb_ragged sgb_ragged;
sgb_ragged *sgb_ragged_create(sgb_plan *const *plans, int nplans, const double *phi_imp,
                              const sgb_refine_spec *spec);
int sgb_ragged_factor(sgb_ragged *batch, void *stream);
void sgb_ragged_destroy(sgb_ragged *batch);

/** Same, from and to host memory (copies inside the call). */
int sgb_plan_substep_host(sgb_plan *p, char method, double phi_exp,
                          double phi_imp, const void *u_in_host,
                          void *u_out_host, const sgb_refine_spec *spec,
                          void *stream);

/** The production operator resident on the device for batched use: the
 *  collocation bands of w, the reference profiles (host pointers with the
 *  strides of ld, copied), the equation positions order[5] (E, u, v, w,
 *  rho; negative omits) and the optional boundary matrices a, b, c (host,
 *  5 x 5 column-major; they need all five equations in order).  No
 *  counterpart in the reference, whose callers pack one wavenumber pair at
 *  a time (apps/perfect/operator_hybrid_isothermal.cpp:612-689). */
typedef struct sgb_rholut sgb_rholut;
sgb_rholut *sgb_rholut_create(const suzerain_rholut_imexop_scenario *s,
                              const suzerain_rholut_imexop_ref *r,
                              const suzerain_rholut_imexop_refld *ld,
                              const suzerain_bsplineop_workspace *w, const int order[5],
                              const double *a, const double *b, const double *c);
int sgb_rholut_destroy(sgb_rholut *h);
/** The BSMBSM geometry of the packed operator. */
int sgb_rholut_geometry(const sgb_rholut *h, suzerain_bsmbsm *A_T);
/** P (M + phi L)^T P^T for nsys wavenumber pairs (km, kn: device arrays)
 *  into packed bands ab (device): entry (R, C) at
 *  ab[s ab_stride + off + KU + R - C + C ldab]; off = 0, ldab = LD is
 *  packc, off = KL, ldab = LD + KL packf (rows above off untouched). */
int sgb_rholut_pack_batched(sgb_rholut *h, double phi_re, double phi_im, int nsys,
                            const double *km, const double *kn, void *ab, int ldab,
                            long long ab_stride, int off, void *stream);
/** y <- (M + phi L) x + beta y for nsys wavenumber pairs; x, y device,
 *  natural order per system (equation position p at p n .. p n + n - 1). */
int sgb_rholut_accumulate_batched(sgb_rholut *h, double phi_re, double phi_im, int nsys,
                                  const double *km, const double *kn, const void *x,
                                  long long x_stride, double beta_re, double beta_im,
                                  void *y, long long y_stride, void *stream);

/** The implicit operator M + phi L of every system of the plan, written as
 *  packed complex128 bands (device memory): A(r, c) at
 *  ab[s ab_stride + off + KU + r - c + c ldab]; the other rows of each
 *  column and positions outside the matrix are zero.  off = 0 with
 *  ldab = KL + KU + 1 is the packc layout that zcgbsvx reads
 *  (suzerain/bsmbsm.h:543-610), off = KL with ldab = 2 KL + KU + 1 the packf
 *  layout of zgbsv.  The caller-packed form of the solve then runs through
 *  sgb_zcgbsvx_batched on these bands. */
int sgb_plan_assemble_packed(sgb_plan *p, double phi, void *ab, int ldab,
                             long long ab_stride, int off, void *stream);

/** Copy the last substep's per-system statistics to host arrays (any may be
 *  NULL): info, siter, diter, res (||r||_2), tolsc, fact ('S'/'D'). */
int sgb_plan_report(const sgb_plan *p, int *info, int *siter, int *diter,
                    double *res, double *tolsc, char *fact);

/** Normwise backward error ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf)
 *  of the last substep for every system, computed in FP64 on the device. */
int sgb_plan_backward_error(sgb_plan *p, double *berr_host, void *stream);

/** A batch: one case's nsys systems split into `parts` resident plans over
 *  consecutive rows (sgb_batch_bounds), each substepped on a stream of its
 *  own that is forked from and joined back into the caller's stream, in the
 *  capturable form (no host synchronization inside, so the parts overlap on
 *  the device; the calls record into a CUDA graph being captured on the
 *  caller's stream).  max_double_slots is the batch's total of complex128
 *  fallback slots, shared evenly by the parts.  Results equal one plan's
 *  capturable substep over the whole batch.  No counterpart in the
 *  reference: its caller loops over wavenumbers one solver at a time
 *  (apps/perfect/operator_hybrid_isothermal.cpp:612-689). */
typedef struct sgb_batch sgb_batch;
/** Row offsets of the parts: bounds[i] = i nsys / parts (integer division),
 *  parts + 1 entries (parts clamped to nsys); returns the part count. */
int sgb_batch_bounds(int nsys, int parts, int *bounds);
sgb_batch *sgb_batch_create(const sgb_case *host_case, int nsys, const double *kx,
                            const double *kz, int parts, int max_double_slots,
                            char method);
int sgb_batch_destroy(sgb_batch *b);
int sgb_batch_parts(const sgb_batch *b);
/** The plan of one part (owned by the batch). */
sgb_plan *sgb_batch_plan(sgb_batch *b, int part);
size_t sgb_batch_device_bytes(const sgb_batch *b);
/** sgb_plan_substep over the batch: device buffers nsys x N, natural order. */
int sgb_batch_substep(sgb_batch *b, char method, double phi_exp, double phi_imp,
                      const void *u_in, void *u_out, const sgb_refine_spec *spec,
                      void *stream);
/** The same from and to HOST buffers (pinned for overlap): each part copies
 *  its rows in, substeps and copies them out on its own stream, so copies
 *  of one part overlap the computation of the others; returns when the
 *  output is in host memory. */
int sgb_batch_substep_host(sgb_batch *b, char method, double phi_exp, double phi_imp,
                           const void *u_in_host, void *u_out_host,
                           const sgb_refine_spec *spec, void *stream);
int sgb_batch_report(const sgb_batch *b, int *info, int *siter, int *diter,
                     double *res, double *tolsc, char *fact);
int sgb_batch_backward_error(sgb_batch *b, double *berr_host, void *stream);
int sgb_batch_unserved(sgb_batch *b, int *count);

/** Record CUDA events around each phase of later substeps (on the stream
 *  they run in); sgb_plan_timings returns "name total_ms calls" lines. */
int sgb_plan_set_timing(sgb_plan *p, int on);
int sgb_plan_timings(sgb_plan *p, char *buf, int buflen);
/** Kernels this library has launched since load (all entry points). */
long long sgb_launch_count(void);

/** Synthetic inputs (host): seeded B-spline case and right-hand sides. */
int sgb_synth_case(int S, int Ny, int k, double htdelta, double left,
                   double right, double offscale, int complex_coupling,
                   uint64_t seed, unsigned dirichlet_mask, int *kl, int *ku,
                   double *M, double *D1, double *D2, double *a, double *b,
                   double *c, double *g);
int sgb_synth_wavenumbers(int Nx, int Nz, double Lx, double Lz, double *kx,
                          double *kz);
int sgb_synth_rhs(uint64_t seed, long long nsys, int N, double *u);

#ifdef __cplusplus
}
#endif

#endif /* SUZERAIN_GB300_H */
