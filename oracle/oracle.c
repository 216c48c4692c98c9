/*
 * ORACLE — test infrastructure, not product code.
 *
 * A plain-C restatement of the reference's banded implicit-solve path, used
 * only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as
 * the checker.  Nothing in suzerain_gb300/ links or calls it.
 *
 * What it restates, with the reference lines it follows:
 *   q / qinv                suzerain/bsmbsm.h:162-186
 *   aPxpby ('N','T')        suzerain/bsmbsm_aPxpby_complex.def:36-329
 *   pack (z, zd)            suzerain/bsmbsm_pack.def:36-122
 *   gbmv (z; 'C' == 'T')    suzerain/blas_et_al/gbmv.def:46-201
 *   zcgbsvx                 suzerain/blas_et_al/dsgbsvx.def:70-313
 *   zgbsv                   suzerain/blas_et_al/lapackext.c:127-147
 * and the third-party LAPACK routines the reference gets from Intel MKL
 * (version unpinned, configure.ac:258), restated from the published
 * reference-LAPACK algorithms:
 *   zgbtf2 / cgbtf2         unblocked partial-pivot band LU (IZAMAX |re|+|im|
 *                           pivot metric, first index wins ties)
 *   zgbtrs / cgbtrs         band solve for 'N', 'T', 'C'
 *   zlangb('F'), dznrm2, dlamch('E')
 *   zgbsvx                  the expert driver (zgbequ, zlaqgb, zlangb, zgbcon
 *                           with zlacn2, zgbrfs), called by the reference at
 *                           suzerain/blas_et_al/lapack.c:548-574 and
 *                           suzerain/bsmbsm_solver.cpp:252-291
 * A runtime switch (orc_use_openblas) routes gbtrf/gbtrs to SciPy's bundled
 * OpenBLAS instead, so the CPU baseline runs production LAPACK code.
 *
 * Synthetic block assembly (orc_assemble_packed) follows the reference app's
 * pattern of building each S x S block from collocation bands and packing it
 * (apps/perfect/operator_hybrid_isothermal.cpp:640-661, suzerain/bsmbsm.h:407)
 * with Dirichlet identity rows in the manner of IsothermalPATPTEnforcer
 * (apps/perfect/operator_hybrid_isothermal.cpp:471-515).
 */
#include <complex.h>
#include <dlfcn.h>
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <ctype.h>

typedef double complex zc;
typedef float complex cc;

static inline int imin(int a, int b) { return a < b ? a : b; }
static inline int imax(int a, int b) { return a > b ? a : b; }

/* ------------------------------------------------------------------------ */
/* BSMBSM permutation (suzerain/bsmbsm.h:162-186)                           */
/* ------------------------------------------------------------------------ */
int orc_q(int S, int n, int i) { return (i % S) * n + i / S; }
int orc_qinv(int S, int n, int i) { return (i % n) * S + i / n; }

/* y <- alpha P x + beta y ('N') or alpha P^T x + beta y ('T'), where
 * (P x)_i = x_{q(i)}.  Returns BLAS-style positive argument positions on
 * error like the reference (1 trans, 2 S, 3 n, 58 aliasing). */
int orc_zaPxpby(char trans, int S, int n, zc alpha, const zc *x, int incx,
                zc beta, zc *y, int incy)
{
    if (S < 0) return 2;
    if (n < 0) return 3;
    if (x == y) return 58;
    switch (toupper((unsigned char) trans)) {
    case 'N': break;
    case 'T': { int t = S; S = n; n = t; } break;
    default: return 1;
    }
    const int N = S * n;
    const int ix0 = incx < 0 ? (1 - N) * incx : 0;
    const int iy0 = incy < 0 ? (1 - N) * incy : 0;
    const int beta_zero = (cimag(beta) == 0 && creal(beta) == 0);
    for (int i = 0; i < N; ++i) {
        const zc xv = x[ix0 + orc_q(S, n, i) * incx];
        zc *yp = y + iy0 + i * incy;
        if (beta_zero) *yp = alpha * xv;
        else           *yp = beta * (*yp) + alpha * xv;
    }
    return 0;
}

/* Scatter alpha*B^{ihat,jhat} into band storage of P A P^T and zero the
 * positions of that block which fall outside B's own band.  b is complex
 * (zpack) when bz != NULL, real (zdpack) when bd != NULL, absent when both
 * are NULL (alpha must then be 0). */
static int orc_pack_impl(int S, int n, int ihat, int jhat, int kl, int ku,
                         zc alpha, const zc *bz, const double *bd, int ldb,
                         int KL, int KU, zc *papt, int ldpapt)
{
    if (S < 0) return 1;
    if (n < 0) return 2;
    if (ihat < 0 || ihat >= S) return 3;
    if (jhat < 0 || jhat >= S) return 4;
    if (kl < 0) return 5;
    if (ku < 0) return 6;
    if (ldb < kl + 1 + ku) return 8;
    if (KL < S * (kl + 1) - 1) return 9;
    if (KU < S * (ku + 1) - 1) return 10;
    if (ldpapt < KL + 1 + KU) return 12;
    const int N = S * n;
    const int alpha_zero = (creal(alpha) == 0 && cimag(alpha) == 0);
    for (int bj = 0; bj < n; ++bj) {
        const int Cj = bj * S + jhat;                  /* qinv(jhat*n + bj) */
        for (int Ri = imax(0, Cj - KU); Ri <= imin(N - 1, Cj + KL); ++Ri) {
            if (Ri % S != ihat) continue;
            const int bi = Ri / S;
            zc v = 0;
            if (!alpha_zero && bj - ku <= bi && bi <= bj + kl) {
                const int o = ku + bi - bj + bj * ldb;
                v = alpha * (bz ? bz[o] : (zc) bd[o]);
            }
            papt[KU + Ri - Cj + Cj * ldpapt] = v;
        }
    }
    return 0;
}

int orc_zpack(int S, int n, int ihat, int jhat, int kl, int ku, zc alpha,
              const zc *b, int ldb, int KL, int KU, zc *papt, int ldpapt)
{
    return orc_pack_impl(S, n, ihat, jhat, kl, ku, alpha, b, NULL, ldb,
                         KL, KU, papt, ldpapt);
}

int orc_zdpack(int S, int n, int ihat, int jhat, int kl, int ku, zc alpha,
               const double *b, int ldb, int KL, int KU, zc *papt, int ldpapt)
{
    return orc_pack_impl(S, n, ihat, jhat, kl, ku, alpha, NULL, b, ldb,
                         KL, KU, papt, ldpapt);
}

/* ------------------------------------------------------------------------ */
/* Complex helpers: reciprocal per Smith (1962), explicit real arithmetic    */
/* ------------------------------------------------------------------------ */
static inline zc zrcp(zc z)
{
    const double a = creal(z), b = cimag(z);
    if (fabs(a) >= fabs(b)) {
        const double r = b / a, d = a + b * r;
        return CMPLX(1.0 / d, -r / d);
    } else {
        const double r = a / b, d = a * r + b;
        return CMPLX(r / d, -1.0 / d);
    }
}
static inline cc crcp(cc z)
{
    const float a = crealf(z), b = cimagf(z);
    if (fabsf(a) >= fabsf(b)) {
        const float r = b / a, d = a + b * r;
        return CMPLXF(1.0f / d, -r / d);
    } else {
        const float r = a / b, d = a * r + b;
        return CMPLXF(r / d, -1.0f / d);
    }
}
static inline zc zmul(zc a, zc b)
{
    return CMPLX(creal(a) * creal(b) - cimag(a) * cimag(b),
                 creal(a) * cimag(b) + cimag(a) * creal(b));
}
static inline cc cmul(cc a, cc b)
{
    return CMPLXF(crealf(a) * crealf(b) - cimagf(a) * cimagf(b),
                  crealf(a) * cimagf(b) + cimagf(a) * crealf(b));
}
static inline zc zdiv(zc a, zc b) { return zmul(a, zrcp(b)); }
static inline cc cdiv(cc a, cc b) { return cmul(a, crcp(b)); }

/* ------------------------------------------------------------------------ */
/* zgbtf2 / cgbtf2 restatement (partial-pivot band LU, in place)            */
/* ab is (2*kl+ku+1) x n column-major; A(i,j) at ab[kl+ku+i-j + j*ldab]      */
/* ------------------------------------------------------------------------ */
#define DEFINE_GBTF2(NAME, T, RCP, MUL, ABS1)                                  \
int NAME(int n, int kl, int ku, T *ab, int ldab, int *ipiv)                 \
{                                                                            \
    if (n < 0) return -2;                                                    \
    if (kl < 0) return -3;                                                   \
    if (ku < 0) return -4;                                                   \
    if (ldab < 2 * kl + ku + 1) return -6;                                   \
    const int kv = ku + kl;                                                  \
    int info = 0;                                                            \
    /* zero the fill-in rows of columns ku+1 .. kv-1 (0-based) */            \
    for (int j = ku + 1; j < imin(kv, n); ++j)                               \
        for (int i = kv - j; i < kl; ++i) ab[i + j * ldab] = 0;              \
    int ju = 0;                                                              \
    for (int j = 0; j < n; ++j) {                                            \
        if (j + kv < n)                                                      \
            for (int i = 0; i < kl; ++i) ab[i + (j + kv) * ldab] = 0;        \
        const int km = imin(kl, n - 1 - j);                                  \
        T *col = ab + kv + j * ldab;           /* A(j..j+km, j) */           \
        int jp = 0;                                                          \
        double best = ABS1(col[0]);                                          \
        for (int i = 1; i <= km; ++i) {                                      \
            const double v = ABS1(col[i]);                                   \
            if (v > best) { best = v; jp = i; }                              \
        }                                                                    \
        ipiv[j] = jp + j + 1;                  /* 1-based like LAPACK */     \
        if (col[jp] != 0) {                                                  \
            ju = imax(ju, imin(j + ku + jp, n - 1));                         \
            if (jp != 0) {                                                   \
                for (int c = 0; c <= ju - j; ++c) {                          \
                    T *a = ab + kv + jp - c + (j + c) * ldab;                \
                    T *b = ab + kv - c + (j + c) * ldab;                     \
                    const T t = *a; *a = *b; *b = t;                         \
                }                                                            \
            }                                                                \
            if (km > 0) {                                                    \
                const T r = RCP(col[0]);                                     \
                for (int i = 1; i <= km; ++i) col[i] = MUL(col[i], r);       \
                for (int c = 1; c <= ju - j; ++c) {                          \
                    const T u = ab[kv - c + (j + c) * ldab];                 \
                    if (u != 0) {                                            \
                        const T t = -u;                                      \
                        T *dst = ab + kv - c + 1 + (j + c) * ldab;           \
                        for (int i = 1; i <= km; ++i)                        \
                            dst[i - 1] += MUL(col[i], t);                    \
                    }                                                        \
                }                                                            \
            }                                                                \
        } else if (info == 0) {                                              \
            info = j + 1;                                                    \
        }                                                                    \
    }                                                                        \
    return info;                                                             \
}
static inline double zabs1(zc z) { return fabs(creal(z)) + fabs(cimag(z)); }
static inline double cabs1f(cc z) { return fabsf(crealf(z)) + fabsf(cimagf(z)); }
DEFINE_GBTF2(orc_builtin_zgbtrf, zc, zrcp, zmul, zabs1)
DEFINE_GBTF2(orc_builtin_cgbtrf, cc, crcp, cmul, cabs1f)

/* zgbtrs / cgbtrs restatement.  'C' uses conjugates of the factors. */
#define DEFINE_GBTRS(NAME, T, MUL, DIV, CONJ)                                  \
int NAME(char trans, int n, int kl, int ku, int nrhs, const T *ab, int ldab, \
         const int *ipiv, T *b, int ldb)                                     \
{                                                                            \
    trans = (char) toupper((unsigned char) trans);                           \
    if (trans != 'N' && trans != 'T' && trans != 'C') return -1;             \
    if (n < 0) return -2;                                                    \
    if (kl < 0) return -3;                                                   \
    if (ku < 0) return -4;                                                   \
    if (nrhs < 0) return -5;                                                 \
    if (ldab < 2 * kl + ku + 1) return -7;                                   \
    if (ldb < imax(1, n)) return -10;                                        \
    const int kd = ku + kl;             /* row of the diagonal (0-based) */  \
    const int doconj = (trans == 'C');                                         \
    for (int r = 0; r < nrhs; ++r) {                                         \
        T *x = b + r * ldb;                                                  \
        if (trans == 'N') {                                                  \
            if (kl > 0) for (int j = 0; j < n - 1; ++j) {                    \
                const int lm = imin(kl, n - 1 - j);                          \
                const int l = ipiv[j] - 1;                                   \
                if (l != j) { const T t = x[l]; x[l] = x[j]; x[j] = t; }     \
                const T xj = x[j];                                           \
                for (int i = 1; i <= lm; ++i)                                \
                    x[j + i] -= MUL(ab[kd + i + j * ldab], xj);              \
            }                                                                \
            for (int j = n - 1; j >= 0; --j) {                               \
                if (x[j] != 0) {                                             \
                    x[j] = DIV(x[j], ab[kd + j * ldab]);                     \
                    const T t = x[j];                                        \
                    for (int i = imax(0, j - kd); i < j; ++i)                \
                        x[i] -= MUL(t, ab[kd + i - j + j * ldab]);           \
                }                                                            \
            }                                                                \
        } else {                                                             \
            for (int j = 0; j < n; ++j) {                                    \
                T t = x[j];                                                  \
                for (int i = imax(0, j - kd); i < j; ++i) {                  \
                    T a = ab[kd + i - j + j * ldab];                         \
                    if (doconj) a = CONJ(a);                                   \
                    t -= MUL(a, x[i]);                                       \
                }                                                            \
                T d = ab[kd + j * ldab];                                     \
                if (doconj) d = CONJ(d);                                       \
                x[j] = DIV(t, d);                                            \
            }                                                                \
            if (kl > 0) for (int j = n - 2; j >= 0; --j) {                   \
                const int lm = imin(kl, n - 1 - j);                          \
                T t = x[j];                                                  \
                for (int i = 1; i <= lm; ++i) {                              \
                    T a = ab[kd + i + j * ldab];                             \
                    if (doconj) a = CONJ(a);                                   \
                    t -= MUL(a, x[j + i]);                                   \
                }                                                            \
                x[j] = t;                                                    \
                const int l = ipiv[j] - 1;                                   \
                if (l != j) { const T s = x[l]; x[l] = x[j]; x[j] = s; }     \
            }                                                                \
        }                                                                    \
    }                                                                        \
    return 0;                                                                \
}
DEFINE_GBTRS(orc_builtin_zgbtrs, zc, zmul, zdiv, conj)
DEFINE_GBTRS(orc_builtin_cgbtrs, cc, cmul, cdiv, conjf)

/* ------------------------------------------------------------------------ */
/* LAPACK backend switch: builtin restatement or SciPy's OpenBLAS           */
/* ------------------------------------------------------------------------ */
typedef void (*f_gbtrf)(const int*, const int*, const int*, const int*,
                        void*, const int*, int*, int*);
typedef void (*f_gbtrs)(const char*, const int*, const int*, const int*,
                        const int*, const void*, const int*, const int*,
                        void*, const int*, int*, size_t);
static f_gbtrf ob_zgbtrf, ob_cgbtrf;
static f_gbtrs ob_zgbtrs, ob_cgbtrs;
static int use_openblas = 0;

/* Returns 0 when the library loaded and every symbol resolved. */
int orc_use_openblas(const char *path)
{
    if (!path) { use_openblas = 0; return 0; }
    void *h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
    if (!h) return 1;
    ob_zgbtrf = (f_gbtrf) dlsym(h, "scipy_zgbtrf_");
    ob_cgbtrf = (f_gbtrf) dlsym(h, "scipy_cgbtrf_");
    ob_zgbtrs = (f_gbtrs) dlsym(h, "scipy_zgbtrs_");
    ob_cgbtrs = (f_gbtrs) dlsym(h, "scipy_cgbtrs_");
    void (*set_threads)(int) = (void (*)(int)) dlsym(h, "scipy_openblas_set_num_threads");
    if (!ob_zgbtrf || !ob_cgbtrf || !ob_zgbtrs || !ob_cgbtrs) return 2;
    if (set_threads) set_threads(1);
    use_openblas = 1;
    return 0;
}

int orc_zgbtrf(int n, int kl, int ku, zc *ab, int ldab, int *ipiv)
{
    if (!use_openblas) return orc_builtin_zgbtrf(n, kl, ku, ab, ldab, ipiv);
    int info = 0;
    ob_zgbtrf(&n, &n, &kl, &ku, ab, &ldab, ipiv, &info);
    return info;
}
int orc_cgbtrf(int n, int kl, int ku, cc *ab, int ldab, int *ipiv)
{
    if (!use_openblas) return orc_builtin_cgbtrf(n, kl, ku, ab, ldab, ipiv);
    int info = 0;
    ob_cgbtrf(&n, &n, &kl, &ku, ab, &ldab, ipiv, &info);
    return info;
}
int orc_zgbtrs(char trans, int n, int kl, int ku, int nrhs, const zc *ab,
               int ldab, const int *ipiv, zc *b, int ldb)
{
    if (!use_openblas)
        return orc_builtin_zgbtrs(trans, n, kl, ku, nrhs, ab, ldab, ipiv, b, ldb);
    int info = 0;
    ob_zgbtrs(&trans, &n, &kl, &ku, &nrhs, ab, &ldab, ipiv, b, &ldb, &info, 1);
    return info;
}
int orc_cgbtrs(char trans, int n, int kl, int ku, int nrhs, const cc *ab,
               int ldab, const int *ipiv, cc *b, int ldb)
{
    if (!use_openblas)
        return orc_builtin_cgbtrs(trans, n, kl, ku, nrhs, ab, ldab, ipiv, b, ldb);
    int info = 0;
    ob_cgbtrs(&trans, &n, &kl, &ku, &nrhs, ab, &ldab, ipiv, b, &ldb, &info, 1);
    return info;
}

/* suzerain_lapackext_zgbsv: factor when *fact == 'N', then solve */
int orc_zgbsv(char *fact, char trans, int n, int kl, int ku, int nrhs,
              zc *ab, int ldab, int *ipiv, zc *b, int ldb)
{
    int info = 0;
    if (toupper((unsigned char) *fact) == 'N') {
        info = orc_zgbtrf(n, kl, ku, ab, ldab, ipiv);
        *fact = 'F';
    }
    if (!info) info = orc_zgbtrs(trans, n, kl, ku, nrhs, ab, ldab, ipiv, b, ldb);
    return info;
}

/* ------------------------------------------------------------------------ */
/* gbmv restatement (netlib semantics, zero-indexed); 'C' takes the 'T'      */
/* branch without conjugation exactly like suzerain/blas_et_al/gbmv.def.    */
/* ------------------------------------------------------------------------ */
int orc_zgbmv(char trans, int m, int n, int kl, int ku, zc alpha,
              const zc *a, int lda, const zc *x, int incx, zc beta,
              zc *y, int incy)
{
    trans = (char) toupper((unsigned char) trans);
    if (trans != 'N' && trans != 'T' && trans != 'C') return 1;
    if (m < 0) return 2;
    if (n < 0) return 3;
    if (kl < 0) return 4;
    if (ku < 0) return 5;
    if (lda <= kl + ku) return 8;
    if (incx == 0) return 10;
    if (incy == 0) return 13;
    if (m == 0 || n == 0) return 0;
    const int lenx = trans == 'N' ? n : m, leny = trans == 'N' ? m : n;
    const int kx = incx > 0 ? 0 : (1 - lenx) * incx;
    const int ky = incy > 0 ? 0 : (1 - leny) * incy;
    if (!(creal(beta) == 1 && cimag(beta) == 0)) {
        for (int i = 0; i < leny; ++i) {
            zc *yp = y + ky + i * incy;
            *yp = (creal(beta) == 0 && cimag(beta) == 0) ? 0 : beta * (*yp);
        }
    }
    if (creal(alpha) == 0 && cimag(alpha) == 0) return 0;
    if (trans == 'N') {
        for (int j = 0; j < n; ++j) {
            const zc t = alpha * x[kx + j * incx];
            for (int i = imax(0, j - ku); i < imin(m, j + kl + 1); ++i)
                y[ky + i * incy] += t * a[ku + i - j + j * lda];
        }
    } else {
        for (int j = 0; j < n; ++j) {
            zc t = 0;
            for (int i = imax(0, j - ku); i < imin(m, j + kl + 1); ++i)
                t += a[ku + i - j + j * lda] * x[kx + i * incx];
            y[ky + j * incy] += alpha * t;
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Norms                                                                    */
/* ------------------------------------------------------------------------ */
double orc_dznrm2(int n, const zc *x)
{
    double scale = 0, ssq = 1;
    for (int i = 0; i < n; ++i) {
        const double parts[2] = { creal(x[i]), cimag(x[i]) };
        for (int k = 0; k < 2; ++k) {
            if (parts[k] != 0) {
                const double a = fabs(parts[k]);
                if (scale < a) { ssq = 1 + ssq * (scale / a) * (scale / a); scale = a; }
                else           { ssq += (a / scale) * (a / scale); }
            }
        }
    }
    return scale * sqrt(ssq);
}

double orc_zlangb_fro(int n, int kl, int ku, const zc *ab, int ldab)
{
    double scale = 0, ssq = 1;
    for (int j = 0; j < n; ++j)
        for (int i = imax(0, j - ku); i <= imin(n - 1, j + kl); ++i) {
            const zc v = ab[ku + i - j + j * ldab];
            const double parts[2] = { creal(v), cimag(v) };
            for (int k = 0; k < 2; ++k) {
                if (parts[k] != 0) {
                    const double a = fabs(parts[k]);
                    if (scale < a) { ssq = 1 + ssq * (scale / a) * (scale / a); scale = a; }
                    else           { ssq += (a / scale) * (a / scale); }
                }
            }
        }
    return scale * sqrt(ssq);
}

double orc_dlamch_eps(void) { return DBL_EPSILON * 0.5; }

/* ------------------------------------------------------------------------ */
/* zgbsvx restatement: the expert driver of reference LAPACK with its        */
/* helpers, from the published algorithms (0-based indices; ab is the band   */
/* with A(i,j) at ab[ku+i-j + j*ldab]; afb the gbtrf storage).               */
/*   ZGBEQU  row scales r_i = 1/max_j |a_ij|_1, then column scales c_j =     */
/*           1/max_i |a_ij|_1 r_i (|.|_1 = |re|+|im|), clamped to            */
/*           [safmin, 1/safmin]; info i+1 / n+j+1 at the first zero row/col  */
/*   ZLAQGB  scale rows when rowcnd < 0.1 or amax outside [small, large],    */
/*           columns when colcnd < 0.1 (small = safmin/precision)            */
/*   ZLANGB  '1', 'I', 'M' with the modulus                                  */
/*   ZGBCON  Higham's estimator (ZLACN2: at most 5 iterations, x = 1/n, the  */
/*           sign vector x_i/|x_i|, unit vectors at the first max modulus,   */
/*           the alternating vector (-1)^i (1 + i/(n-1)) with 2 s/(3n))      */
/*           over the solves with the factor; ZLATBS's overflow rescaling    */
/*           is not taken (scale stays 1)                                    */
/*   ZGBRFS  residual, componentwise backward error with nz = min(kl+ku+2,   */
/*           n+1), safe1 = nz safmin, safe2 = safe1/eps; at most 5           */
/*           corrections while berr > eps and berr halves; ferr from the     */
/*           estimator on diag(w) inv(op(A)^H) and inv(op(A)) diag(w)        */
/* ------------------------------------------------------------------------ */
static const double kSafmin = DBL_MIN;               /* dlamch('S') */
static const double kPrec = DBL_EPSILON;             /* dlamch('P') */

static int orc_zgbequ(int n, int kl, int ku, const zc *ab, int ldab, double *r,
                      double *c, double *rowcnd, double *colcnd, double *amax)
{
    const double smlnum = kSafmin, bignum = 1.0 / smlnum;
    *rowcnd = 1; *colcnd = 1; *amax = 0;
    for (int i = 0; i < n; ++i) r[i] = 0;
    for (int j = 0; j < n; ++j)
        for (int i = imax(0, j - ku); i <= imin(n - 1, j + kl); ++i)
            r[i] = fmax(r[i], zabs1(ab[ku + i - j + j * ldab]));
    double mn = bignum, mx = 0;
    for (int i = 0; i < n; ++i) { mx = fmax(mx, r[i]); mn = fmin(mn, r[i]); }
    *amax = mx;
    if (mn == 0) {
        for (int i = 0; i < n; ++i) if (r[i] == 0) return i + 1;
    }
    for (int i = 0; i < n; ++i) r[i] = 1.0 / fmin(fmax(r[i], smlnum), bignum);
    *rowcnd = fmax(mn, smlnum) / fmin(mx, bignum);
    for (int j = 0; j < n; ++j) c[j] = 0;
    for (int j = 0; j < n; ++j)
        for (int i = imax(0, j - ku); i <= imin(n - 1, j + kl); ++i)
            c[j] = fmax(c[j], zabs1(ab[ku + i - j + j * ldab]) * r[i]);
    mn = bignum; mx = 0;
    for (int j = 0; j < n; ++j) { mn = fmin(mn, c[j]); mx = fmax(mx, c[j]); }
    if (mn == 0) {
        for (int j = 0; j < n; ++j) if (c[j] == 0) return n + j + 1;
    }
    for (int j = 0; j < n; ++j) c[j] = 1.0 / fmin(fmax(c[j], smlnum), bignum);
    *colcnd = fmax(mn, smlnum) / fmin(mx, bignum);
    return 0;
}

static char orc_zlaqgb(int n, int kl, int ku, zc *ab, int ldab, const double *r,
                       const double *c, double rowcnd, double colcnd, double amax)
{
    const double small = kSafmin / kPrec, large = 1.0 / small;
    char equed;
    if (rowcnd >= 0.1 && amax >= small && amax <= large)
        equed = colcnd >= 0.1 ? 'N' : 'C';
    else
        equed = colcnd >= 0.1 ? 'R' : 'B';
    if (equed == 'N') return equed;
    for (int j = 0; j < n; ++j)
        for (int i = imax(0, j - ku); i <= imin(n - 1, j + kl); ++i) {
            double f = equed == 'C' ? c[j] : (equed == 'R' ? r[i] : c[j] * r[i]);
            ab[ku + i - j + j * ldab] *= f;
        }
    return equed;
}

static double orc_zlangb(char norm, int n, int kl, int ku, const zc *ab, int ldab)
{
    double v = 0;
    if (norm == 'M') {
        for (int j = 0; j < n; ++j)
            for (int i = imax(0, j - ku); i <= imin(n - 1, j + kl); ++i)
                v = fmax(v, cabs(ab[ku + i - j + j * ldab]));
    } else if (norm == '1') {
        for (int j = 0; j < n; ++j) {
            double s = 0;
            for (int i = imax(0, j - ku); i <= imin(n - 1, j + kl); ++i)
                s += cabs(ab[ku + i - j + j * ldab]);
            v = fmax(v, s);
        }
    } else {
        for (int i = 0; i < n; ++i) {
            double s = 0;
            for (int j = imax(0, i - kl); j <= imin(n - 1, i + ku); ++j)
                s += cabs(ab[ku + i - j + j * ldab]);
            v = fmax(v, s);
        }
    }
    return v;
}

static double dzsum1(int n, const zc *x)
{
    double s = 0;
    for (int i = 0; i < n; ++i) s += cabs(x[i]);
    return s;
}
static int izmax1(int n, const zc *x)
{
    int k = 0;
    double best = cabs(x[0]);
    for (int i = 1; i < n; ++i) if (cabs(x[i]) > best) { best = cabs(x[i]); k = i; }
    return k;
}
static void sign_vec(int n, zc *x)
{
    for (int i = 0; i < n; ++i) {
        const double a = cabs(x[i]);
        x[i] = a > kSafmin ? creal(x[i]) / a + I * (cimag(x[i]) / a) : 1.0;
    }
}

/* ZLACN2 reverse communication; isave[0] = state, [1] = index, [2] = iter */
static void orc_zlacn2(int n, zc *v, zc *x, double *est, int *kase, int isave[3])
{
    if (*kase == 0) {
        for (int i = 0; i < n; ++i) x[i] = 1.0 / (double) n;
        *kase = 1; isave[0] = 1;
        return;
    }
    switch (isave[0]) {
    case 1:
        if (n == 1) { v[0] = x[0]; *est = cabs(v[0]); *kase = 0; return; }
        *est = dzsum1(n, x);
        sign_vec(n, x);
        *kase = 2; isave[0] = 2;
        return;
    case 2:
        isave[1] = izmax1(n, x);
        isave[2] = 2;
        goto unit;
    case 3: {
        memcpy(v, x, (size_t) n * sizeof(zc));
        const double estold = *est;
        *est = dzsum1(n, v);
        if (*est <= estold) goto alt;
        sign_vec(n, x);
        *kase = 2; isave[0] = 4;
        return;
    }
    case 4: {
        const int jlast = isave[1];
        isave[1] = izmax1(n, x);
        if (cabs(x[jlast]) != cabs(x[isave[1]]) && isave[2] < 5) {
            isave[2] += 1;
            goto unit;
        }
        goto alt;
    }
    case 5: {
        const double temp = 2.0 * (dzsum1(n, x) / (double) (3 * n));
        if (temp > *est) { memcpy(v, x, (size_t) n * sizeof(zc)); *est = temp; }
        *kase = 0;
        return;
    }
    }
unit:
    for (int i = 0; i < n; ++i) x[i] = 0;
    x[isave[1]] = 1;
    *kase = 1; isave[0] = 3;
    return;
alt:
    for (int i = 0; i < n; ++i)
        x[i] = ((i & 1) ? -1.0 : 1.0) * (1.0 + (double) i / (double) (n - 1));
    *kase = 1; isave[0] = 5;
}

static double orc_zgbcon(char norm, int n, int kl, int ku, const zc *afb, int ldafb,
                         const int *ipiv, double anorm, zc *work)
{
    if (n == 0) return 1;
    if (anorm == 0) return 0;
    const int kase1 = norm == '1' ? 1 : 2;
    zc *x = work, *v = work + n;
    double ainvnm = 0;
    int kase = 0, isave[3] = {0, 0, 0};
    for (;;) {
        orc_zlacn2(n, v, x, &ainvnm, &kase, isave);
        if (!kase) break;
        orc_zgbtrs(kase == kase1 ? 'N' : 'C', n, kl, ku, 1, afb, ldafb, ipiv, x, n);
    }
    return ainvnm != 0 ? (1.0 / ainvnm) / anorm : 0;
}

static void orc_zgbrfs(char trans, int n, int kl, int ku, const zc *ab, int ldab,
                       const zc *afb, int ldafb, const int *ipiv, const zc *b, zc *x,
                       double *ferr, double *berr, zc *work, double *rw)
{
    const int notran = trans == 'N';
    const char transn = notran ? 'N' : 'C', transt = notran ? 'C' : 'N';
    const double nz = imin(kl + ku + 2, n + 1);
    const double eps = DBL_EPSILON * 0.5, safe1 = nz * kSafmin, safe2 = safe1 / eps;
    zc *r = work, *ex = work + n, *ev = work + 2 * n;
    int count = 1;
    double lstres = 3;
    for (;;) {
        for (int i = 0; i < n; ++i) { r[i] = b[i]; rw[i] = zabs1(b[i]); }
        if (notran) {
            for (int k = 0; k < n; ++k) {
                const double xk = zabs1(x[k]);
                for (int i = imax(0, k - ku); i <= imin(n - 1, k + kl); ++i) {
                    const zc a = ab[ku + i - k + k * ldab];
                    r[i] -= a * x[k];
                    rw[i] += zabs1(a) * xk;
                }
            }
        } else {
            for (int k = 0; k < n; ++k) {
                double s = 0;
                for (int i = imax(0, k - ku); i <= imin(n - 1, k + kl); ++i) {
                    zc a = ab[ku + i - k + k * ldab];
                    if (trans == 'C') a = conj(a);
                    r[k] -= a * x[i];
                    s += zabs1(a) * zabs1(x[i]);
                }
                rw[k] += s;
            }
        }
        double s = 0;
        for (int i = 0; i < n; ++i)
            s = fmax(s, rw[i] > safe2 ? zabs1(r[i]) / rw[i] : (zabs1(r[i]) + safe1) / (rw[i] + safe1));
        *berr = s;
        if (s > eps && 2 * s <= lstres && count <= 5) {
            orc_zgbtrs(trans, n, kl, ku, 1, afb, ldafb, ipiv, r, n);
            for (int i = 0; i < n; ++i) x[i] += r[i];
            lstres = s;
            count += 1;
            continue;
        }
        break;
    }
    for (int i = 0; i < n; ++i)
        rw[i] = rw[i] > safe2 ? zabs1(r[i]) + nz * eps * rw[i] : zabs1(r[i]) + nz * eps * rw[i] + safe1;
    int kase = 0, isave[3] = {0, 0, 0};
    *ferr = 0;
    for (;;) {
        orc_zlacn2(n, ev, ex, ferr, &kase, isave);
        if (!kase) break;
        if (kase == 1) {
            orc_zgbtrs(transt, n, kl, ku, 1, afb, ldafb, ipiv, ex, n);
            for (int i = 0; i < n; ++i) ex[i] *= rw[i];
        } else {
            for (int i = 0; i < n; ++i) ex[i] *= rw[i];
            orc_zgbtrs(transn, n, kl, ku, 1, afb, ldafb, ipiv, ex, n);
        }
    }
    double xm = 0;
    for (int i = 0; i < n; ++i) xm = fmax(xm, zabs1(x[i]));
    if (xm != 0) *ferr /= xm;
}

/* suzerain_lapack_zgbsvx semantics (fact 'N', 'E', 'F'; nrhs columns);
 * returns info; *rpvgrw receives what LAPACK leaves in rwork[0]. */
int orc_zgbsvx(char fact, char trans, int n, int kl, int ku, int nrhs, zc *ab, int ldab,
               zc *afb, int ldafb, int *ipiv, char *equed, double *r, double *c, zc *b,
               int ldb, zc *x, int ldx, double *rcond, double *ferr, double *berr,
               double *rpvgrw)
{
    fact = (char) toupper((unsigned char) fact);
    trans = (char) toupper((unsigned char) trans);
    const int nofact = fact == 'N', equil = fact == 'E', notran = trans == 'N';
    int rowequ = 0, colequ = 0;
    double rowcnd = 1, colcnd = 1, amax = 0;
    const double smlnum = kSafmin, bignum = 1.0 / smlnum;
    if (nofact || equil) *equed = 'N';
    else {
        *equed = (char) toupper((unsigned char) *equed);
        rowequ = *equed == 'R' || *equed == 'B';
        colequ = *equed == 'C' || *equed == 'B';
    }
    if (!nofact && !equil && fact != 'F') return -1;
    if (!notran && trans != 'T' && trans != 'C') return -2;
    if (n < 0) return -3;
    if (kl < 0) return -4;
    if (ku < 0) return -5;
    if (nrhs < 0) return -6;
    if (ldab < kl + ku + 1) return -8;
    if (ldafb < 2 * kl + ku + 1) return -10;
    if (fact == 'F' && !(rowequ || colequ || *equed == 'N')) return -12;
    if (rowequ) {
        double mn = bignum, mx = 0;
        for (int j = 0; j < n; ++j) { mn = fmin(mn, r[j]); mx = fmax(mx, r[j]); }
        if (mn <= 0) return -13;
        rowcnd = n > 0 ? fmax(mn, smlnum) / fmin(mx, bignum) : 1;
    }
    if (colequ) {
        double mn = bignum, mx = 0;
        for (int j = 0; j < n; ++j) { mn = fmin(mn, c[j]); mx = fmax(mx, c[j]); }
        if (mn <= 0) return -14;
        colcnd = n > 0 ? fmax(mn, smlnum) / fmin(mx, bignum) : 1;
    }
    if (ldb < imax(1, n)) return -16;
    if (ldx < imax(1, n)) return -18;
    if (equil) {
        if (orc_zgbequ(n, kl, ku, ab, ldab, r, c, &rowcnd, &colcnd, &amax) == 0) {
            *equed = orc_zlaqgb(n, kl, ku, ab, ldab, r, c, rowcnd, colcnd, amax);
            rowequ = *equed == 'R' || *equed == 'B';
            colequ = *equed == 'C' || *equed == 'B';
        }
    }
    for (int j = 0; j < nrhs; ++j)
        for (int i = 0; i < n; ++i) {
            if (notran && rowequ) b[i + j * ldb] *= r[i];
            else if (!notran && colequ) b[i + j * ldb] *= c[i];
        }
    const int kv = kl + ku;
    int info = 0;
    if (nofact || equil) {
        for (int j = 0; j < n; ++j) {
            for (int t = 0; t < ldafb; ++t) afb[t + j * ldafb] = 0;
            for (int i = imax(0, j - ku); i <= imin(n - 1, j + kl); ++i)
                afb[kl + ku + i - j + j * ldafb] = ab[ku + i - j + j * ldab];
        }
        info = orc_zgbtrf(n, kl, ku, afb, ldafb, ipiv);
        if (info > 0) {
            double an = 0, um = 0;
            for (int j = 0; j < info; ++j)
                for (int i = imax(0, j - ku); i <= imin(n - 1, j + kl); ++i)
                    an = fmax(an, cabs(ab[ku + i - j + j * ldab]));
            for (int j = 0; j < info; ++j)
                for (int i = imax(0, j - kv); i <= j; ++i)
                    um = fmax(um, cabs(afb[kv + i - j + j * ldafb]));
            *rpvgrw = um == 0 ? 1 : an / um;
            *rcond = 0;
            return info;
        }
    }
    const char norm = notran ? '1' : 'I';
    const double anorm = orc_zlangb(norm, n, kl, ku, ab, ldab);
    double um = 0;
    for (int j = 0; j < n; ++j)
        for (int i = imax(0, j - kv); i <= j; ++i)
            um = fmax(um, cabs(afb[kv + i - j + j * ldafb]));
    *rpvgrw = um == 0 ? 1 : orc_zlangb('M', n, kl, ku, ab, ldab) / um;
    zc *work = (zc *) malloc((size_t) 3 * imax(n, 1) * sizeof(zc));
    double *rw = (double *) malloc((size_t) imax(n, 1) * sizeof(double));
    *rcond = orc_zgbcon(norm, n, kl, ku, afb, ldafb, ipiv, anorm, work);
    for (int j = 0; j < nrhs; ++j) {
        for (int i = 0; i < n; ++i) x[i + j * ldx] = b[i + j * ldb];
        orc_zgbtrs(trans, n, kl, ku, 1, afb, ldafb, ipiv, x + j * ldx, ldx);
        orc_zgbrfs(trans, n, kl, ku, ab, ldab, afb, ldafb, ipiv, b + j * ldb, x + j * ldx,
                   ferr + j, berr + j, work, rw);
    }
    free(work);
    free(rw);
    for (int j = 0; j < nrhs; ++j) {
        if (notran && colequ) {
            for (int i = 0; i < n; ++i) x[i + j * ldx] *= c[i];
            ferr[j] /= colcnd;
        } else if (!notran && rowequ) {
            for (int i = 0; i < n; ++i) x[i + j * ldx] *= r[i];
            ferr[j] /= rowcnd;
        }
    }
    if (*rcond < DBL_EPSILON * 0.5) info = n + 1;
    return info;
}

/* LAPACK's own zgbsvx from SciPy's OpenBLAS, for pinning the restatement;
 * returns -1000 when the library or the symbol is missing. */
typedef void (*f_gbsvx)(const char*, const char*, const int*, const int*, const int*,
                        const int*, void*, const int*, void*, const int*, int*, char*,
                        double*, double*, void*, const int*, void*, const int*, double*,
                        double*, double*, void*, double*, int*, size_t, size_t, size_t);
int orc_openblas_zgbsvx(const char *path, char fact, char trans, int n, int kl, int ku,
                        int nrhs, zc *ab, int ldab, zc *afb, int ldafb, int *ipiv,
                        char *equed, double *r, double *c, zc *b, int ldb, zc *x, int ldx,
                        double *rcond, double *ferr, double *berr, double *rpvgrw)
{
    void *h = path ? dlopen(path, RTLD_NOW | RTLD_LOCAL) : NULL;
    if (!h) return -1000;
    f_gbsvx f = (f_gbsvx) dlsym(h, "scipy_zgbsvx_");
    void (*set_threads)(int) = (void (*)(int)) dlsym(h, "scipy_openblas_set_num_threads");
    if (!f) return -1000;
    if (set_threads) set_threads(1);
    zc *work = (zc *) malloc((size_t) 2 * imax(n, 1) * sizeof(zc));
    double *rwork = (double *) malloc((size_t) imax(n, 1) * sizeof(double));
    int info = 0;
    f(&fact, &trans, &n, &kl, &ku, &nrhs, ab, &ldab, afb, &ldafb, ipiv, equed, r, c, b, &ldb,
      x, &ldx, rcond, ferr, berr, work, rwork, &info, 1, 1, 1);
    *rpvgrw = rwork[0];
    free(work);
    free(rwork);
    return info;
}

/* ------------------------------------------------------------------------ */
/* zcgbsvx restatement (suzerain/blas_et_al/dsgbsvx.def:70-313)             */
/* ------------------------------------------------------------------------ */
static int zcgbsvx_impl(char *fact, int *apprx, int aiter, char trans, int n,
                        int kl, int ku, zc *ab, double *afrob, zc *afb,
                        int *ipiv, const zc *b, zc *x, int *siter,
                        int *diter, double *tolsc, zc *r, double *res)
{
    *fact = (char) toupper((unsigned char) *fact);
    trans = (char) toupper((unsigned char) trans);
    int info = 0;
    if (*fact != 'N' && *fact != 'S' && *fact != 'D') info = -1;
    else if (*apprx < 0) info = -2;
    else if (aiter < 0) info = -3;
    else if (trans != 'N' && trans != 'T' && trans != 'C') info = -4;
    else if (n < 0) info = -5;
    else if (kl < 0) info = -6;
    else if (ku < 0) info = -7;
    else if (*tolsc < 0) info = -16;
    else if (*siter < 0 && *diter < 0) info = -99;
    if (info) return info;

    const double eps = orc_dlamch_eps();
    const int ldab = kl + 1 + ku, ldafb = 2 * kl + 1 + ku;

    memset(x, 0, (size_t) n * sizeof(zc));
    memcpy(r, b, (size_t) n * sizeof(zc));
    *res = orc_dznrm2(n, r);
    const double resdecay = 2;
    double lastres = (resdecay + 1) * (*res + 1);

    const int use_eps_tol = (*tolsc == 0.0);
    double tolconst, tol;
    if (use_eps_tol) { tolconst = 1; tol = eps; }
    else {
        if (*afrob < 0) *afrob = orc_zlangb_fro(n, kl, ku, ab, ldab);
        tolconst = *afrob * eps * sqrt((double) n) * (*tolsc);
        tol = 0;
    }

    const int smax = *siter; *siter = -1;
    const int dmax = *diter; *diter = -1;

    if (smax >= 0 && *fact != 'D' && *res > tol) {
        cc *afs = (cc *) afb;   /* single-precision factor, packed densely */
        if (*fact != 'S') {
            *fact = 'S';
            *apprx = 0;
            for (int j = 0; j < n; ++j)
                for (int i = 0; i < ldafb; ++i)
                    afs[i + j * ldafb] = (i < kl) ? 0 : (cc) ab[(i - kl) + j * ldab];
            info = orc_cgbtrf(n, kl, ku, afs, ldafb, ipiv);
            if (info > 0 && dmax >= 0) goto double_precision_attempt;
            else if (info < 0) return info;
        }
        cc *rs = (cc *) malloc((size_t) n * sizeof(cc));
        while (*siter < smax && *res > tol) {
            *siter += 1;
            for (int i = 0; i < n; ++i) rs[i] = (cc) r[i];
            orc_cgbtrs(trans, n, kl, ku, 1, afs, ldafb, ipiv, rs, n);
            for (int i = 0; i < n; ++i) x[i] += (zc) rs[i];
            double xn = use_eps_tol ? eps : orc_dznrm2(n, x);
            tol = xn * tolconst;
            memcpy(r, b, (size_t) n * sizeof(zc));
            orc_zgbmv(trans, n, n, kl, ku, -1, ab, ldab, x, 1, 1, r, 1);
            *res = orc_dznrm2(n, r);
            if (isnan(*res)) { free(rs); return -1000; }
            if (*siter >= aiter && lastres < *res * resdecay) {
                if (*apprx) {
                    free(rs);
                    *fact = 'N'; *siter = smax; *diter = dmax;
                    return zcgbsvx_impl(fact, apprx, aiter, trans, n, kl, ku,
                                        ab, afrob, afb, ipiv, b, x, siter,
                                        diter, tolsc, r, res);
                }
                break;
            }
            lastres = *res;
        }
        free(rs);
    } else {
        *siter = 0;
    }

double_precision_attempt:
    if (dmax >= 0 && *res > tol) {
        if (*fact != 'D') {
            *fact = 'D';
            *apprx = 0;
            for (int j = 0; j < n; ++j)
                for (int i = 0; i < ldafb; ++i)
                    afb[i + j * ldafb] = (i < kl) ? 0 : ab[(i - kl) + j * ldab];
            info = orc_zgbtrf(n, kl, ku, afb, ldafb, ipiv);
            if (info < 0) return info;
            if (info > 0) return info;
        }
        while (*diter < dmax && *res > tol) {
            *diter += 1;
            orc_zgbtrs(trans, n, kl, ku, 1, afb, ldafb, ipiv, r, n);
            for (int i = 0; i < n; ++i) x[i] += r[i];
            double xn = use_eps_tol ? eps : orc_dznrm2(n, x);
            tol = xn * tolconst;
            memcpy(r, b, (size_t) n * sizeof(zc));
            orc_zgbmv(trans, n, n, kl, ku, -1, ab, ldab, x, 1, 1, r, 1);
            *res = orc_dznrm2(n, r);
            if (isnan(*res)) return -1001;
            if (*diter >= aiter && lastres < *res * resdecay) {
                if (*apprx) {
                    *fact = 'N'; *siter = smax; *diter = dmax;
                    return zcgbsvx_impl(fact, apprx, aiter, trans, n, kl, ku,
                                        ab, afrob, afb, ipiv, b, x, siter,
                                        diter, tolsc, r, res);
                }
                break;
            }
            lastres = *res;
        }
    } else {
        *diter = 0;
    }

    *tolsc = (*res == 0) ? 0 : *res / tol;
    if (isnan(*res)) for (int i = 0; i < n; ++i) x[i] = NAN;
    return info;
}

int orc_zcgbsvx(char *fact, int *apprx, int aiter, char trans, int n, int kl,
                int ku, zc *ab, double *afrob, zc *afb, int *ipiv,
                const zc *b, zc *x, int *siter, int *diter, double *tolsc,
                zc *r, double *res)
{
    return zcgbsvx_impl(fact, apprx, aiter, trans, n, kl, ku, ab, afrob, afb,
                        ipiv, b, x, siter, diter, tolsc, r, res);
}

/* ------------------------------------------------------------------------ */
/* Synthetic block assembly into packed P A P^T                             */
/* ------------------------------------------------------------------------ */
/*
 * Block (e,f) = cM(e,f) M + cD1(e,f) D1 + cD2(e,f) D2, with real collocation
 * bands M, D1, D2 (n x n, bandwidths kl/ku, leading dimension ld, LAPACK
 * band layout) and complex coefficients.  Each entry is evaluated as
 *   re = fma(cD2.re, D2, fma(cD1.re, D1, cM.re * M)), im likewise,
 * which the device assembly reproduces bit for bit.  Rows (e, p) with
 * dirichlet[e] != 0 and p in {0, n-1} become identity rows.
 * The result is written with leading dimension ldpapt starting at row
 * offset `off` (0 for packc layout, KL for packf layout).
 */
void orc_assemble_packed(int S, int n, int kl, int ku, const double *M,
                         const double *D1, const double *D2, int ld,
                         const zc *cM, const zc *cD1, const zc *cD2,
                         const int *dirichlet, zc *papt, int ldpapt, int off)
{
    const int KL = S * (kl + 1) - 1, KU = S * (ku + 1) - 1, N = S * n;
    zc *blk = (zc *) malloc((size_t) ld * n * sizeof(zc));
    for (int e = 0; e < S; ++e)
        for (int f = 0; f < S; ++f) {
            const zc a = cM[e * S + f], b = cD1[e * S + f], c = cD2[e * S + f];
            for (int k = 0; k < ld * n; ++k) {
                const double re = fma(creal(c), D2[k], fma(creal(b), D1[k], creal(a) * M[k]));
                const double im = fma(cimag(c), D2[k], fma(cimag(b), D1[k], cimag(a) * M[k]));
                blk[k] = CMPLX(re, im);
            }
            orc_zpack(S, n, e, f, kl, ku, 1.0, blk, ld, KL, KU, papt + off, ldpapt);
        }
    free(blk);
    for (int e = 0; e < S; ++e) {
        if (!dirichlet[e]) continue;
        const int pts[2] = { 0, n - 1 };
        for (int t = 0; t < 2; ++t) {
            const int Ri = pts[t] * S + e;
            for (int Cj = imax(0, Ri - KU); Cj <= imin(N - 1, Ri + KL); ++Cj)
                papt[off + KU + Ri - Cj + Cj * ldpapt] = (Ri == Cj) ? 1.0 : 0.0;
        }
    }
}

/* Block coefficients of the synthetic operator for one wavenumber pair:
 *   cM = delta_ef - phi c_ef (kx^2 + kz^2) + i phi g_ef kx,
 *   cD1 = phi a_ef, cD2 = phi b_ef,
 * evaluated with the same roundings the device uses. */
void orc_block_coefs(int S, const double *a, const double *b, const double *c,
                     const double *g, double phi, double kx, double kz,
                     zc *cM, zc *cD1, zc *cD2)
{
    const double ksq = fma(kx, kx, kz * kz);
    for (int e = 0; e < S; ++e)
        for (int f = 0; f < S; ++f) {
            const int ef = e * S + f;
            const double pc = phi * c[ef];
            cM[ef] = CMPLX(fma(-pc, ksq, e == f ? 1.0 : 0.0), (phi * g[ef]) * kx);
            cD1[ef] = CMPLX(phi * a[ef], 0.0);
            cD2[ef] = CMPLX(phi * b[ef], 0.0);
        }
}

/* ------------------------------------------------------------------------ */
/* Batched CPU drivers (CPU baseline and bulk parity), one system/thread     */
/* ------------------------------------------------------------------------ */
typedef struct {
    int nsys, S, n, kl, ku, trans;
    const double *M, *D1, *D2; int ld;
    const double *a, *b, *c, *g;  /* S*S case coefficients */
    const int *dirichlet;         /* S flags */
    const double *kx, *kz;        /* per system */
    double phi_exp, phi_imp;
    const zc *u;                  /* nsys x N, natural order */
    zc *x;                        /* nsys x N, natural order */
    int *info;
    int mixed;                    /* 0: zgbsv path, 1: zcgbsvx path */
    int aiter, siter, diter; double tolsc;
    int *siter_out, *diter_out; double *res_out, *tolsc_out; char *fact_out;
    double *latency_s;            /* per system wall seconds, may be NULL */
    int next;                     /* work counter */
    pthread_mutex_t lock;
} orc_batch;

static double now_s(void)
{
    struct timespec t; clock_gettime(CLOCK_MONOTONIC, &t);
    return t.tv_sec + 1e-9 * t.tv_nsec;
}

static void *batch_worker(void *arg)
{
    orc_batch *B = (orc_batch *) arg;
    const int S = B->S, n = B->n, N = S * n;
    const int KL = S * (B->kl + 1) - 1, KU = S * (B->ku + 1) - 1;
    const int LD = KL + KU + 1, LDF = LD + KL;
    zc *papt = malloc((size_t) LD * N * sizeof(zc));
    zc *lu = malloc((size_t) LDF * N * sizeof(zc));
    zc *pu = malloc((size_t) N * sizeof(zc));
    zc *pb = malloc((size_t) N * sizeof(zc));
    zc *px = malloc((size_t) N * sizeof(zc));
    zc *r = malloc((size_t) N * sizeof(zc));
    zc *cM = malloc((size_t) 3 * S * S * sizeof(zc));
    zc *cD1 = cM + S * S, *cD2 = cM + 2 * S * S;
    int *ipiv = malloc((size_t) N * sizeof(int));
    for (;;) {
        pthread_mutex_lock(&B->lock);
        const int s = B->next++;
        pthread_mutex_unlock(&B->lock);
        if (s >= B->nsys) break;
        const double t0 = now_s();
        const char trans = (char) B->trans;
        const zc *us = B->u + (size_t) s * N;
        if (B->phi_exp != 0.0) {
            /* explicit operator: pb = (P E P^T) P u, wall rows zeroed */
            orc_block_coefs(S, B->a, B->b, B->c, B->g, B->phi_exp, B->kx[s], B->kz[s], cM, cD1, cD2);
            orc_assemble_packed(S, n, B->kl, B->ku, B->M, B->D1, B->D2, B->ld,
                                cM, cD1, cD2, B->dirichlet, papt, LD, 0);
            orc_zaPxpby('N', S, n, 1, us, 1, 0, pu, 1);
            orc_zgbmv('N', N, N, KL, KU, 1, papt, LD, pu, 1, 0, pb, 1);
            for (int e = 0; e < S; ++e)
                if (B->dirichlet[e]) { pb[e] = 0; pb[(n - 1) * S + e] = 0; }
        } else {
            orc_zaPxpby('N', S, n, 1, us, 1, 0, pb, 1);
        }
        orc_block_coefs(S, B->a, B->b, B->c, B->g, B->phi_imp, B->kx[s], B->kz[s], cM, cD1, cD2);
        if (!B->mixed) {
            orc_assemble_packed(S, n, B->kl, B->ku, B->M, B->D1, B->D2, B->ld,
                                cM, cD1, cD2, B->dirichlet, lu, LDF, KL);
            char fact = 'N';
            B->info[s] = orc_zgbsv(&fact, trans, N, KL, KU, 1, lu, LDF, ipiv, pb, N);
            orc_zaPxpby('T', S, n, 1, pb, 1, 0, B->x + (size_t) s * N, 1);
        } else {
            orc_assemble_packed(S, n, B->kl, B->ku, B->M, B->D1, B->D2, B->ld,
                                cM, cD1, cD2, B->dirichlet, papt, LD, 0);
            char fact = 'N'; int apprx = 0, si = B->siter, di = B->diter;
            double afrob = -1, tolsc = B->tolsc, res = 0;
            B->info[s] = orc_zcgbsvx(&fact, &apprx, B->aiter, trans, N, KL, KU,
                                     papt, &afrob, lu, ipiv, pb, px, &si, &di,
                                     &tolsc, r, &res);
            orc_zaPxpby('T', S, n, 1, px, 1, 0, B->x + (size_t) s * N, 1);
            if (B->siter_out) B->siter_out[s] = si;
            if (B->diter_out) B->diter_out[s] = di;
            if (B->res_out) B->res_out[s] = res;
            if (B->tolsc_out) B->tolsc_out[s] = tolsc;
            if (B->fact_out) B->fact_out[s] = fact;
        }
        if (B->latency_s) B->latency_s[s] = now_s() - t0;
    }
    free(papt); free(lu); free(pu); free(pb); free(px); free(r); free(cM); free(ipiv);
    return NULL;
}

/*
 * One synthetic substep for nsys systems on nthreads host threads:
 * optional explicit operator (phi_exp != 0), assemble packed P A P^T with
 * phi_imp, solve with zgbsv (mixed == 0) or zcgbsvx (mixed == 1), permute the
 * solution to natural order.  Returns wall seconds.
 */
double orc_batch_solve(int nsys, int S, int n, int kl, int ku, char trans,
                       const double *M, const double *D1, const double *D2,
                       int ld, const double *a, const double *b,
                       const double *c, const double *g, const int *dirichlet,
                       const double *kx, const double *kz, double phi_exp,
                       double phi_imp, const zc *u, zc *x, int *info,
                       int mixed, int aiter, int siter, int diter,
                       double tolsc, int *siter_out, int *diter_out,
                       double *res_out, double *tolsc_out, char *fact_out,
                       double *latency_s, int nthreads)
{
    orc_batch B = { nsys, S, n, kl, ku, trans, M, D1, D2, ld, a, b, c, g,
                    dirichlet, kx, kz, phi_exp, phi_imp, u, x, info, mixed,
                    aiter, siter, diter, tolsc, siter_out, diter_out, res_out,
                    tolsc_out, fact_out, latency_s, 0,
                    PTHREAD_MUTEX_INITIALIZER };
    if (nthreads < 1) nthreads = 1;
    pthread_t *th = malloc((size_t) nthreads * sizeof(pthread_t));
    const double t0 = now_s();
    for (int t = 0; t < nthreads; ++t) pthread_create(&th[t], NULL, batch_worker, &B);
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
    const double dt = now_s() - t0;
    free(th);
    return dt;
}
