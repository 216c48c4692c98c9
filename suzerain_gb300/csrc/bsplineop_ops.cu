// B-spline operator drop-ins beyond the workspace itself (suzerain/bsplineop.h,
// suzerain/bsplineop.c:222-400, 870-1610):
//
//   suzerain_bsplineop_apply, _accumulate, _apply_complex
//       x <- alpha D^m x and y <- alpha D^m x + beta y with the stored
//       transposes D_T (band 'T' products, one thread per output element);
//   suzerain_bsplineop_lu_*, suzerain_bsplineop_luz_*
//       the real and complex operator workspaces: accumulate a linear
//       combination of the D^m into the band (opaccumulate / opform /
//       opform_mass), its 1-norm (opnorm), LU factor (factor, factor_mass),
//       condition estimate (rcond) and transposed solves (solve), with the
//       reference's usage checks (ipiv[0] < 0 marks an operator that is not
//       factored, -ipiv[0] counts the accumulations).
//
// Workspaces live in host memory, as the reference allocates them; every
// computation runs on the GPU (host buffers are staged through device
// memory).  The real factor, condition estimate and solve run in complex
// arithmetic on the band with zero imaginary parts (the complex kernels'
// results there are the real ones up to the rounding of the pivot's
// reciprocal).  Argument and usage errors return the reference's codes:
// SUZERAIN_EINVAL (4) for invalid arguments and wrong call order,
// SUZERAIN_ESANITY (7) when the factorization or estimate reports an error,
// SUZERAIN_ENOMEM (8) for allocation failures.
#include "suzerain_gb300.h"
#include "sgb_internal.h"
#include "sgb_stage.h"
#include "sgb_timer.h"

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>

using namespace sgb;

namespace {

constexpr int kEinval = 4, kEsanity = 7, kEnomem = 8;

int fail(int code, const char *msg)
{
    sgb_set_error(cudaErrorInvalidValue, msg, __FILE__, __LINE__);
    return code;
}

__device__ __forceinline__ double mulr(double a, double x) { return a * x; }
__device__ __forceinline__ double2 mulr(double a, double2 x) { return make_double2(a * x.x, a * x.y); }
__device__ __forceinline__ double addv(double a, double b) { return a + b; }
__device__ __forceinline__ double2 addv(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 cmulv(double2 a, double2 b)
{
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double scalev(double a, double x) { return a * x; }
__device__ __forceinline__ double2 scalev(double2 a, double2 x) { return cmulv(a, x); }
template <typename T> __device__ __forceinline__ T zerov();
template <> __device__ __forceinline__ double zerov<double>() { return 0.0; }
template <> __device__ __forceinline__ double2 zerov<double2>() { return make_double2(0, 0); }

// y[j] <- alpha sum_i A(i, j) x[i] + beta y[j] ('T' band product, A(i, j) at
// a[ku + i - j + j lda]), for right-hand side blockIdx.y.  The sum runs over
// i ascending; beta 0 does not read y.  T is double or double2, S the type
// of alpha and beta.
template <typename T, typename S>
__global__ void k_bop(int n, int kl, int ku, S alpha, const double *__restrict__ a, int lda,
                      const T *__restrict__ x, int incx, long long ldx, S beta, bool beta_zero,
                      T *__restrict__ y, int incy, long long ldy)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const T *xr = x + blockIdx.y * ldx;
    T *yr = y + blockIdx.y * ldy;
    T acc = zerov<T>();
    for (int i = max(0, j - ku); i <= min(n - 1, j + kl); ++i)
        acc = addv(acc, mulr(a[ku + i - j + (long long) j * lda], xr[(long long) i * incx]));
    T *yp = yr + (long long) j * incy;
    const T base = beta_zero ? zerov<T>() : scalev(beta, *yp);
    *yp = addv(base, scalev(alpha, acc));
}

// Copy of operator m's own band (kl[m] + ku[m] + 1 rows of each column)
// into device memory with the workspace's leading dimension.
double *device_operator(const suzerain_bsplineop_workspace *w, int m, cudaError_t &e)
{
    double *d = nullptr;
    const size_t cnt = (size_t) w->ld * w->n;
    e = cudaMalloc(&d, cnt * sizeof(double));
    if (e != cudaSuccess) return nullptr;
    std::vector<double> h(cnt, 0.0);
    const int rows = w->kl[m] + 1 + w->ku[m];
    for (int j = 0; j < w->n; ++j)
        for (int r = 0; r < rows; ++r) h[(size_t) j * w->ld + r] = w->D_T[m][(size_t) j * w->ld + r];
    e = cudaMemcpy(d, h.data(), cnt * sizeof(double), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) { cudaFree(d); return nullptr; }
    return d;
}

size_t strided_bytes(int n, int inc, int nrhs, int ld, size_t el)
{
    if (n <= 0 || nrhs <= 0) return 0;
    return ((size_t) (nrhs - 1) * ld + (size_t) (n - 1) * inc + 1) * el;
}

template <typename T, typename S>
int bop(const char *who, int nderiv, int nrhs, S alpha, const T *x, int incx, int ldx, S beta,
        bool beta_zero, T *y, int incy, int ldy, const suzerain_bsplineop_workspace *w)
{
    const int n = w->n;
    if (nrhs <= 0 || n == 0) return 0;
    if (incx <= 0 || incy <= 0) return fail(kEinval, "bsplineop: increments must be positive");
    cudaError_t e = cudaSuccess;
    double *da = device_operator(w, nderiv, e);
    if (!da) return err_of(e, who);
    {
        Stage sx(x, strided_bytes(n, incx, nrhs, ldx, sizeof(T)), true);
        Stage sy(y, strided_bytes(n, incy, nrhs, ldy, sizeof(T)), !beta_zero);
        if (sx.err || sy.err) e = sx.err ? sx.err : sy.err;
        if (e == cudaSuccess) {
            count_launch(1);
            k_bop<T, S><<<dim3((n + 127) / 128, nrhs), 128>>>(
                n, w->kl[nderiv], w->ku[nderiv], alpha, da, w->ld, static_cast<const T *>(sx.dev),
                incx, ldx, beta, beta_zero, static_cast<T *>(sy.dev), incy, ldy);
            e = cudaGetLastError();
            if (e == cudaSuccess) e = cudaDeviceSynchronize();
            if (e == cudaSuccess) e = sy.back();
        }
    }
    cudaFree(da);
    return err_of(e, who);
}

int check_deriv(const suzerain_bsplineop_workspace *w, int nderiv, int nrhs, int ldx, int ldy)
{
    if (!w) return fail(kEinval, "bsplineop: null workspace");
    if (nderiv < 0 || w->nderiv < nderiv) return fail(kEinval, "nderiv out of range");
    if (nrhs > 1 && ldx < w->n) return fail(kEinval, "nrhs > 1 && ldx < w->n");
    if (nrhs > 1 && ldy < w->n) return fail(kEinval, "nrhs > 1 && ldy < w->n");
    return 0;
}

// x_j <- alpha D^m x_j in place: the product into a device scratch copy,
// then back into x.
template <typename T>
int bop_inplace(const char *who, int nderiv, int nrhs, double alpha, T *x, int incx, int ldx,
                const suzerain_bsplineop_workspace *w)
{
    if (int rc = check_deriv(w, nderiv, nrhs, ldx, w ? w->n : 0)) return rc;
    const int n = w->n;
    if (nrhs <= 0 || n == 0) return 0;
    if (incx <= 0) return fail(kEinval, "bsplineop: increments must be positive");
    Stage sx(x, strided_bytes(n, incx, nrhs, ldx, sizeof(T)), true);
    if (sx.err) return err_of(sx.err, who);
    T *copy = nullptr;
    const size_t bytes = strided_bytes(n, incx, nrhs, ldx, sizeof(T));
    cudaError_t e = cudaMalloc(&copy, bytes);
    if (e != cudaSuccess) return fail(kEnomem, "failed to allocate scratch space");
    e = cudaMemcpy(copy, sx.dev, bytes, cudaMemcpyDeviceToDevice);
    int rc = 0;
    if (e == cudaSuccess) {
        using S = T;
        S al, be;
        if constexpr (sizeof(T) == 8) { al = alpha; be = 0.0; }
        else { al = make_double2(alpha, 0); be = make_double2(0, 0); }
        rc = bop<T, S>(who, nderiv, nrhs, al, copy, incx, ldx, be, true, static_cast<T *>(sx.dev), incx,
                       ldx, w);
        if (rc == 0) e = sx.back();
    }
    cudaFree(copy);
    if (rc) return rc;
    return err_of(e, who);
}

}  // namespace

extern "C" int suzerain_bsplineop_accumulate(int nderiv, int nrhs, double alpha, const double *x,
                                             int incx, int ldx, double beta, double *y, int incy,
                                             int ldy, const suzerain_bsplineop_workspace *w)
{
    if (int rc = check_deriv(w, nderiv, nrhs, ldx, ldy)) return rc;
    if (x == y) return fail(kEinval, "x == y not allowed");
    return bop<double, double>(__func__, nderiv, nrhs, alpha, x, incx, ldx, beta, beta == 0.0, y, incy,
                               ldy, w);
}

extern "C" int suzerain_bsplineop_apply(int nderiv, int nrhs, double alpha, double *x, int incx,
                                        int ldx, const suzerain_bsplineop_workspace *w)
{
    return bop_inplace<double>(__func__, nderiv, nrhs, alpha, x, incx, ldx, w);
}

extern "C" int suzerain_bsplineop_apply_complex(int nderiv, int nrhs, double alpha,
                                                sgb_complex_double *x, int incx, int ldx,
                                                const suzerain_bsplineop_workspace *w)
{
    return bop_inplace<double2>(__func__, nderiv, nrhs, alpha, reinterpret_cast<double2 *>(x), incx,
                                ldx, w);
}

extern "C" int suzerain_bsplineop_accumulate_complex(int nderiv, int nrhs,
                                                     const sgb_complex_double alpha,
                                                     const sgb_complex_double *x, int incx, int ldx,
                                                     const sgb_complex_double beta,
                                                     sgb_complex_double *y, int incy, int ldy,
                                                     const suzerain_bsplineop_workspace *w)
{
    if (int rc = check_deriv(w, nderiv, nrhs, ldx, ldy)) return rc;
    if ((const void *) x == (const void *) y) return fail(kEinval, "x == y not allowed");
    double2 al, be;
    std::memcpy(&al, &alpha, sizeof al);
    std::memcpy(&be, &beta, sizeof be);
    return bop<double2, double2>(__func__, nderiv, nrhs, al, reinterpret_cast<const double2 *>(x), incx,
                                 ldx, be, be.x == 0 && be.y == 0, reinterpret_cast<double2 *>(y), incy,
                                 ldy, w);
}

// ---------------------------------------------------------------------------
// Operator workspaces
// ---------------------------------------------------------------------------
namespace {

// A (ld x n, gbtrf layout: the unfactored band starts at row kl) <- the
// accumulation of one opaccumulate call.  ncoef == 0 scales every stored
// entry; otherwise, within the (kl, ku) band of the n x n matrix, column by
// column as the reference's band accumulations: a <- c0 D0 + scale a, then
// a <- ck Dk + a for k >= 1 (scale_zero: the storage was zeroed first).
// ops holds the nderiv + 1 operators with their common leading dimension
// ldw, each viewed with the workspace's maximal (kl, ku).
template <typename T>
__global__ void k_opacc(int n, int kl, int ku, int ld, T *__restrict__ A, int ncoef,
                        const T *__restrict__ coef, T scale, bool scale_zero,
                        const double *__restrict__ ops, int ldw, long long opstride)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;     // row of the storage
    const int j = blockIdx.y;
    if (r >= ld || j >= n) return;
    T *p = A + (long long) j * ld + r;
    if (ncoef == 0) { *p = scalev(scale, *p); return; }
    if (scale_zero) *p = zerov<T>();
    // band element (i, j) of the unfactored operator sits at row kl + ku + i - j
    const int i = j + r - kl - ku;
    if (r < kl || i < 0 || i >= n || i < j - ku || i > j + kl) return;
    T v = *p;
    for (int k = 0; k < ncoef; ++k) {
        const double d = ops[k * opstride + (long long) j * ldw + ku + i - j];
        const T term = mulr(d, coef[k]);
        v = (k == 0 && !scale_zero) ? addv(term, scalev(scale, v)) : addv(term, v);
    }
    *p = v;
}

__global__ void k_promote_band(long long cnt, const double *__restrict__ a, double2 *__restrict__ z)
{
    const long long t = (long long) blockIdx.x * blockDim.x + threadIdx.x;
    if (t < cnt) z[t] = make_double2(a[t], 0.0);
}
__global__ void k_real_part(long long cnt, const double2 *__restrict__ z, double *__restrict__ a)
{
    const long long t = (long long) blockIdx.x * blockDim.x + threadIdx.x;
    if (t < cnt) a[t] = z[t].x;
}

// Right-hand sides: gather (strided, incb / ldb) into / scatter from an
// n x nrhs contiguous complex block.
template <typename T>
__global__ void k_gather(int n, int nrhs, const T *__restrict__ b, int incb, long long ldb,
                         double2 *__restrict__ z)
{
    const long long t = (long long) blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long) n * nrhs) return;
    const int i = (int) (t % n), c = (int) (t / n);
    const T v = b[c * ldb + (long long) i * incb];
    if constexpr (sizeof(T) == 8) z[t] = make_double2(v, 0.0);
    else z[t] = v;
}
template <typename T>
__global__ void k_scatter(int n, int nrhs, const double2 *__restrict__ z, T *__restrict__ b, int incb,
                          long long ldb)
{
    const long long t = (long long) blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long) n * nrhs) return;
    const int i = (int) (t % n), c = (int) (t / n);
    if constexpr (sizeof(T) == 8) b[c * ldb + (long long) i * incb] = z[t].x;
    else b[c * ldb + (long long) i * incb] = z[t];
}

template <typename W, typename T>
W *lu_alloc_impl(const suzerain_bsplineop_workspace *w)
{
    if (!w) return nullptr;
    W *luw = static_cast<W *>(std::calloc(1, sizeof(W)));
    if (!luw) return nullptr;
    luw->n = w->n;
    luw->kl = w->max_kl;
    luw->ku = w->max_ku;
    luw->ld = 2 * luw->kl + luw->ku + 1;          // room for the factor's fill
    luw->ipiv = static_cast<int *>(std::calloc((size_t) std::max(1, w->n), sizeof(int)));
    luw->A_T = static_cast<decltype(luw->A_T)>(std::calloc((size_t) luw->ld * std::max(1, w->n), sizeof(T)));
    if (!luw->ipiv || !luw->A_T) {
        std::free(luw->ipiv);
        std::free(luw->A_T);
        std::free(luw);
        return nullptr;
    }
    luw->ipiv[0] = -1;                            // not factored
    return luw;
}

template <typename W>
void lu_free_impl(W *luw)
{
    if (!luw) return;
    std::free(luw->A_T);
    std::free(luw->ipiv);
    std::free(luw);
}

template <typename W, typename T>
int opaccumulate_impl(const char *who, int ncoef, const T *coef, const suzerain_bsplineop_workspace *w,
                      T scale, bool scale_is_zero, W *luw)
{
    const bool scale_zero = ncoef > 0 && scale_is_zero;   // the storage is zeroed first
    if (!w || !luw) return fail(kEinval, "bsplineop: null workspace");
    if (ncoef < 0) return fail(kEinval, "Number of coefficients cannot be negative");
    if (ncoef > w->nderiv + 1) return fail(kEinval, "More coefficients provided than derivatives available");
    if (luw->n < w->n) return fail(kEinval, "Incompatible workspaces: luw->n < w->n");
    if (luw->ld < 2 * w->max_kl + w->max_ku + 1) return fail(kEinval, "Incompatible workspaces: luw->ld too small");
    if (!scale_is_zero && luw->ipiv[0] >= 0) return fail(kEinval, "Unable to accumulate into a factored operator");
    if (ncoef > 0 && !coef) return fail(kEinval, "bsplineop: null coefficients");
    const int n = luw->n, ld = luw->ld;
    const size_t abytes = (size_t) ld * n * sizeof(T);
    // the nderiv + 1 operators, each at its own maximal-band view
    const int nop = std::max(1, ncoef);
    const size_t opstride = (size_t) w->ld * n;          // columns past w->n stay zero
    std::vector<double> hops(opstride * nop, 0.0);
    for (int k = 0; k < ncoef; ++k) {
        const double *view = w->D_T[k] - (w->max_ku - w->ku[k]);
        for (int j = 0; j < w->n; ++j)
            for (int r = 0; r < w->ld; ++r) {
                // rows of the maximal view that hold operator k's band
                const int i = j + r - w->max_ku;
                if (i >= j - w->ku[k] && i <= j + w->kl[k])
                    hops[k * opstride + (size_t) j * w->ld + r] = view[(size_t) j * w->ld + r];
            }
    }
    T *dA = nullptr, *dc = nullptr;
    double *dops = nullptr;
    cudaError_t e = cudaMalloc(&dA, abytes);
    if (e == cudaSuccess) e = cudaMalloc(&dops, hops.size() * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&dc, (size_t) nop * sizeof(T));
    if (e != cudaSuccess) {
        cudaFree(dA); cudaFree(dops); cudaFree(dc);
        return fail(kEnomem, "bsplineop opaccumulate: device memory");
    }
    if (!scale_zero) e = cudaMemcpy(dA, luw->A_T, abytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dops, hops.data(), hops.size() * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && ncoef > 0) e = cudaMemcpy(dc, coef, (size_t) ncoef * sizeof(T), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        count_launch(1);
        k_opacc<T><<<dim3((ld + 63) / 64, n), 64>>>(n, w->max_kl, w->max_ku, ld, dA, ncoef, dc, scale,
                                                   scale_zero, dops, w->ld, (long long) opstride);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(luw->A_T, dA, abytes, cudaMemcpyDeviceToHost);
    cudaFree(dA); cudaFree(dops); cudaFree(dc);
    if (e != cudaSuccess) return err_of(e, who);
    luw->ipiv[0] = std::min(-1, luw->ipiv[0] - 1);   // -ipiv[0]: accumulations so far
    return 0;
}

// The factor of the (complex or real) operator in device memory as complex
// gbtrf storage: a promoted copy for a real workspace.
template <typename T>
double2 *device_complex_band(const T *A, size_t cnt, cudaError_t &e)
{
    double2 *z = nullptr;
    e = cudaMalloc(&z, cnt * sizeof(double2));
    if (e != cudaSuccess) return nullptr;
    if constexpr (sizeof(T) == 16) {
        e = cudaMemcpy(z, A, cnt * sizeof(double2), cudaMemcpyHostToDevice);
    } else {
        double *d = nullptr;
        e = cudaMalloc(&d, cnt * sizeof(double));
        if (e == cudaSuccess) e = cudaMemcpy(d, A, cnt * sizeof(double), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) {
            count_launch(1);
            k_promote_band<<<(unsigned) ((cnt + 255) / 256), 256>>>((long long) cnt, d, z);
            e = cudaGetLastError();
        }
        cudaFree(d);
    }
    if (e != cudaSuccess) { cudaFree(z); return nullptr; }
    return z;
}

template <typename T>
cudaError_t band_back(const double2 *z, T *A, size_t cnt)
{
    if constexpr (sizeof(T) == 16) return cudaMemcpy(A, z, cnt * sizeof(double2), cudaMemcpyDeviceToHost);
    double *d = nullptr;
    cudaError_t e = cudaMalloc(&d, cnt * sizeof(double));
    if (e == cudaSuccess) {
        count_launch(1);
        k_real_part<<<(unsigned) ((cnt + 255) / 256), 256>>>((long long) cnt, z, d);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(A, d, cnt * sizeof(double), cudaMemcpyDeviceToHost);
    cudaFree(d);
    return e;
}

template <typename W, typename T>
int factor_impl(const char *who, W *luw)
{
    if (!luw) return fail(kEinval, "bsplineop: null workspace");
    if (luw->ipiv[0] >= 0) return fail(kEinval, "Unable to factor an already-factored operator");
    const size_t cnt = (size_t) luw->ld * luw->n;
    cudaError_t e = cudaSuccess;
    double2 *z = device_complex_band(luw->A_T, cnt, e);
    if (!z) return err_of(e, who);
    int *dpv = nullptr;
    e = cudaMalloc(&dpv, (size_t) luw->n * sizeof(int));
    int info = 0;
    if (e == cudaSuccess)
        info = suzerain_lapack_zgbtrf(luw->n, luw->n, luw->kl, luw->ku,
                                      reinterpret_cast<sgb_complex_double *>(z), luw->ld, dpv);
    if (e == cudaSuccess) e = band_back(z, luw->A_T, cnt);
    if (e == cudaSuccess) e = cudaMemcpy(luw->ipiv, dpv, (size_t) luw->n * sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(z);
    cudaFree(dpv);
    if (e != cudaSuccess) return err_of(e, who);
    if (info) return fail(kEsanity, "suzerain_lapack_zgbtrf reported an error");
    return 0;
}

template <typename W>
int opnorm_impl(const W *luw, double *norm)
{
    if (!luw || !norm) return fail(kEinval, "bsplineop: null argument");
    if (luw->ipiv[0] >= 0) return fail(kEinval, "Unable to obtain norm from a factored operator");
    int info;
    // the infinity norm of A is the 1-norm of the stored A^T (band at A_T + kl)
    if constexpr (sizeof(*luw->A_T) == 16)
        info = suzerain_blasext_zgbnorm1(luw->n, luw->n, luw->kl, luw->ku, luw->A_T + luw->kl, luw->ld, norm);
    else
        info = suzerain_blasext_dgbnorm1(luw->n, luw->n, luw->kl, luw->ku, luw->A_T + luw->kl, luw->ld, norm);
    if (info) return fail(kEsanity, "band 1-norm reported an error");
    return 0;
}

template <typename W>
int rcond_impl(const char *who, double norm, double *rcond, const W *luw)
{
    if (!luw || !rcond) return fail(kEinval, "bsplineop: null argument");
    if (luw->ipiv[0] < 0) return fail(kEinval, "factor not called before rcond");
    const size_t cnt = (size_t) luw->ld * luw->n;
    cudaError_t e = cudaSuccess;
    double2 *z = device_complex_band(luw->A_T, cnt, e);
    if (!z) return err_of(e, who);
    // the infinity condition number of A is the 1-norm one of A^T
    const int info = suzerain_lapack_zgbcon('1', luw->n, luw->kl, luw->ku,
                                            reinterpret_cast<const sgb_complex_double *>(z), luw->ld,
                                            luw->ipiv, norm, rcond, nullptr, nullptr);
    cudaFree(z);
    if (info) return fail(kEsanity, "suzerain_lapack_zgbcon reported an error");
    return 0;
}

template <typename W, typename T>
int solve_impl(const char *who, int nrhs, T *B, int incb, int ldb, const W *luw)
{
    if (!luw) return fail(kEinval, "bsplineop: null workspace");
    if (luw->ipiv[0] < 0) return fail(kEinval, "factor not called before solve");
    const int n = luw->n;
    if (nrhs <= 0 || n == 0) return 0;
    if (incb <= 0) return fail(kEinval, "bsplineop solve: incb must be positive");
    if (incb == 1 && nrhs > 1 && ldb < n)          // the contiguous solve's gbtrs argument check
        return fail(kEsanity, "suzerain_lapack_zgbtrs reported error -10");
    const size_t cnt = (size_t) luw->ld * n;
    cudaError_t e = cudaSuccess;
    double2 *z = device_complex_band(luw->A_T, cnt, e);
    if (!z) return err_of(e, who);
    Stage sb(B, strided_bytes(n, incb, nrhs, ldb, sizeof(T)), true);
    double2 *rhs = nullptr;
    if (sb.err == cudaSuccess) e = cudaMalloc(&rhs, (size_t) n * nrhs * sizeof(double2));
    else e = sb.err;
    int info = 0;
    const unsigned g = (unsigned) (((long long) n * nrhs + 255) / 256);
    if (e == cudaSuccess) {
        count_launch(1);
        k_gather<T><<<g, 256>>>(n, nrhs, static_cast<const T *>(sb.dev), incb, ldb, rhs);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        info = suzerain_lapack_zgbtrs('T', n, luw->kl, luw->ku, nrhs,
                                      reinterpret_cast<const sgb_complex_double *>(z), luw->ld, luw->ipiv,
                                      reinterpret_cast<sgb_complex_double *>(rhs), n);
    if (e == cudaSuccess && info == 0) {
        count_launch(1);
        k_scatter<T><<<g, 256>>>(n, nrhs, rhs, static_cast<T *>(sb.dev), incb, ldb);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
        if (e == cudaSuccess) e = sb.back();
    }
    cudaFree(z);
    cudaFree(rhs);
    if (e != cudaSuccess) return err_of(e, who);
    if (info) return fail(kEsanity, "suzerain_lapack_zgbtrs reported an error");
    return 0;
}

}  // namespace

// ---- real operator workspace (suzerain/bsplineop.c:930-1262) --------------
extern "C" suzerain_bsplineop_lu_workspace *
suzerain_bsplineop_lu_alloc(const suzerain_bsplineop_workspace *w)
{
    return lu_alloc_impl<suzerain_bsplineop_lu_workspace, double>(w);
}

extern "C" void suzerain_bsplineop_lu_free(suzerain_bsplineop_lu_workspace *luw)
{
    lu_free_impl(luw);
}

extern "C" int suzerain_bsplineop_lu_opaccumulate(int ncoefficients, const double *coefficients,
                                                  const suzerain_bsplineop_workspace *w,
                                                  const double scale,
                                                  suzerain_bsplineop_lu_workspace *luw)
{
    return opaccumulate_impl(__func__, ncoefficients, coefficients, w, scale, scale == 0.0, luw);
}

extern "C" int suzerain_bsplineop_lu_opnorm(const suzerain_bsplineop_lu_workspace *luw, double *norm)
{
    return opnorm_impl(luw, norm);
}

extern "C" int suzerain_bsplineop_lu_factor(suzerain_bsplineop_lu_workspace *luw)
{
    return factor_impl<suzerain_bsplineop_lu_workspace, double>(__func__, luw);
}

extern "C" int suzerain_bsplineop_lu_rcond(const double norm, double *rcond,
                                           const suzerain_bsplineop_lu_workspace *luw)
{
    return rcond_impl(__func__, norm, rcond, luw);
}

extern "C" int suzerain_bsplineop_lu_solve(int nrhs, double *B, int incb, int ldb,
                                           const suzerain_bsplineop_lu_workspace *luw)
{
    return solve_impl(__func__, nrhs, B, incb, ldb, luw);
}

extern "C" int suzerain_bsplineop_lu_opform(int ncoefficients, const double *coefficients,
                                            const suzerain_bsplineop_workspace *w,
                                            suzerain_bsplineop_lu_workspace *luw)
{
    return suzerain_bsplineop_lu_opaccumulate(ncoefficients, coefficients, w, 0.0, luw);
}

extern "C" int suzerain_bsplineop_lu_opform_mass(const suzerain_bsplineop_workspace *w,
                                                 suzerain_bsplineop_lu_workspace *luw)
{
    const double one = 1.0;
    return suzerain_bsplineop_lu_opform(1, &one, w, luw);
}

extern "C" int suzerain_bsplineop_lu_factor_mass(const suzerain_bsplineop_workspace *w,
                                                 suzerain_bsplineop_lu_workspace *luw)
{
    if (int rc = suzerain_bsplineop_lu_opform_mass(w, luw)) return rc;
    return suzerain_bsplineop_lu_factor(luw);
}

// ---- complex operator workspace (suzerain/bsplineop.c:1265-1610) ----------
extern "C" suzerain_bsplineop_luz_workspace *
suzerain_bsplineop_luz_alloc(const suzerain_bsplineop_workspace *w)
{
    return lu_alloc_impl<suzerain_bsplineop_luz_workspace, double2>(w);
}

extern "C" void suzerain_bsplineop_luz_free(suzerain_bsplineop_luz_workspace *luzw)
{
    lu_free_impl(luzw);
}

extern "C" int suzerain_bsplineop_luz_opaccumulate(int ncoefficients,
                                                   const sgb_complex_double *coefficients,
                                                   const suzerain_bsplineop_workspace *w,
                                                   const sgb_complex_double scale,
                                                   suzerain_bsplineop_luz_workspace *luzw)
{
    double2 sc;
    std::memcpy(&sc, &scale, sizeof sc);
    return opaccumulate_impl(__func__, ncoefficients, reinterpret_cast<const double2 *>(coefficients), w,
                             sc, sc.x == 0.0 && sc.y == 0.0, luzw);
}

extern "C" int suzerain_bsplineop_luz_opnorm(const suzerain_bsplineop_luz_workspace *luzw, double *norm)
{
    return opnorm_impl(luzw, norm);
}

extern "C" int suzerain_bsplineop_luz_factor(suzerain_bsplineop_luz_workspace *luzw)
{
    return factor_impl<suzerain_bsplineop_luz_workspace, double2>(__func__, luzw);
}

extern "C" int suzerain_bsplineop_luz_rcond(const double norm, double *rcond,
                                            const suzerain_bsplineop_luz_workspace *luzw)
{
    return rcond_impl(__func__, norm, rcond, luzw);
}

extern "C" int suzerain_bsplineop_luz_solve(int nrhs, sgb_complex_double *B, int incb, int ldb,
                                            const suzerain_bsplineop_luz_workspace *luzw)
{
    return solve_impl(__func__, nrhs, reinterpret_cast<double2 *>(B), incb, ldb, luzw);
}

extern "C" int suzerain_bsplineop_luz_opform(int ncoefficients, const sgb_complex_double *coefficients,
                                             const suzerain_bsplineop_workspace *w,
                                             suzerain_bsplineop_luz_workspace *luzw)
{
    sgb_complex_double zero;
    std::memset(&zero, 0, sizeof zero);
    return suzerain_bsplineop_luz_opaccumulate(ncoefficients, coefficients, w, zero, luzw);
}

extern "C" int suzerain_bsplineop_luz_opform_mass(const suzerain_bsplineop_workspace *w,
                                                  suzerain_bsplineop_luz_workspace *luzw)
{
    sgb_complex_double one;
    const double v[2] = {1.0, 0.0};
    std::memcpy(&one, v, sizeof one);
    return suzerain_bsplineop_luz_opform(1, &one, w, luzw);
}

extern "C" int suzerain_bsplineop_luz_factor_mass(const suzerain_bsplineop_workspace *w,
                                                  suzerain_bsplineop_luz_workspace *luzw)
{
    if (int rc = suzerain_bsplineop_luz_opform_mass(w, luzw)) return rc;
    return suzerain_bsplineop_luz_factor(luzw);
}
