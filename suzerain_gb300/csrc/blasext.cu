// Block-assembly and helper drop-ins of the reference's blas_et_al layer that
// build and convert banded operators (suzerain/blas_et_al/blasext.c,
// suzerain/blas_et_al/blas.c), on the GPU, with the reference's names,
// signatures, argument meaning and argument-error positions:
//
//   suzerain_blasext_zgb_{d,dd,ddd,dddd,ddddd}diag_scale_acc_d
//       B <- (sum_k alpha_k D_k) A + beta B   (side 'L') or
//       B <- A (sum_k alpha_k D_k) + beta B   (side 'R')
//       for a real band A, real diagonals D_k and a complex band B;
//   suzerain_blas_zgb_acc_d   B <- alpha A + beta B (the one-diagonal form
//                             with D = 1, as the reference builds it);
//   suzerain_blasext_{z,d}{de,pro}mote   in-place precision changes;
//   suzerain_blasext_zgbnorm1            maximum column sum of |a_ij|.
//
// One thread per band element.  Pointers may be host or device memory.
#include "suzerain_gb300.h"
#include "sgb_internal.h"
#include "sgb_stage.h"
#include "sgb_timer.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <complex>
#include <cstdio>
#include <vector>

using namespace sgb;

namespace {

constexpr int MAXK = 5;

struct DiagArgs {
    int K;
    double2 alpha[MAXK];
    const double *d[MAXK];
    int ldd[MAXK];
};

// Element (i, j) of a band (kl, ku, row stride inc, column stride ld) sits
// at (ku + i - j) inc + j ld.  The scale index is j for side 'R', i for 'L'.
__global__ void k_diag_scale_acc(bool right, int m, int n, int kl, int ku, DiagArgs da,
                                 const double *__restrict__ a, int inca, int lda, double2 beta,
                                 bool beta_one, double2 *__restrict__ b, int incb, int ldb)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;   // band row 0 .. kl + ku
    const int j = blockIdx.y;
    if (r > kl + ku || j >= n) return;
    const int i = j + r - ku;
    if (i < 0 || i >= m) return;
    const int sidx = right ? j : i;
    double tre = 0, tim = 0;                    // sum_k alpha_k d_k[sidx]
    for (int k = 0; k < da.K; ++k) {
        const double dv = da.d[k][(long long) sidx * da.ldd[k]];
        tre += da.alpha[k].x * dv;
        tim += da.alpha[k].y * dv;
    }
    const double av = a[(long long) r * inca + (long long) j * lda];
    double2 &bv = b[(long long) r * incb + (long long) j * ldb];
    if (beta_one) {
        bv.x += tre * av;
        bv.y += tim * av;
    } else if (beta.x == 0 && beta.y == 0) {
        bv = make_double2(tre * av, tim * av);
    } else {
        const double yr = bv.x * beta.x - bv.y * beta.y, yi = bv.x * beta.y + bv.y * beta.x;
        bv = make_double2(yr + tre * av, yi + tim * av);
    }
}

int xerbla(const char *who, int pos)
{
    char msg[160];
    std::snprintf(msg, sizeof msg, "%s: argument %d is invalid", who, pos);
    sgb_set_error(cudaErrorInvalidValue, msg, __FILE__, __LINE__);
    return pos;
}

// The shared body of the K-diagonal forms.  The reference checks, for K >= 2,
// lda a second time where ldb is meant (suzerain/blas_et_al/blasext.c:2170,
// :2255, :2346, :2447); the same checks are made here.
int diag_scale_acc(const char *who, char side, int m, int n, int kl, int ku, int K,
                   const sgb_complex_double *alpha, const double *const *d, const int *ldd,
                   const double *a, int inca, int lda, sgb_complex_double beta,
                   sgb_complex_double *b, int incb, int ldb)
{
    if (kl < 0) return xerbla(who, 4);
    if (ku < 0) return xerbla(who, 5);
    for (int k = 0; k < K; ++k)
        if (ldd[k] < 0) return xerbla(who, 8 + 3 * k);
    if (inca < 1) return xerbla(who, 7 + 3 * K);
    if (lda <= kl + ku) return xerbla(who, 8 + 3 * K);
    if (incb < 1) return xerbla(who, 11 + 3 * K);
    if ((K == 1 ? ldb : lda) <= kl + ku) return xerbla(who, 12 + 3 * K);
    const char s = (char) std::toupper((unsigned char) side);
    if (s != 'R' && s != 'L') return xerbla(who, 1);
    bool all_zero = true;
    DiagArgs da;
    da.K = K;
    for (int k = 0; k < K; ++k) {
        const std::complex<double> z(alpha[k]);
        da.alpha[k] = make_double2(z.real(), z.imag());
        if (z != 0.0) all_zero = false;
        da.ldd[k] = ldd[k];
    }
    const std::complex<double> bt(beta);
    const bool beta_one = (bt == 1.0);
    if ((all_zero && beta_one) || m <= 0 || n <= 0) return 0;
    // extents: a and b span up to (kl + ku) inc + (n - 1) ld + 1 elements;
    // each diagonal max(m, n) strided entries
    const int ncol = s == 'R' ? n : m;
    const size_t na = (size_t) (kl + ku) * inca + (size_t) (ncol - 1) * lda + 1;
    const size_t nb = (size_t) (kl + ku) * incb + (size_t) (ncol - 1) * ldb + 1;
    const int nd = n;   // the scaled index runs over columns 0..n-1 ('R') or rows 0..n-1 ('L')
    Stage sa(a, na * sizeof(double), true), sb(b, nb * sizeof(double2), true);
    Stage sd0(K > 0 ? d[0] : nullptr, K > 0 ? span_bytes(nd, ldd[0], 8) : 0, true);
    Stage sd1(K > 1 ? d[1] : nullptr, K > 1 ? span_bytes(nd, ldd[1], 8) : 0, true);
    Stage sd2(K > 2 ? d[2] : nullptr, K > 2 ? span_bytes(nd, ldd[2], 8) : 0, true);
    Stage sd3(K > 3 ? d[3] : nullptr, K > 3 ? span_bytes(nd, ldd[3], 8) : 0, true);
    Stage sd4(K > 4 ? d[4] : nullptr, K > 4 ? span_bytes(nd, ldd[4], 8) : 0, true);
    Stage *sds[MAXK] = {&sd0, &sd1, &sd2, &sd3, &sd4};
    for (Stage *st : {&sa, &sb, &sd0, &sd1, &sd2, &sd3, &sd4})
        if (st->err != cudaSuccess) return err_of(st->err, who);
    for (int k = 0; k < K; ++k) da.d[k] = static_cast<const double *>(sds[k]->dev);
    // side 'L' covers rows 0..n-1 and columns 0..m-1: the reference recasts a
    // left scaling as a traversal by rows without exchanging m and n
    const int rows = s == 'R' ? m : n, cols = s == 'R' ? n : m;
    dim3 grd((unsigned) ((kl + ku + 1 + 63) / 64), (unsigned) cols);
    count_launch(1);
    k_diag_scale_acc<<<grd, 64>>>(s == 'R', rows, cols, kl, ku, da, static_cast<const double *>(sa.dev),
                                  inca, lda, make_double2(bt.real(), bt.imag()), beta_one,
                                  static_cast<double2 *>(sb.dev), incb, ldb);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = sb.back();
    return err_of(e, who);
}

__global__ void k_demote_z(long long n, const double2 *__restrict__ src, float2 *__restrict__ dst)
{
    const long long i = (long long) blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = make_float2((float) src[i].x, (float) src[i].y);
}
__global__ void k_promote_z(long long n, const float2 *__restrict__ src, double2 *__restrict__ dst)
{
    const long long i = (long long) blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = make_double2((double) src[i].x, (double) src[i].y);
}
__global__ void k_demote_d(long long n, const double *__restrict__ src, float *__restrict__ dst)
{
    const long long i = (long long) blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = (float) src[i];
}
__global__ void k_promote_d(long long n, const float *__restrict__ src, double *__restrict__ dst)
{
    const long long i = (long long) blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = (double) src[i];
}

// In-place precision change of n elements of x (src_el bytes each on entry,
// dst_el bytes on exit).  The source is copied aside on the device first, so
// that no thread reads an element another has already overwritten.
template <typename S, typename D>
int convert(const char *who, int n, void *x, void (*kern)(long long, const S *, D *))
{
    if (n < 0) return -1;
    if (!x) return -2;
    if (n == 0) return 0;
    const size_t wide = (size_t) n * std::max(sizeof(S), sizeof(D));
    Stage sx(x, wide, true);
    if (sx.err != cudaSuccess) return err_of(sx.err, who);
    S *src = nullptr;
    cudaError_t e = cudaMalloc(&src, (size_t) n * sizeof(S));
    if (e == cudaSuccess) e = cudaMemcpy(src, sx.dev, (size_t) n * sizeof(S), cudaMemcpyDeviceToDevice);
    if (e == cudaSuccess) {
        count_launch(1);
        kern<<<(unsigned) ((n + 255) / 256), 256>>>((long long) n, src, static_cast<D *>(sx.dev));
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (src) cudaFree(src);
    if (e == cudaSuccess) e = sx.back();
    return err_of(e, who);
}

__device__ __forceinline__ double absval(double v) { return fabs(v); }
__device__ __forceinline__ double absval(double2 v) { return hypot(v.x, v.y); }

template <typename T>
__global__ void k_gbnorm1(int m, int n, int kl, int ku, const T *__restrict__ a, int lda,
                          double *__restrict__ colsum)
{
    const int j = blockIdx.x * blockDim.y + threadIdx.y;
    if (j >= n) return;
    const int ib = ku - j > 0 ? ku - j : 0;
    const int ie = ku + (kl + 1 < m - j ? kl + 1 : m - j);
    double s = 0;
    for (int i = ib + (int) threadIdx.x; i < ie; i += 32) s += absval(a[(long long) j * lda + i]);
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) colsum[j] = s;
}

}  // namespace

extern "C" int suzerain_blasext_zgb_diag_scale_acc_d(
    char side, int m, int n, int kl, int ku, const sgb_complex_double alpha, const double *d,
    int ldd, const double *a, int inca, int lda, const sgb_complex_double beta,
    sgb_complex_double *b, int incb, int ldb)
{
    const sgb_complex_double al[1] = {alpha};
    const double *ds[1] = {d};
    const int lds[1] = {ldd};
    return diag_scale_acc(__func__, side, m, n, kl, ku, 1, al, ds, lds, a, inca, lda, beta, b,
                          incb, ldb);
}

extern "C" int suzerain_blasext_zgb_ddiag_scale_acc_d(
    char side, int m, int n, int kl, int ku, const sgb_complex_double alpha0, const double *d0,
    int ldd0, const sgb_complex_double alpha1, const double *d1, int ldd1, const double *a,
    int inca, int lda, const sgb_complex_double beta, sgb_complex_double *b, int incb, int ldb)
{
    const sgb_complex_double al[2] = {alpha0, alpha1};
    const double *ds[2] = {d0, d1};
    const int lds[2] = {ldd0, ldd1};
    return diag_scale_acc(__func__, side, m, n, kl, ku, 2, al, ds, lds, a, inca, lda, beta, b,
                          incb, ldb);
}

extern "C" int suzerain_blasext_zgb_dddiag_scale_acc_d(
    char side, int m, int n, int kl, int ku, const sgb_complex_double alpha0, const double *d0,
    int ldd0, const sgb_complex_double alpha1, const double *d1, int ldd1,
    const sgb_complex_double alpha2, const double *d2, int ldd2, const double *a, int inca,
    int lda, const sgb_complex_double beta, sgb_complex_double *b, int incb, int ldb)
{
    const sgb_complex_double al[3] = {alpha0, alpha1, alpha2};
    const double *ds[3] = {d0, d1, d2};
    const int lds[3] = {ldd0, ldd1, ldd2};
    return diag_scale_acc(__func__, side, m, n, kl, ku, 3, al, ds, lds, a, inca, lda, beta, b,
                          incb, ldb);
}

extern "C" int suzerain_blasext_zgb_ddddiag_scale_acc_d(
    char side, int m, int n, int kl, int ku, const sgb_complex_double alpha0, const double *d0,
    int ldd0, const sgb_complex_double alpha1, const double *d1, int ldd1,
    const sgb_complex_double alpha2, const double *d2, int ldd2,
    const sgb_complex_double alpha3, const double *d3, int ldd3, const double *a, int inca,
    int lda, const sgb_complex_double beta, sgb_complex_double *b, int incb, int ldb)
{
    const sgb_complex_double al[4] = {alpha0, alpha1, alpha2, alpha3};
    const double *ds[4] = {d0, d1, d2, d3};
    const int lds[4] = {ldd0, ldd1, ldd2, ldd3};
    return diag_scale_acc(__func__, side, m, n, kl, ku, 4, al, ds, lds, a, inca, lda, beta, b,
                          incb, ldb);
}

extern "C" int suzerain_blasext_zgb_dddddiag_scale_acc_d(
    char side, int m, int n, int kl, int ku, const sgb_complex_double alpha0, const double *d0,
    int ldd0, const sgb_complex_double alpha1, const double *d1, int ldd1,
    const sgb_complex_double alpha2, const double *d2, int ldd2,
    const sgb_complex_double alpha3, const double *d3, int ldd3,
    const sgb_complex_double alpha4, const double *d4, int ldd4, const double *a, int inca,
    int lda, const sgb_complex_double beta, sgb_complex_double *b, int incb, int ldb)
{
    const sgb_complex_double al[5] = {alpha0, alpha1, alpha2, alpha3, alpha4};
    const double *ds[5] = {d0, d1, d2, d3, d4};
    const int lds[5] = {ldd0, ldd1, ldd2, ldd3, ldd4};
    return diag_scale_acc(__func__, side, m, n, kl, ku, 5, al, ds, lds, a, inca, lda, beta, b,
                          incb, ldb);
}

extern "C" int suzerain_blas_zgb_acc_d(int m, int n, int kl, int ku,
                                       const sgb_complex_double alpha, const double *a, int lda,
                                       const sgb_complex_double beta, sgb_complex_double *b,
                                       int ldb)
{
    const double one = 1.0;
    const sgb_complex_double al[1] = {alpha};
    const double *ds[1] = {&one};
    const int lds[1] = {0};
    return diag_scale_acc(__func__, 'R', m, n, kl, ku, 1, al, ds, lds, a, 1, lda, beta, b, 1, ldb);
}

extern "C" int suzerain_blasext_zdemote(const int n, void *x)
{
    return convert<double2, float2>(__func__, n, x, k_demote_z);
}

extern "C" int suzerain_blasext_zpromote(const int n, void *x)
{
    return convert<float2, double2>(__func__, n, x, k_promote_z);
}

extern "C" int suzerain_blasext_ddemote(const int n, void *x)
{
    return convert<double, float>(__func__, n, x, k_demote_d);
}

extern "C" int suzerain_blasext_dpromote(const int n, void *x)
{
    return convert<float, double>(__func__, n, x, k_promote_d);
}

// Maximum column sum of |a_ij| over the band of an m x n matrix, {z,d}langb
// ('1') for the square case (suzerain/blas_et_al/blasext.c:2659-2778).  For
// complex entries |z| is hypot(re, im), the reference's cabs.
template <typename T>
int gbnorm1(const char *who, int m, int n, int kl, int ku, const T *a, int lda, double *norm1)
{
    if (m < 0) return -1;
    if (n < 0) return -2;
    if (kl < 0) return -3;
    if (ku < 0) return -4;
    if (!a) return -5;
    if (lda < kl + ku + 1) return -6;
    if (!norm1) return -7;
    *norm1 = 0;
    if (m == 0 || n == 0) return 0;
    Stage sa(a, ((size_t) (n - 1) * lda + kl + ku + 1) * sizeof(T), true);
    if (sa.err != cudaSuccess) return err_of(sa.err, who);
    double *cs = nullptr;
    cudaError_t e = cudaMalloc(&cs, (size_t) n * sizeof(double));
    if (e == cudaSuccess) {
        count_launch(1);
        k_gbnorm1<T><<<(unsigned) ((n + 3) / 4), dim3(32, 4)>>>(
            m, n, kl, ku, static_cast<const T *>(sa.dev), lda, cs);
        e = cudaGetLastError();
    }
    std::vector<double> h(n);
    if (e == cudaSuccess) e = cudaMemcpy(h.data(), cs, (size_t) n * sizeof(double), cudaMemcpyDeviceToHost);
    if (cs) cudaFree(cs);
    if (e != cudaSuccess) return err_of(e, who);
    double mx = 0;
    for (double v : h) mx = std::fmax(mx, v);   // NaN columns: fmax keeps the other value
    *norm1 = mx;
    return 0;
}

extern "C" int suzerain_blasext_zgbnorm1(const int m, const int n, const int kl, const int ku,
                                         const sgb_complex_double *a, const int lda,
                                         double *norm1)
{
    return gbnorm1(__func__, m, n, kl, ku, reinterpret_cast<const double2 *>(a), lda, norm1);
}

extern "C" int suzerain_blasext_dgbnorm1(const int m, const int n, const int kl, const int ku,
                                         const double *a, const int lda, double *norm1)
{
    return gbnorm1(__func__, m, n, kl, ku, a, lda, norm1);
}
