// Shared device/host helpers for the GB300 banded-solve kernels.
//
// Complex arithmetic is written out on float2/double2 so every operation is
// explicit (the kernels choose where FMAs go).  Complex reciprocal follows
// R. L. Smith, "Algorithm 116: Complex division", CACM 5(8), 1962.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#define SGB_HD __host__ __device__ __forceinline__

template <typename R> struct cplx;
template <> struct cplx<float>  { using t = float2; };
template <> struct cplx<double> { using t = double2; };
template <typename R> using cplx_t = typename cplx<R>::t;

template <typename R> SGB_HD cplx_t<R> mk(R re, R im) { cplx_t<R> z; z.x = re; z.y = im; return z; }
SGB_HD float2  cadd(float2 a, float2 b)   { return make_float2(a.x + b.x, a.y + b.y); }
SGB_HD double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
SGB_HD float2  csub(float2 a, float2 b)   { return make_float2(a.x - b.x, a.y - b.y); }
SGB_HD double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }

// a * b
SGB_HD float2 cmul(float2 a, float2 b)
{ return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x)); }
SGB_HD double2 cmul(double2 a, double2 b)
{ return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x)); }

// c - a * b   (the rank-1 / axpy update of every kernel)
SGB_HD float2 cfnma(float2 a, float2 b, float2 c)
{
    return make_float2(fmaf(a.y, b.y, fmaf(-a.x, b.x, c.x)),
                       fmaf(-a.y, b.x, fmaf(-a.x, b.y, c.y)));
}
SGB_HD double2 cfnma(double2 a, double2 b, double2 c)
{
    return make_double2(fma(a.y, b.y, fma(-a.x, b.x, c.x)),
                        fma(-a.y, b.x, fma(-a.x, b.y, c.y)));
}
// c + a * b
SGB_HD float2 cfma(float2 a, float2 b, float2 c)
{
    return make_float2(fmaf(-a.y, b.y, fmaf(a.x, b.x, c.x)),
                       fmaf(a.y, b.x, fmaf(a.x, b.y, c.y)));
}
SGB_HD double2 cfma(double2 a, double2 b, double2 c)
{
    return make_double2(fma(-a.y, b.y, fma(a.x, b.x, c.x)),
                        fma(a.y, b.x, fma(a.x, b.y, c.y)));
}
// Two-lane FMA on a pair of floats (fma.rn.f32x2, sm_100 and later): lane k
// of the result is fma(a_k, b_k, c_k), rounded once, as the scalar fmaf.
__device__ __forceinline__ float2 ffma2(float2 a, float2 b, float2 c)
{
    float2 d;
    asm("{\n .reg .b64 ra, rb, rc, rd;\n mov.b64 ra, {%2, %3};\n mov.b64 rb, {%4, %5};\n"
        " mov.b64 rc, {%6, %7};\n fma.rn.f32x2 rd, ra, rb, rc;\n mov.b64 {%0, %1}, rd;\n}"
        : "=f"(d.x), "=f"(d.y) : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return d;
}
// c - a * b as two packed FMAs with cfnma's roundings in cfnma's order, from
// the operand forms la = (-a.x, -a.x), lb = (a.y, -a.y), b and bs = (b.y, b.x).
__device__ __forceinline__ float2 cfnma2(float2 la, float2 lb, float2 b, float2 bs, float2 c)
{
    return ffma2(lb, bs, ffma2(la, b, c));
}

SGB_HD float2  cconj(float2 a)  { return make_float2(a.x, -a.y); }
SGB_HD double2 cconj(double2 a) { return make_double2(a.x, -a.y); }

// 1 / z by the textbook formula conj(z) / |z|^2 after an exact power-of-two
// scaling of z (D. M. Priest, "Efficient scaling for complex division", ACM
// TOMS 30(4), 2004): with s = 2^(-e), e the binary exponent of max(|re|,|im|),
// zs = s z has max(|re|,|im|) in [1, 2), so |zs|^2 in [1, 8) neither
// overflows nor underflows, and 1/z = s conj(zs) / |zs|^2 with one
// correctly rounded reciprocal.  The scale is built from the exponent field
// (clamped so that it stays a normal number); zero, infinite and NaN inputs
// give infinite or NaN results, as a division would.
__device__ __forceinline__ float2 crcp_impl(float2 z)
{
    const float m = fmaxf(fabsf(z.x), fabsf(z.y));
    int e = (int) ((__float_as_uint(m) >> 23) & 0xffu);      // biased exponent
    e = e > 253 ? 253 : e;
    const float sc = __uint_as_float((unsigned) (254 - e) << 23);   // 2^(127 - e)
    const float a = z.x * sc, b = z.y * sc;                         // exact
    const float inv = __frcp_rn(fmaf(a, a, b * b));
    return make_float2(a * inv * sc, -b * inv * sc);
}
__device__ __forceinline__ double2 crcp_impl(double2 z)
{
    const double m = fmax(fabs(z.x), fabs(z.y));
    long long e = (long long) ((__double_as_longlong(m) >> 52) & 0x7ff);
    e = e > 2045 ? 2045 : e;
    const double sc = __longlong_as_double((2046ll - e) << 52);     // 2^(1023 - e)
    const double a = z.x * sc, b = z.y * sc;
    const double inv = __drcp_rn(fma(a, a, b * b));
    return make_double2(a * inv * sc, -b * inv * sc);
}
template <typename R> __device__ __forceinline__ cplx_t<R> crcp(cplx_t<R> z) { return crcp_impl(z); }

// LAPACK's IZAMAX metric |re| + |im|.
template <typename R> SGB_HD R cabs1(cplx_t<R> z)
{ return (z.x < 0 ? -z.x : z.x) + (z.y < 0 ? -z.y : z.y); }
template <typename R> SGB_HD bool cnz(cplx_t<R> z) { return z.x != R(0) || z.y != R(0); }

SGB_HD float2  demote(double2 z) { return make_float2((float) z.x, (float) z.y); }
SGB_HD double2 promote(float2 z) { return make_double2((double) z.x, (double) z.y); }
template <typename R> SGB_HD cplx_t<R> from_z(double2 z);
template <> SGB_HD float2  from_z<float>(double2 z)  { return demote(z); }
template <> SGB_HD double2 from_z<double>(double2 z) { return z; }
template <typename R> SGB_HD double2 to_z(cplx_t<R> z);
template <> SGB_HD double2 to_z<float>(float2 z)   { return promote(z); }
template <> SGB_HD double2 to_z<double>(double2 z) { return z; }

SGB_HD int imin(int a, int b) { return a < b ? a : b; }
SGB_HD int imax(int a, int b) { return a > b ? a : b; }

// Status words written per system instead of traps or asserts.
enum sgb_status : int {
    SGB_OK            = 0,
    SGB_ACTIVE        = 1,   // still refining
    SGB_BAD_GEOMETRY  = -900,
};

#define SGB_CUDA_TRY(call)                                                   \
    do {                                                                     \
        cudaError_t e__ = (call);                                            \
        if (e__ != cudaSuccess) return sgb_set_error(e__, #call, __FILE__, __LINE__); \
    } while (0)

int sgb_set_error(cudaError_t e, const char *what, const char *file, int line);
