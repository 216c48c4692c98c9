// FP64 operator applications: the refinement residual r = b - op(A) x over a
// packed band (suzerain_blas_zgbmv, suzerain/blas_et_al/gbmv.def:46-201) or
// over the synthetic model's collocation bands, and the explicit substep
// operator y = P (M + phi L) u (suzerain/bsplineop.c:261-298 per block,
// written in the permuted order that aPxpby('N') produces).
//
// The model form applies the three real bands once per component and mixes
// the results with the S x S coefficients (complex for M, real for D1 and
// D2): ~(3 S n ld + 2 S^2 n) complex-real multiply-adds and S^2 n complex
// ones instead of the S^2 n ld complex ones of the packed band, which
// matters on a part whose FP64 pipe is 1/62 of its FP32 pipe.
#include "sgb_internal.h"

namespace sgb {

__device__ __forceinline__ double warp_dsum(double v)
{
#pragma unroll
    for (int off = 16; off; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

// ---------------------------------------------------------------------------
// Packed band residual
// ---------------------------------------------------------------------------
template <int TRANS>
__global__ void __launch_bounds__(32)
k_residual_packed(int nsys, int N, int KL, int KU, PackedSource src,
                  const double2 *__restrict__ b, long long b_stride,
                  const double2 *__restrict__ x, long long x_stride,
                  double2 *__restrict__ r, long long r_stride,
                  double *__restrict__ rnorm, double *__restrict__ xnorm,
                  const int *__restrict__ sys_list, const int *__restrict__ d_count,
                  const int *__restrict__ status, int status_want)
{
    const int lane = threadIdx.x;
    if (d_count && (int) blockIdx.x >= *d_count) return;
    const int s = sys_list ? sys_list[blockIdx.x] : (int) blockIdx.x;
    if (s < 0 || s >= nsys) return;
    if (status && status[s] != status_want) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double2 *xs = reinterpret_cast<double2 *>(smem_raw);
    double2 *rs = xs + N;
    const double2 *ab = src.ab + s * src.stride + src.off;
    const long long ldab = src.ldab;
    double xn = 0;
    for (int i = lane; i < N; i += 32) {
        const double2 v = x[s * x_stride + i];
        xs[i] = v;
        rs[i] = b[s * b_stride + i];
        xn = fma(v.x, v.x, fma(v.y, v.y, xn));
    }
    __syncwarp();
    if (TRANS == 0) {
        // Each lane owns the rows i == lane (mod 32): no races, no barriers.
        for (int c = 0; c < N; ++c) {
            const double2 xc = xs[c];
            const int i0 = imax(0, c - KU), i1 = imin(N - 1, c + KL);
            int i = i0 + ((lane - i0) & 31);
            for (; i <= i1; i += 32) {
                const double2 a = __ldg(ab + KU + i - c + c * ldab);
                rs[i] = cfnma(a, xc, rs[i]);
            }
        }
    } else {
        for (int c = 0; c < N; ++c) {
            const int i0 = imax(0, c - KU), i1 = imin(N - 1, c + KL);
            double2 acc = make_double2(0, 0);
            for (int i = i0 + lane; i <= i1; i += 32) {
                double2 a = __ldg(ab + KU + i - c + c * ldab);
                if (TRANS == 2) a = cconj(a);
                acc = cfma(a, xs[i], acc);
            }
            acc.x = warp_dsum(acc.x);
            acc.y = warp_dsum(acc.y);
            if (lane == (c & 31)) rs[c] = csub(rs[c], acc);
        }
    }
    __syncwarp();
    double rn = 0;
    for (int i = lane; i < N; i += 32) {
        const double2 v = rs[i];
        r[s * r_stride + i] = v;
        rn = fma(v.x, v.x, fma(v.y, v.y, rn));
    }
    rn = warp_dsum(rn);
    xn = warp_dsum(xn);
    if (lane == 0) {
        if (rnorm) rnorm[s] = sqrt(rn);
        if (xnorm) xnorm[s] = sqrt(xn);
    }
}

// ---------------------------------------------------------------------------
// Model operator: MODE 0 residual r = b - A x (permuted in, permuted out),
// MODE 1 explicit y = A u (natural in, permuted out, Dirichlet rows -> 0,
// plus beta * y_prev when beta != 0).
// ---------------------------------------------------------------------------
template <int MODE>
__global__ void __launch_bounds__(32)
k_model_op(int nsys, ModelSource ms,
           const double2 *__restrict__ b, long long b_stride,
           const double2 *__restrict__ x, long long x_stride,
           double2 *__restrict__ r, long long r_stride,
           double *__restrict__ rnorm, double *__restrict__ xnorm,
           const int *__restrict__ sys_list, const int *__restrict__ d_count,
           const int *__restrict__ status, int status_want, double beta)
{
    const int lane = threadIdx.x;
    if (d_count && (int) blockIdx.x >= *d_count) return;
    const int s = sys_list ? sys_list[blockIdx.x] : (int) blockIdx.x;
    if (s < 0 || s >= nsys) return;
    if (status && status[s] != status_want) return;
    const sgb_case &cs = ms.cs;
    const int S = cs.S, n = cs.n, N = S * n, kl = cs.kl, ku = cs.ku, ld = cs.ld;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double2 *xs = reinterpret_cast<double2 *>(smem_raw);   // permuted x
    // S^2 complex M coefficients, then the D1 and D2 ones, which
    // sgb_block_coefs makes real (a, b scaled by phi): their products with
    // the complex band sums take two multiply-adds instead of four, the same
    // values as the complex product with a zero imaginary part
    double2 *cf = xs + N;
    double *cd = reinterpret_cast<double *>(cf + S * S);   // 2 S^2 reals
    const double kx = ms.kx[s], kz = ms.kz[s];
    for (int idx = lane; idx < S * S; idx += 32) {
        sgb_coef cM, cD1, cD2;
        sgb_block_coefs(&cs, idx / S, idx % S, ms.phi, kx, kz, &cM, &cD1, &cD2);
        cf[idx] = make_double2(cM.re, cM.im);
        cd[idx] = cD1.re;
        cd[S * S + idx] = cD2.re;
    }
    double xn = 0;
    for (int i = lane; i < N; i += 32) {
        // MODE 0: x already permuted.  MODE 1: natural u[f*n + p] -> xs[p*S+f]
        const double2 v = x[s * x_stride + i];
        const int o = MODE == 0 ? i : (i % n) * S + i / n;
        xs[o] = v;
        xn = fma(v.x, v.x, fma(v.y, v.y, xn));
    }
    __syncwarp();
    double rn = 0;
    constexpr int SMAX = 8;
    for (int p = lane; p < n; p += 32) {
        double2 u[SMAX], v[SMAX], w[SMAX];
        for (int f = 0; f < S; ++f) {
            u[f] = make_double2(0, 0); v[f] = u[f]; w[f] = u[f];
        }
        const int q0 = imax(0, p - kl), q1 = imin(n - 1, p + ku);
        for (int q = q0; q <= q1; ++q) {
            const int k = ku + p - q + q * ld;
            const double m = __ldg(cs.M + k), d1 = __ldg(cs.D1 + k), d2 = __ldg(cs.D2 + k);
            for (int f = 0; f < S; ++f) {
                const double2 xv = xs[q * S + f];
                u[f].x = fma(m, xv.x, u[f].x);   u[f].y = fma(m, xv.y, u[f].y);
                v[f].x = fma(d1, xv.x, v[f].x);  v[f].y = fma(d1, xv.y, v[f].y);
                w[f].x = fma(d2, xv.x, w[f].x);  w[f].y = fma(d2, xv.y, w[f].y);
            }
        }
        for (int e = 0; e < S; ++e) {
            const int I = p * S + e;
            double2 y = make_double2(0, 0);
            const bool dir = ((cs.dirichlet_mask >> e) & 1u) && (p == 0 || p == n - 1);
            if (dir) {
                y = MODE == 0 ? xs[I] : make_double2(0, 0);
            } else {
                for (int f = 0; f < S; ++f) {
                    const int ef = e * S + f;
                    y = cfma(cf[ef], u[f], y);
                    const double c1 = cd[ef], c2 = cd[S * S + ef];
                    y.x = fma(c1, v[f].x, y.x);
                    y.y = fma(c1, v[f].y, y.y);
                    y.x = fma(c2, w[f].x, y.x);
                    y.y = fma(c2, w[f].y, y.y);
                }
            }
            double2 out;
            if (MODE == 0) {
                out = csub(b[s * b_stride + I], y);
                rn = fma(out.x, out.x, fma(out.y, out.y, rn));
            } else {
                out = y;
                if (beta != 0.0 && !dir) {
                    const double2 prev = r[s * r_stride + I];
                    out.x = fma(beta, prev.x, out.x);
                    out.y = fma(beta, prev.y, out.y);
                }
            }
            r[s * r_stride + I] = out;
        }
    }
    if (MODE == 0) {
        rn = warp_dsum(rn);
        xn = warp_dsum(xn);
        if (lane == 0) {
            if (rnorm) rnorm[s] = sqrt(rn);
            if (xnorm) xnorm[s] = sqrt(xn);
        }
    }
}

cudaError_t launch_residual(const ResidualArgs &a, cudaStream_t st)
{
    const int grid = a.sys_list ? a.nlist : a.nsys;
    if (grid == 0) return cudaSuccess;
    if (a.model) {
        const int S = a.ms.cs.S, N = S * a.ms.cs.n;
        if (S > 8) return cudaErrorInvalidValue;
        const size_t smem = ((size_t) N + 3 * S * S) * sizeof(double2);
        cudaError_t e = smem_attr((const void *) k_model_op<0>, smem);
        if (e != cudaSuccess) return e;
        k_model_op<0><<<grid, 32, smem, st>>>(a.nsys, a.ms, a.b, a.b_stride, a.x, a.x_stride,
                                              a.r, a.r_stride, a.rnorm2, a.xnorm2, a.sys_list, a.d_count,
                                              a.status, a.status_want, 0.0);
        return cudaGetLastError();
    }
    const size_t smem = 2 * (size_t) a.N * sizeof(double2);
    const int t = a.trans == 'N' ? 0 : (a.trans == 'T' ? 1 : 2);
    void (*kern)(int, int, int, int, PackedSource, const double2 *, long long,
                 const double2 *, long long, double2 *, long long, double *, double *,
                 const int *, const int *, const int *, int) = t == 0 ? k_residual_packed<0> : (t == 1 ? k_residual_packed<1> : k_residual_packed<2>);
    cudaError_t e = smem_attr((const void *) kern, smem);
    if (e != cudaSuccess) return e;
    kern<<<grid, 32, smem, st>>>(a.nsys, a.N, a.KL, a.KU, a.src, a.b, a.b_stride, a.x, a.x_stride,
                                 a.r, a.r_stride, a.rnorm2, a.xnorm2, a.sys_list, a.d_count,
                                 a.status, a.status_want);
    return cudaGetLastError();
}

cudaError_t launch_model_apply(const ApplyArgs &a, cudaStream_t st)
{
    if (a.nsys == 0) return cudaSuccess;
    const int S = a.ms.cs.S, N = S * a.ms.cs.n;
    if (S > 8) return cudaErrorInvalidValue;
    const size_t smem = ((size_t) N + 3 * S * S) * sizeof(double2);
    cudaError_t e = smem_attr((const void *) k_model_op<1>, smem);
    if (e != cudaSuccess) return e;
    k_model_op<1><<<a.nsys, 32, smem, st>>>(a.nsys, a.ms, nullptr, 0, a.u, a.u_stride,
                                            a.y, a.y_stride, nullptr, nullptr, nullptr, nullptr,
                                            nullptr, 0, a.beta);
    return cudaGetLastError();
}

}  // namespace sgb
