// Batched band solves with the row-panel LU factor (zgbtrs / cgbtrs
// semantics for trans 'N', 'T', 'C').  One warp per system; the right-hand
// side lives in shared memory while the factor streams from HBM.
//
//   'N':  forward  b <- L^{-1} P b   (interchange, then axpy with column j of L)
//         backward x_j = (b_j - sum_k U(j,j+k) x_{j+k}) / U(j,j)    (row dot)
//   'T'/'C': U^T (U^H) forward in axpy form with row j of U, then
//         L^T (L^H) backward as dot products followed by the interchange.
// The output is written (or accumulated, for refinement x += d) in FP64,
// optionally scattered to natural order x[q(i)] (suzerain_bsmbsm_zaPxpby 'T').
#include "sgb_internal.h"

namespace sgb {

template <typename R>
__device__ __forceinline__ cplx_t<R> warp_csum(cplx_t<R> v)
{
#pragma unroll
    for (int off = 16; off; off >>= 1) {
        v.x += __shfl_xor_sync(0xffffffffu, v.x, off);
        v.y += __shfl_xor_sync(0xffffffffu, v.y, off);
    }
    return v;
}

template <typename R, int TRANS, bool FWD_DONE, bool ACCUM>
__global__ void __launch_bounds__(32)
k_gbtrs(FactorGeom g, int nsys, const cplx_t<R> *__restrict__ fac,
        long long fac_stride, const int *__restrict__ ipiv,
        const double2 *__restrict__ b, const cplx_t<R> *__restrict__ yin,
        long long b_stride, double2 *__restrict__ x, long long x_stride,
        const int *__restrict__ sys_list, const int *__restrict__ d_count,
        bool slot_mode, const int *__restrict__ status, int status_want, int unS, int unn)
{
    using T2 = cplx_t<R>;
    const int lane = threadIdx.x;
    if (d_count && (int) blockIdx.x >= *d_count) return;
    const int s = sys_list ? sys_list[blockIdx.x] : (int) blockIdx.x;
    if (s < 0 || s >= nsys) return;
    if (status && status[s] != status_want) return;
    const long long fi = slot_mode ? (long long) blockIdx.x : (long long) s;
    const int N = g.N, KL = g.KL, UW = g.UW(), KV = UW - 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T2 *xs = reinterpret_cast<T2 *>(smem_raw);
    const T2 *fu = fac + fi * fac_stride;
    const T2 *fl = fu + (long long) N * UW;
    const int *pv = ipiv + fi * N;
    const bool cj = (TRANS == 2);

    for (int i = lane; i < N; i += 32)
        xs[i] = FWD_DONE ? yin[s * b_stride + i] : from_z<R>(b[s * b_stride + i]);
    __syncwarp();

    if (TRANS == 0) {
        if (!FWD_DONE && KL > 0) {
            for (int j = 0; j < N - 1; ++j) {
                const int lm = imin(KL, N - 1 - j);
                const int l = pv[j] - 1;
                if (l != j) {
                    T2 a = xs[j], c = xs[l];
                    __syncwarp();
                    if (lane == 0) { xs[j] = c; xs[l] = a; }
                    __syncwarp();
                }
                const T2 xj = xs[j];
                for (int i = lane; i < lm; i += 32)
                    xs[j + 1 + i] = cfnma(fl[(long long) j * KL + i], xj, xs[j + 1 + i]);
                __syncwarp();
            }
        }
        for (int j = N - 1; j >= 0; --j) {
            T2 acc = mk<R>(R(0), R(0));
            const T2 *ur = fu + (long long) j * UW;
            for (int k = 1 + lane; k <= KV && j + k < N; k += 32)
                acc = cfma(ur[k], xs[j + k], acc);
            acc = warp_csum<R>(acc);
            if (lane == 0) xs[j] = cmul(csub(xs[j], acc), crcp<R>(ur[0]));
            __syncwarp();
        }
    } else {
        for (int j = 0; j < N; ++j) {
            const T2 *ur = fu + (long long) j * UW;
            T2 d = ur[0];
            if (cj) d = cconj(d);
            const T2 xj = cmul(xs[j], crcp<R>(d));
            __syncwarp();
            if (lane == 0) xs[j] = xj;
            for (int k = 1 + lane; k <= KV && j + k < N; k += 32) {
                T2 u = ur[k];
                if (cj) u = cconj(u);
                xs[j + k] = cfnma(u, xj, xs[j + k]);
            }
            __syncwarp();
        }
        if (KL > 0) {
            for (int j = N - 2; j >= 0; --j) {
                const int lm = imin(KL, N - 1 - j);
                T2 acc = mk<R>(R(0), R(0));
                for (int i = lane; i < lm; i += 32) {
                    T2 l = fl[(long long) j * KL + i];
                    if (cj) l = cconj(l);
                    acc = cfma(l, xs[j + 1 + i], acc);
                }
                acc = warp_csum<R>(acc);
                const int l = pv[j] - 1;
                const T2 xj = csub(xs[j], acc);
                __syncwarp();
                if (lane == 0) {
                    if (l != j) { xs[j] = xs[l]; xs[l] = xj; }
                    else xs[j] = xj;
                }
                __syncwarp();
            }
        }
    }
    __syncwarp();
    for (int i = lane; i < N; i += 32) {
        const int o = unS ? (i % unS) * unn + i / unS : i;
        double2 *dst = x + s * x_stride + o;
        const double2 v = to_z<R>(xs[i]);
        if (ACCUM) { double2 t = *dst; t.x += v.x; t.y += v.y; *dst = t; }
        else *dst = v;
    }
}

template <typename R, int TRANS, bool FWD_DONE, bool ACCUM>
static cudaError_t launch_t(const GbtrsArgs &a, cudaStream_t st)
{
    const size_t smem = (size_t) a.g.N * sizeof(cplx_t<R>);
    auto kern = k_gbtrs<R, TRANS, FWD_DONE, ACCUM>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
    if (e != cudaSuccess) return e;
    const int grid = a.sys_list ? a.nlist : a.nsys;
    if (grid == 0) return cudaSuccess;
    kern<<<grid, 32, smem, st>>>(a.g, a.nsys, reinterpret_cast<const cplx_t<R> *>(a.fac),
                                 a.fac_stride, a.ipiv, a.b,
                                 reinterpret_cast<const cplx_t<R> *>(a.yin), a.b_stride,
                                 a.x, a.x_stride, a.sys_list, a.d_count, a.slot_mode,
                                 a.status, a.status_want, a.unpermute_S, a.unpermute_n);
    return cudaGetLastError();
}

template <typename R>
static cudaError_t launch_r(const GbtrsArgs &a, cudaStream_t st)
{
    const int t = a.trans == 'N' ? 0 : (a.trans == 'T' ? 1 : 2);
    if (t == 0) {
        if (a.fwd_done) return a.accumulate ? launch_t<R, 0, true, true>(a, st) : launch_t<R, 0, true, false>(a, st);
        return a.accumulate ? launch_t<R, 0, false, true>(a, st) : launch_t<R, 0, false, false>(a, st);
    }
    if (t == 1) return a.accumulate ? launch_t<R, 1, false, true>(a, st) : launch_t<R, 1, false, false>(a, st);
    return a.accumulate ? launch_t<R, 2, false, true>(a, st) : launch_t<R, 2, false, false>(a, st);
}

cudaError_t launch_gbtrs(const GbtrsArgs &a, cudaStream_t st)
{
    if (a.trans != 'N' && a.fwd_done) return cudaErrorInvalidValue;
    return a.prec == 'Z' ? launch_r<double>(a, st) : launch_r<float>(a, st);
}

}  // namespace sgb
