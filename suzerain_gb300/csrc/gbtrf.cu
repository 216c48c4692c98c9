// Batched partial-pivot band LU kernels; see gbtrf.cuh for the design.
#include "gbtrf.cuh"
#include "sgb_internal.h"

#include <climits>

namespace sgb {

template <typename R>
__device__ __forceinline__ cplx_t<R> model_entry(const sgb_case &cs,
                                                 const cplx_t<R> *coef,
                                                 int i, int j)
{
    const int S = cs.S;
    const int p = i / S, e = i - p * S;
    const int q = j / S, f = j - q * S;
    if (((cs.dirichlet_mask >> e) & 1u) && (p == 0 || p == cs.n - 1))
        return mk<R>(i == j ? R(1) : R(0), R(0));
    const int d = p - q;
    if (d > cs.kl || -d > cs.ku) return mk<R>(R(0), R(0));
    const int k = cs.ku + d + q * cs.ld;
    const int ef = e * S + f;
    const double m = __ldg(cs.M + k), d1 = __ldg(cs.D1 + k), d2 = __ldg(cs.D2 + k);
    const cplx_t<R> a = coef[ef], b = coef[S * S + ef], c = coef[2 * S * S + ef];
    if constexpr (sizeof(R) == 8) {
        sgb_coef cM{a.x, a.y}, cD1{b.x, b.y}, cD2{c.x, c.y};
        double re, im;
        sgb_block_entry(cM, cD1, cD2, m, d1, d2, &re, &im);
        return mk<R>(re, im);
    } else {
        const float mf = (float) m, d1f = (float) d1, d2f = (float) d2;
        return mk<R>(fmaf(c.x, d2f, fmaf(b.x, d1f, a.x * mf)),
                     fmaf(c.y, d2f, fmaf(b.y, d1f, a.y * mf)));
    }
}

template <typename R, bool MODEL, bool FWD>
__global__ void __launch_bounds__(32)
k_gbtrf(FactorGeom g, int nsys, PackedSource src, ModelSource ms,
        cplx_t<R> *__restrict__ fac, long long fac_stride,
        int *__restrict__ ipiv, int *__restrict__ info,
        const double2 *__restrict__ rhs, long long rhs_stride,
        cplx_t<R> *__restrict__ y, long long y_stride,
        const int *__restrict__ sys_list, const int *__restrict__ d_count,
        bool slot_mode)
{
    using T2 = cplx_t<R>;
    const int lane = threadIdx.x;
    if (d_count && (int) blockIdx.x >= *d_count) return;
    const int s = sys_list ? sys_list[blockIdx.x] : (int) blockIdx.x;
    if (s < 0 || s >= nsys) return;
    const long long fi = slot_mode ? (long long) blockIdx.x : (long long) s;

    const int N = g.N, KL = g.KL, KU = g.KU, RR = g.R(), C = g.C(), UW = g.UW();
    const int S = MODEL ? ms.cs.S : 1;

    extern __shared__ __align__(16) unsigned char smem_raw[];
    T2 *win = reinterpret_cast<T2 *>(smem_raw);
    T2 *lmul = win + RR * C;
    T2 *rslot = lmul + RR;
    T2 *coef = rslot + RR;
    int *label = reinterpret_cast<int *>(coef + (MODEL ? 3 * S * S : 0));
    int *pos = label + RR;

    T2 *fu = fac + fi * fac_stride;                // U rows
    T2 *fl = fu + (long long) N * UW;              // L columns
    int *pv = ipiv + fi * N;

    if (MODEL) {
        const double kx = ms.kx[s], kz = ms.kz[s];
        for (int idx = lane; idx < S * S; idx += 32) {
            sgb_coef cM, cD1, cD2;
            sgb_block_coefs(&ms.cs, idx / S, idx % S, ms.phi, kx, kz, &cM, &cD1, &cD2);
            coef[idx] = mk<R>((R) cM.re, (R) cM.im);
            coef[S * S + idx] = mk<R>((R) cD1.re, (R) cD1.im);
            coef[2 * S * S + idx] = mk<R>((R) cD2.re, (R) cD2.im);
        }
        __syncwarp();
    }

    auto A = [&](int i, int j) -> T2 {
        if constexpr (MODEL) return model_entry<R>(ms.cs, coef, i, j);
        else return from_z<R>(src.entry(s, KU, i, j));
    };

    // Initial window: logical rows 0..RR-1 in slots 0..RR-1, columns 0..C-1.
    for (int idx = lane; idx < RR * C; idx += 32) {
        const int sl = idx / C, c = idx - sl * C;
        T2 v = mk<R>(R(0), R(0));
        if (sl < N && c < N && c - sl <= KU && sl - c <= KL) v = A(sl, c);
        win[idx] = v;
    }
    for (int sl = lane; sl < RR; sl += 32) {
        label[sl] = sl < N ? sl : INT_MAX;
        pos[sl] = sl;
        if (FWD) rslot[sl] = sl < N ? from_z<R>(rhs[s * rhs_stride + sl]) : mk<R>(R(0), R(0));
    }
    __syncwarp();

    int ju = 0, inf = 0, cj = 0;
    for (int j = 0; j < N; ++j) {
        const int km = imin(KL, N - 1 - j);

        // ---- pivot search (IZAMAX semantics) --------------------------------
        R best = R(-1);
        int bl = INT_MAX, bs = -1;
        for (int sl = lane; sl < RR; sl += 32) {
            const int lb = label[sl];
            if (lb >= j && lb <= j + km) {
                R m = cabs1<R>(win[sl * C + cj]);
                if (m != m) m = (lb == j) ? R(INFINITY) : R(-1);
                if (m > best || (m == best && lb < bl)) { best = m; bl = lb; bs = sl; }
            }
        }
#pragma unroll
        for (int off = 16; off; off >>= 1) {
            const R ob = __shfl_xor_sync(0xffffffffu, best, off);
            const int ol = __shfl_xor_sync(0xffffffffu, bl, off);
            const int os = __shfl_xor_sync(0xffffffffu, bs, off);
            if (ob > best || (ob == best && ol < bl)) { best = ob; bl = ol; bs = os; }
        }
        const int psl = bs, p = bl;
        const T2 piv = win[psl * C + cj];
        const int sj = pos[j % RR];
        if (lane == 0) pv[j] = p + 1;

        if (cnz<R>(piv)) {
            ju = imax(ju, imin(j + KU + (p - j), N - 1));
            const T2 rp = crcp<R>(piv);
            for (int sl = lane; sl < RR; sl += 32) {
                const int lb = label[sl];
                T2 l = mk<R>(R(0), R(0));
                if (sl != psl && lb >= j && lb <= j + km) l = cmul(win[sl * C + cj], rp);
                lmul[sl] = l;
            }
            __syncwarp();
            if (lane == 0 && psl != sj) { label[sj] = p; pos[p % RR] = sj; }
            __syncwarp();
            for (int i = lane; i < KL; i += 32) {
                T2 v = mk<R>(R(0), R(0));
                if (i < km) v = lmul[pos[(j + 1 + i) % RR]];
                fl[(long long) j * KL + i] = v;
            }
            for (int k = lane; k < UW; k += 32) {
                int cc = cj + k; if (cc >= C) cc -= C;
                fu[(long long) j * UW + k] = win[psl * C + cc];
            }
            if (FWD) {
                const T2 yj = rslot[psl];
                if (lane == 0) y[s * y_stride + j] = yj;
                for (int sl = lane; sl < RR; sl += 32)
                    if (sl != psl) rslot[sl] = cfnma(lmul[sl], yj, rslot[sl]);
            }
            // rank-1 update of the live window, columns j+1..ju
            for (int c0 = j + 1 + lane; c0 <= ju; c0 += 32) {
                int cc = cj + (c0 - j); if (cc >= C) cc -= C;
                const T2 u = win[psl * C + cc];
                if (cnz<R>(u)) {
                    for (int sl = 0; sl < RR; ++sl) {
                        if (sl == psl) continue;
                        const T2 l = lmul[sl];
                        win[sl * C + cc] = cfnma(l, u, win[sl * C + cc]);
                    }
                }
            }
        } else {
            if (inf == 0) inf = j + 1;
            for (int i = lane; i < KL; i += 32) fl[(long long) j * KL + i] = mk<R>(R(0), R(0));
            for (int k = lane; k < UW; k += 32) {
                int cc = cj + k; if (cc >= C) cc -= C;
                fu[(long long) j * UW + k] = win[psl * C + cc];
            }
            if (FWD && lane == 0) y[s * y_stride + j] = rslot[psl];
        }
        __syncwarp();

        // ---- retire the pivot slot; column j's storage becomes column j+C ----
        for (int sl = lane; sl < RR; sl += 32) win[sl * C + cj] = mk<R>(R(0), R(0));
        __syncwarp();
        const int nr = j + RR;
        if (nr < N) {
            for (int k = lane; k < C; k += 32) {
                const int col = j + 1 + k;
                int cc = cj + 1 + k; if (cc >= C) cc -= C;
                win[psl * C + cc] = col < N ? A(nr, col) : mk<R>(R(0), R(0));
            }
            if (lane == 0) {
                label[psl] = nr;
                pos[nr % RR] = psl;
                if (FWD) rslot[psl] = from_z<R>(rhs[s * rhs_stride + nr]);
            }
        } else if (lane == 0) {
            label[psl] = INT_MAX;
            if (FWD) rslot[psl] = mk<R>(R(0), R(0));
        }
        cj = (cj + 1 == C) ? 0 : cj + 1;
        __syncwarp();
    }
    if (lane == 0) info[fi] = inf;
}

size_t gbtrf_smem_bytes(int prec_bytes, const FactorGeom &g, int S)
{
    const int R_ = g.R(), C_ = g.C();
    const size_t el = 2 * (size_t) prec_bytes;
    return (size_t) R_ * C_ * el + 2 * (size_t) R_ * el + 3 * (size_t) S * S * el
         + 2 * (size_t) R_ * sizeof(int) + 16;
}

template <typename R, bool MODEL, bool FWD>
static cudaError_t launch_one(const GbtrfArgs &a, cudaStream_t st)
{
    const int S = MODEL ? a.ms.cs.S : 1;
    const size_t smem = gbtrf_smem_bytes(sizeof(R), a.g, S);
    auto kern = k_gbtrf<R, MODEL, FWD>;
    cudaError_t e = smem_attr((const void *) kern, smem);
    if (e != cudaSuccess) return e;
    const int grid = a.sys_list ? a.nlist : a.nsys;
    if (grid == 0) return cudaSuccess;
    kern<<<grid, 32, smem, st>>>(a.g, a.nsys, a.src, a.ms,
                                 reinterpret_cast<cplx_t<R> *>(a.fac), a.fac_stride,
                                 a.ipiv, a.info, a.rhs, a.rhs_stride,
                                 reinterpret_cast<cplx_t<R> *>(a.y), a.y_stride,
                                 a.sys_list, a.d_count, a.slot_mode);
    return cudaGetLastError();
}

cudaError_t launch_gbtrf(const GbtrfArgs &a, cudaStream_t st)
{
    if (a.variant == 0 || a.variant == 2) {
        // complex64 assembly of the model reads the float band copies
        if (a.model && a.prec == 'C' && !a.ms.mdf) return cudaErrorInvalidValue;
        int nb = a.nb, nw = a.nw;
        gbtrf_blk_choice(a.prec, a.g, nb, nw, a.model);
        GbtrfArgs b = a;
        if (nw < 0) { b.variant = 2; nw = -nw; }   // the shape table's lookahead entries
        if (gbtrf_blk_supported(a.g, nb, nw)) return launch_gbtrf_blk(b, nb, nw, st);
    }
    const bool fwd = a.rhs != nullptr;
    if (a.prec == 'Z') {
        if (a.model) return fwd ? launch_one<double, true, true>(a, st) : launch_one<double, true, false>(a, st);
        return fwd ? launch_one<double, false, true>(a, st) : launch_one<double, false, false>(a, st);
    } else {
        if (a.model) return fwd ? launch_one<float, true, true>(a, st) : launch_one<float, true, false>(a, st);
        return fwd ? launch_one<float, false, true>(a, st) : launch_one<float, false, false>(a, st);
    }
}

}  // namespace sgb
