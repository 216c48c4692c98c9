// Blocked batched band LU: same results as k_gbtrf (zgbtf2 order), far
// fewer instructions per flop.
//
// One warp factors one system in panels of NB columns.  The live window -
// rows j0 .. j0+KL+NB-1 by columns j0 .. j0+KL+KU+NB-1 - sits in shared
// memory as a circular buffer in both dimensions, rows in logical order
// (interchanges are physical, as in LAPACK).  Per panel:
//   1. factor the NB panel columns column by column: IZAMAX pivot over the
//      KL+1 candidates, interchange of whole panel rows, scale by the
//      reciprocal pivot, rank-1 update of the remaining panel columns;
//      column k of L goes to HBM at step k (zgbtf2's unswapped storage);
//   2. apply the panel's interchanges to the trailing columns, in order;
//   3. U12 = L11^{-1} A12 by forward substitution, column per lane;
//   4. A22 -= L21 U12 as a register-tiled GEMM: lanes form a 4 x 8 grid, each
//      holds MAXTR x TC complex accumulators and subtracts the NB products in
//      panel order.
// Every element therefore receives exactly the sequence of multiply-adds of
// the unblocked algorithm (zgbtf2), only batched: the rank-1 updates are
// deferred, not reordered.  Outputs are the row-panel factor of gbtrf.cuh.
#include "sgb_internal.h"

#include <climits>

namespace sgb {

template <typename R>
__device__ __forceinline__ cplx_t<R> model_entry_blk(const sgb_case &cs, const cplx_t<R> *coef,
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

template <typename R, int NB, int MAXTR, bool MODEL, bool FWD>
__global__ void __launch_bounds__(32)
k_gbtrf_blk(FactorGeom g, int nsys, PackedSource src, ModelSource ms,
            cplx_t<R> *__restrict__ fac, long long fac_stride,
            int *__restrict__ ipiv, int *__restrict__ info,
            const double2 *__restrict__ rhs, long long rhs_stride,
            cplx_t<R> *__restrict__ y, long long y_stride,
            const int *__restrict__ sys_list, const int *__restrict__ d_count,
            bool slot_mode, unsigned long long *__restrict__ prof)
{
    using T2 = cplx_t<R>;
    constexpr int TC = sizeof(R) == 8 ? 3 : 5;   // GEMM columns per lane per pass
    const int lane = threadIdx.x;
    if (d_count && (int) blockIdx.x >= *d_count) return;
    const int s = sys_list ? sys_list[blockIdx.x] : (int) blockIdx.x;
    if (s < 0 || s >= nsys) return;
    const long long fi = slot_mode ? (long long) blockIdx.x : (long long) s;

    const int N = g.N, KL = g.KL, KU = g.KU, UW = g.UW(), KV = UW - 1;
    const int WR = KL + NB, WC = KL + KU + NB;
    const int S = MODEL ? ms.cs.S : 1;

    extern __shared__ __align__(16) unsigned char smem_raw[];
    T2 *win = reinterpret_cast<T2 *>(smem_raw);       // WR x WC, row-major
    T2 *rs = win + WR * WC;                           // RHS per row slot
    T2 *coef = rs + WR;                               // 3 S^2 (model)
    int *pvoff = reinterpret_cast<int *>(coef + (MODEL ? 3 * S * S : 0));   // NB

    T2 *fu = fac + fi * fac_stride;
    T2 *fl = fu + (long long) N * UW;
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
        if constexpr (MODEL) return model_entry_blk<R>(ms.cs, coef, i, j);
        else return from_z<R>(src.entry(s, KU, i, j));
    };
    const T2 zero = mk<R>(R(0), R(0));
    // Optional per-phase cycle counters (diagnostics): 0 init, 1 panel,
    // 2 interchanges + U12, 3 GEMM, 4 U rows out, 5 retire/load.
    unsigned long long tph[6] = {0, 0, 0, 0, 0, 0};
    long long tmark = prof ? clock64() : 0;
    auto tick = [&](int ph) {
        if (prof) { const long long t = clock64(); tph[ph] += (unsigned long long) (t - tmark); tmark = t; }
    };

    // Initial window: rows 0..WR-1, columns 0..WC-1 (slots equal indices).
    for (int idx = lane; idx < WR * WC; idx += 32) {
        const int r = idx / WC, c = idx - r * WC;
        T2 v = zero;
        if (r < N && c < N && c - r <= KU && r - c <= KL) v = A(r, c);
        win[idx] = v;
    }
    if (FWD)
        for (int r = lane; r < WR; r += 32)
            rs[r] = r < N ? from_z<R>(rhs[s * rhs_stride + r]) : zero;
    __syncwarp();
    tick(0);

    int ju = 0, inf = 0;
    for (int j0 = 0; j0 < N; j0 += NB) {
        const int rb = j0 % WR, cb = j0 % WC;
        const int nbk = imin(NB, N - j0);
        // window slot of row j0+i (0 <= i < WR) and column j0+c (0 <= c < WC)
        auto rsl = [&](int i) { int t = rb + i; return t >= WR ? t - WR : t; };
        auto csl = [&](int c) { int t = cb + c; return t >= WC ? t - WC : t; };
        auto W = [&](int i, int c) -> T2 & { return win[rsl(i) * WC + csl(c)]; };

        // ---------------- 1. panel factorization --------------------------
        for (int k = 0; k < nbk; ++k) {
            const int jj = j0 + k;
            const int km = imin(KL, N - 1 - jj);
            R best = R(-1);
            int bt = INT_MAX;
            for (int t = lane; t <= km; t += 32) {
                R m = cabs1<R>(W(k + t, k));
                if (m != m) m = (t == 0) ? R(INFINITY) : R(-1);
                if (m > best || (m == best && t < bt)) { best = m; bt = t; }
            }
#pragma unroll
            for (int off = 16; off; off >>= 1) {
                const R ob = __shfl_xor_sync(0xffffffffu, best, off);
                const int ot = __shfl_xor_sync(0xffffffffu, bt, off);
                if (ob > best || (ob == best && ot < bt)) { best = ob; bt = ot; }
            }
            const T2 piv = W(k + bt, k);
            if (lane == 0) pv[jj] = jj + bt + 1;
            if (cnz<R>(piv)) {
                ju = imax(ju, imin(jj + KU + bt, N - 1));
                if (bt != 0) {
                    // Interchange whole panel rows, earlier multiplier columns
                    // included, so the panel's L moves with its rows and the
                    // trailing update can apply every interchange first.  The
                    // stored factor keeps zgbtf2's unswapped L: column k is
                    // written to HBM below, before any later interchange.
                    for (int c = lane; c < nbk; c += 32) {
                        T2 &a = W(k, c), &b = W(k + bt, c);
                        const T2 t = a; a = b; b = t;
                    }
                    if (FWD && lane == 0) {
                        T2 &a = rs[rsl(k)], &b = rs[rsl(k + bt)];
                        const T2 t = a; a = b; b = t;
                    }
                }
                if (lane == 0) pvoff[k] = bt;
                __syncwarp();
                const T2 rp = crcp<R>(piv);
                for (int t = 1 + lane; t <= km; t += 32) W(k + t, k) = cmul(W(k + t, k), rp);
                __syncwarp();
                for (int t = lane; t < KL; t += 32)
                    fl[(long long) jj * KL + t] = (t < km) ? W(k + 1 + t, k) : zero;
                if (FWD) {
                    const T2 yj = rs[rsl(k)];
                    if (lane == 0) y[s * y_stride + jj] = yj;
                    for (int t = 1 + lane; t <= km; t += 32)
                        rs[rsl(k + t)] = cfnma(W(k + t, k), yj, rs[rsl(k + t)]);
                }
                // rank-1 update of the remaining panel columns
                const int pc = nbk - 1 - k;
                for (int e = lane; e < km * pc; e += 32) {
                    const int t = 1 + e / pc, c = k + 1 + e % pc;
                    const T2 u = W(k, c);
                    if (cnz<R>(u)) W(k + t, c) = cfnma(W(k + t, k), u, W(k + t, c));
                }
            } else {
                if (inf == 0) inf = jj + 1;
                if (lane == 0) pvoff[k] = 0;
                for (int t = lane; t < KL; t += 32) fl[(long long) jj * KL + t] = zero;
                if (FWD && lane == 0) y[s * y_stride + jj] = rs[rsl(k)];
            }
            __syncwarp();
        }

        tick(1);
        // trailing columns j0+nbk .. ju  (relative nbk .. ju-j0)
        const int ce = ju - j0;              // last trailing column (relative), < WC
        const int ntr = ce - nbk + 1;

        // ---------------- 2./3. interchanges and U12 ----------------------
        for (int c = nbk + lane; c <= ce; c += 32) {
            for (int k = 0; k < nbk; ++k) {
                const int bt = pvoff[k];
                if (bt) { T2 &a = W(k, c), &b = W(k + bt, c); const T2 t = a; a = b; b = t; }
            }
            T2 u[NB];
#pragma unroll
            for (int k = 0; k < NB; ++k) {
                if (k < nbk) {
                    T2 v = W(k, c);
#pragma unroll
                    for (int m = 0; m < NB; ++m)
                        if (m < k) v = cfnma(W(k, m), u[m], v);
                    u[k] = v;
                    W(k, c) = v;
                }
            }
        }
        __syncwarp();
        tick(2);

        // ---------------- 4. A22 -= L21 U12 (register-tiled GEMM) -----------
        if (ntr > 0) {
            const int rg = lane >> 3, cg = lane & 7;
            const int nrow = imin(KL, N - j0 - nbk);     // rows nbk .. nbk+nrow-1
            for (int c0 = 0; c0 < ntr; c0 += 8 * TC) {
                T2 acc[MAXTR][TC];
#pragma unroll
                for (int t = 0; t < MAXTR; ++t)
#pragma unroll
                    for (int u = 0; u < TC; ++u) {
                        const int i = rg + 4 * t, c = c0 + cg + 8 * u;
                        acc[t][u] = (i < nrow && c < ntr) ? W(nbk + i, nbk + c) : zero;
                    }
#pragma unroll
                for (int m = 0; m < NB; ++m) {
                    if (m < nbk) {
                        T2 l[MAXTR], uu[TC];
#pragma unroll
                        for (int t = 0; t < MAXTR; ++t) {
                            const int i = rg + 4 * t;
                            l[t] = (i < nrow) ? W(nbk + i, m) : zero;
                        }
#pragma unroll
                        for (int u = 0; u < TC; ++u) {
                            const int c = c0 + cg + 8 * u;
                            uu[u] = (c < ntr) ? W(m, nbk + c) : zero;
                        }
#pragma unroll
                        for (int t = 0; t < MAXTR; ++t)
#pragma unroll
                            for (int u = 0; u < TC; ++u)
                                acc[t][u] = cfnma(l[t], uu[u], acc[t][u]);
                    }
                }
#pragma unroll
                for (int t = 0; t < MAXTR; ++t)
#pragma unroll
                    for (int u = 0; u < TC; ++u) {
                        const int i = rg + 4 * t, c = c0 + cg + 8 * u;
                        if (i < nrow && c < ntr) W(nbk + i, nbk + c) = acc[t][u];
                    }
            }
        }
        __syncwarp();
        tick(3);

        // ---------------- 5. U rows out -------------------------------------
        for (int k = 0; k < nbk; ++k) {
            const int jj = j0 + k;
            for (int t = lane; t < UW; t += 32)
                fu[(long long) jj * UW + t] = W(k, k + t);
        }
        __syncwarp();
        tick(4);

        // ---------------- 6. retire rows/columns, enter new ones ------------
        if (j0 + nbk < N) {
            // retiring column slots j0..j0+nbk-1 become j0+WC.. : zero them
            for (int idx = lane; idx < WR * nbk; idx += 32) {
                const int i = idx / nbk, c = idx - i * nbk;
                win[i * WC + csl(c)] = zero;
            }
            __syncwarp();
            // retiring row slots j0..j0+nbk-1 become rows j0+WR..; the next
            // window's columns are j0+nbk .. j0+nbk+WC-1
            for (int idx = lane; idx < nbk * WC; idx += 32) {
                const int k = idx / WC, cc = idx - k * WC;     // cc relative to j0+nbk
                const int r = j0 + WR + k, col = j0 + nbk + cc;
                T2 v = zero;
                if (r < N && col < N && col - r <= KU && r - col <= KL) v = A(r, col);
                int cs = cb + nbk + cc;              // < 3 WC: wrap at most twice
                if (cs >= WC) cs -= WC;
                if (cs >= WC) cs -= WC;
                win[rsl(k) * WC + cs] = v;
            }
            if (FWD)
                for (int k = lane; k < nbk; k += 32) {
                    const int r = j0 + WR + k;
                    rs[rsl(k)] = r < N ? from_z<R>(rhs[s * rhs_stride + r]) : zero;
                }
            __syncwarp();
        }
        tick(5);
    }
    if (lane == 0) info[fi] = inf;
    if (prof && lane == 0)
        for (int ph = 0; ph < 6; ++ph) atomicAdd(prof + ph, tph[ph]);
}

size_t gbtrf_blk_smem_bytes(int prec_bytes, const FactorGeom &g, int S, int nb)
{
    const size_t el = 2 * (size_t) prec_bytes;
    const int WR = g.KL + nb, WC = g.KL + g.KU + nb;
    return (size_t) WR * WC * el + (size_t) WR * el + 3 * (size_t) S * S * el
         + (size_t) nb * sizeof(int) + 16;
}

template <typename R, int NB, int MAXTR, bool MODEL, bool FWD>
static cudaError_t launch_blk_one(const GbtrfArgs &a, cudaStream_t st)
{
    const int S = MODEL ? a.ms.cs.S : 1;
    const size_t smem = gbtrf_blk_smem_bytes(sizeof(R), a.g, S, NB);
    auto kern = k_gbtrf_blk<R, NB, MAXTR, MODEL, FWD>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
    if (e != cudaSuccess) return e;
    const int grid = a.sys_list ? a.nlist : a.nsys;
    if (grid == 0) return cudaSuccess;
    kern<<<grid, 32, smem, st>>>(a.g, a.nsys, a.src, a.ms,
                                 reinterpret_cast<cplx_t<R> *>(a.fac), a.fac_stride,
                                 a.ipiv, a.info, a.rhs, a.rhs_stride,
                                 reinterpret_cast<cplx_t<R> *>(a.y), a.y_stride,
                                 a.sys_list, a.d_count, a.slot_mode, a.prof);
    return cudaGetLastError();
}

template <typename R, int NB, int MAXTR>
static cudaError_t launch_blk_r(const GbtrfArgs &a, cudaStream_t st)
{
    const bool fwd = a.rhs != nullptr;
    if (a.model) return fwd ? launch_blk_one<R, NB, MAXTR, true, true>(a, st)
                            : launch_blk_one<R, NB, MAXTR, true, false>(a, st);
    return fwd ? launch_blk_one<R, NB, MAXTR, false, true>(a, st)
               : launch_blk_one<R, NB, MAXTR, false, false>(a, st);
}

// KL <= 4*MAXTR rows per GEMM; NB in {4, 8, 16}.
bool gbtrf_blk_supported(const FactorGeom &g, int nb)
{
    return (nb == 4 || nb == 8 || nb == 16) && g.KL <= 52;
}

cudaError_t launch_gbtrf_blk(const GbtrfArgs &a, int nb, cudaStream_t st)
{
    const bool wide = a.g.KL > 36;
    if (a.prec == 'Z') {
        if (nb == 4) return wide ? launch_blk_r<double, 4, 13>(a, st) : launch_blk_r<double, 4, 9>(a, st);
        if (nb == 16) return wide ? launch_blk_r<double, 16, 13>(a, st) : launch_blk_r<double, 16, 9>(a, st);
        return wide ? launch_blk_r<double, 8, 13>(a, st) : launch_blk_r<double, 8, 9>(a, st);
    }
    if (nb == 4) return wide ? launch_blk_r<float, 4, 13>(a, st) : launch_blk_r<float, 4, 9>(a, st);
    if (nb == 16) return wide ? launch_blk_r<float, 16, 13>(a, st) : launch_blk_r<float, 16, 9>(a, st);
    return wide ? launch_blk_r<float, 8, 13>(a, st) : launch_blk_r<float, 8, 9>(a, st);
}

}  // namespace sgb
