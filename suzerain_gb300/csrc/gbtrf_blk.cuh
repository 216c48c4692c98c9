// Blocked batched band LU, one CTA of NW warps per system.  Same results as
// the unblocked k_gbtrf (zgbtf2's multiply-add sequence), far fewer
// instructions per flop and NW warps to hide the sequential latency.
//
// The live window - rows j0 .. j0+KL+NB-1 by columns j0 .. j0+KL+KU+NB-1 -
// sits in shared memory as a circular buffer in both dimensions, rows in
// logical order (interchanges are physical).  Per panel of NB columns:
//   1. warp 0 factors the panel column by column: IZAMAX pivot over the KL+1
//      candidates, interchange of whole panel rows (multiplier columns
//      included, so the panel's L moves with its rows), scale by the
//      reciprocal pivot, rank-1 update of the remaining panel columns; column
//      k of L goes to HBM at step k, before any later interchange, which keeps
//      zgbtf2's unswapped L storage;
//   2. all warps apply the panel's interchanges to the trailing columns in
//      order, then U12 = L11^{-1} A12 by forward substitution, one column per
//      thread;
//   3. all warps update A22 -= L21 U12 as a register-tiled GEMM (threads form
//      an (NT/8) x 8 grid, each holding MAXTR x TC complex accumulators) that
//      subtracts the NB products in panel order;
//   4. U rows out, retired columns zeroed, the next NB rows of A enter.
// Every element receives exactly the multiply-adds of the unblocked
// algorithm in the same order: the rank-1 updates are deferred, not
// reordered.
#pragma once
#include "sgb_internal.h"

#include <climits>

namespace sgb {

// Row pitch of the shared-memory window: odd, so that a column walked by the
// lanes of a warp spreads over the banks.
__host__ __device__ __forceinline__ int blk_pitch(int wc) { return wc | 1; }

// floor(x / S) for 0 <= x < 65536 and 2 <= S <= 65536 by a multiply-high
// with m = ceil(2^32 / S) = (2^32 + e) / S, 0 <= e < S: x m / 2^32 exceeds
// x / S by x e / (S 2^32) < 1 / S, less than the gap from x / S to the next
// integer.  S = 1 (m = 2^32 does not fit) is passed as m = 0.
__device__ __forceinline__ int div_small(int x, unsigned m)
{
    return m ? (int) __umulhi((unsigned) x, m) : x;
}

// Entry (r, col) of the synthetic operator for a row r = p S + e (wall row
// when dir), zero outside the block band and beyond column N-1.  Same
// arithmetic as sgb_block_entry: complex128 from the FP64 bands, complex64
// from their float copies in ms.mdf (the conversions the unblocked kernel
// makes on the fly, done once per plan).
template <typename R>
__device__ __forceinline__ cplx_t<R> model_entry(const ModelSource &ms, const cplx_t<R> *coef,
                                                 unsigned magic, int p, int e, bool dir, int r,
                                                 int col, int N)
{
    const sgb_case &cs = ms.cs;
    const int S = cs.S;
    if (col >= N) return mk<R>(R(0), R(0));
    if (dir) return mk<R>(col == r ? R(1) : R(0), R(0));
    const int q = div_small(col, magic), f = col - q * S;
    const int d = p - q;
    if (d > cs.kl || -d > cs.ku) return mk<R>(R(0), R(0));
    const int k = cs.ku + d + q * cs.ld;
    const int ef = e * S + f;
    const cplx_t<R> a = coef[ef], b = coef[S * S + ef], c = coef[2 * S * S + ef];
    if constexpr (sizeof(R) == 8) {
        const double m = __ldg(cs.M + k), d1 = __ldg(cs.D1 + k), d2 = __ldg(cs.D2 + k);
        sgb_coef cM{a.x, a.y}, cD1{b.x, b.y}, cD2{c.x, c.y};
        double re, im;
        sgb_block_entry(cM, cD1, cD2, m, d1, d2, &re, &im);
        return mk<R>(re, im);
    } else {
        const float4 v = __ldg(ms.mdf + k);
        return mk<R>(fmaf(c.x, v.z, fmaf(b.x, v.y, a.x * v.x)),
                     fmaf(c.y, v.z, fmaf(b.y, v.y, a.y * v.x)));
    }
}

// Warp shuffle of a complex value from lane src.
template <typename R>
__device__ __forceinline__ cplx_t<R> shfl_c(cplx_t<R> z, int src)
{
    return mk<R>(__shfl_sync(0xffffffffu, z.x, src), __shfl_sync(0xffffffffu, z.y, src));
}

// v[q][c] for a warp-uniform slot q.
template <typename R, int RS, int NB>
__device__ __forceinline__ cplx_t<R> pick(const cplx_t<R> (&v)[RS][NB], int q, int c)
{
    cplx_t<R> r = v[0][c];
#pragma unroll
    for (int t = 1; t < RS; ++t) if (q == t) r = v[t][c];
    return r;
}

template <typename R, int RS, int NB>
__device__ __forceinline__ void put_slot(cplx_t<R> (&v)[RS][NB], int q, int c, cplx_t<R> z)
{
#pragma unroll
    for (int t = 0; t < RS; ++t) if (q == t) v[t][c] = z;
}

// Ordering key of a pivot candidate, IZAMAX's: |re|+|im| as an unsigned
// integer (the bit pattern of a non-negative float is monotone in its value)
// plus one, so that 0 marks "not a candidate"; a NaN wins as the first
// candidate and never elsewhere.
__device__ __forceinline__ unsigned long long pivot_key(double m, bool first)
{
    if (m != m) return first ? ~0ull : 0ull;
    return (unsigned long long) __double_as_longlong(m) + 1ull;
}
__device__ __forceinline__ unsigned pivot_key(float m, bool first)
{
    if (m != m) return first ? ~0u : 0u;
    return __float_as_uint(m) + 1u;
}

// Row (window-relative) of the pivot of panel step k: the candidate rows
// k..k+km held as v[q][k] by lane l for row l + 32 q.  Largest key, then the
// smallest row among equal keys (reference IZAMAX takes the first maximum).
template <typename R, int RS, int NB>
__device__ __forceinline__ int warp_argmax_rows(const cplx_t<R> (&v)[RS][NB], int k, int km, int lane)
{
    using K = decltype(pivot_key(R(0), false));
    K key[RS];
    K best = 0;
#pragma unroll
    for (int q = 0; q < RS; ++q) {
        const int i = lane + 32 * q;
        key[q] = (i >= k && i <= k + km) ? pivot_key(cabs1<R>(v[q][k]), i == k) : K(0);
        best = key[q] > best ? key[q] : best;
    }
    K top;
    if constexpr (sizeof(K) == 8) {
        const unsigned hi = __reduce_max_sync(0xffffffffu, (unsigned) (best >> 32));
        const unsigned lo = __reduce_max_sync(0xffffffffu,
                                              (unsigned) (best >> 32) == hi ? (unsigned) best : 0u);
        top = ((K) hi << 32) | lo;
    } else {
        top = __reduce_max_sync(0xffffffffu, best);
    }
    int ip = -1;
#pragma unroll
    for (int q = 0; q < RS; ++q) {
        const unsigned b = __ballot_sync(0xffffffffu, key[q] == top);
        if (ip < 0 && b) ip = 32 * q + __ffs(b) - 1;
    }
    return ip;
}

// Resident CTAs per SM the register budget is cut for: the window of one
// system (KL = KU = 34, NB = 4 or 8) leaves room for about 8 complex64 or 4
// complex128 systems per SM.
template <typename R, int NW>
constexpr int blk_min_blocks() { return sizeof(R) == 8 ? (NW == 4 ? 3 : 4) : (NW == 4 ? 5 : 8); }

template <typename R, int NB, int NW, int MAXTR, bool MODEL, bool FWD>
__global__ void __launch_bounds__(32 * NW, (blk_min_blocks<R, NW>()))
k_gbtrf_cta(FactorGeom g, int nsys, PackedSource src, ModelSource ms,
            cplx_t<R> *__restrict__ fac, long long fac_stride,
            int *__restrict__ ipiv, int *__restrict__ info,
            const double2 *__restrict__ rhs, long long rhs_stride,
            cplx_t<R> *__restrict__ y, long long y_stride,
            const int *__restrict__ sys_list, const int *__restrict__ d_count,
            bool slot_mode, unsigned long long *__restrict__ prof)
{
    using T2 = cplx_t<R>;
    constexpr int NT = 32 * NW;
    constexpr int TC = sizeof(R) == 8 ? 3 : 5;      // GEMM columns per thread per pass
    constexpr int RGN = NT / 8;                       // GEMM row groups
    constexpr bool STAGE = NW > 1;                    // warps 1.. assemble rows during the panel
    constexpr int LNB = NB == 4 ? 2 : NB == 8 ? 3 : 4;
    constexpr int RS = RGN * MAXTR > 48 ? 3 : 2;      // panel rows per lane: WR <= 32 RS
    static_assert((1 << LNB) == NB, "NB must be 4, 8 or 16");
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (d_count && (int) blockIdx.x >= *d_count) return;
    const int s = sys_list ? sys_list[blockIdx.x] : (int) blockIdx.x;
    if (s < 0 || s >= nsys) return;
    const long long fi = slot_mode ? (long long) blockIdx.x : (long long) s;

    const int N = g.N, KL = g.KL, KU = g.KU, UW = g.UW();
    const int WR = KL + NB, WC = KL + KU + NB, P = blk_pitch(WC);
    const int S = MODEL ? ms.cs.S : 1;
    const unsigned magic = (MODEL && S > 1) ? (unsigned) ((0x100000000ull + S - 1) / S) : 0u;

    extern __shared__ __align__(16) unsigned char smem_raw[];
    T2 *win = reinterpret_cast<T2 *>(smem_raw);       // WR x WC, row pitch P
    T2 *rs = win + WR * P;                            // RHS per row slot
    T2 *stg = rs + WR;                                // NB x WC staged rows (STAGE)
    T2 *stgr = stg + (STAGE ? NB * WC : 0);           // NB staged RHS entries (STAGE)
    T2 *coef = stgr + (STAGE ? NB : 0);               // 3 S^2 (model)
    int *pvoff = reinterpret_cast<int *>(coef + (MODEL ? 3 * S * S : 0));   // NB
    int *shv = pvoff + NB;                            // [0] ju, [1] info

    T2 *fu = fac + fi * fac_stride;
    T2 *fl = fu + (long long) N * UW;
    int *pv = ipiv + fi * N;
    const T2 zero = mk<R>(R(0), R(0));

    // Optional per-phase cycle counters (diagnostics), read on thread 0:
    // 0 init, 1 panel (+ staging), 2 interchanges + U12, 3 GEMM + U rows out,
    // 4 unused, 5 retire/enter.
    unsigned long long tph[6] = {0, 0, 0, 0, 0, 0};
    long long tmark = prof ? clock64() : 0;
    auto tick = [&](int ph) {
        if (prof) { const long long t = clock64(); tph[ph] += (unsigned long long) (t - tmark); tmark = t; }
    };

    if (MODEL) {
        const double kx = ms.kx[s], kz = ms.kz[s];
        for (int idx = tid; idx < S * S; idx += NT) {
            sgb_coef cM, cD1, cD2;
            sgb_block_coefs(&ms.cs, idx / S, idx % S, ms.phi, kx, kz, &cM, &cD1, &cD2);
            coef[idx] = mk<R>((R) cM.re, (R) cM.im);
            coef[S * S + idx] = mk<R>((R) cD1.re, (R) cD1.im);
            coef[2 * S * S + idx] = mk<R>((R) cD2.re, (R) cD2.im);
        }
        __syncthreads();
    }
    // Row r < N of A at columns cbase + cc, cc = lane, lane + 32, ... < WC,
    // handed to put(cc, value).
    auto row_to = [&](int r, int cbase, auto put) {
        if constexpr (MODEL) {
            const int p = div_small(r, magic), e = r - p * S;
            const bool dir = ((ms.cs.dirichlet_mask >> e) & 1u) && (p == 0 || p == ms.cs.n - 1);
            for (int cc = lane; cc < WC; cc += 32)
                put(cc, model_entry<R>(ms, coef, magic, p, e, dir, r, cbase + cc, N));
        } else {
            for (int cc = lane; cc < WC; cc += 32) {
                const int col = cbase + cc;
                T2 v = zero;
                if (col < N && col - r <= KU && r - col <= KL) v = from_z<R>(src.entry(s, KU, r, col));
                put(cc, v);
            }
        }
    };

    // Initial window: rows 0..WR-1, columns 0..WC-1 (slots equal indices).
    for (int r = warp; r < WR; r += NW) {
        T2 *dst = win + r * P;
        if (r < N) row_to(r, 0, [&](int cc, T2 v) { dst[cc] = v; });
        else for (int cc = lane; cc < WC; cc += 32) dst[cc] = zero;
    }
    if (FWD)
        for (int r = tid; r < WR; r += NT)
            rs[r] = r < N ? from_z<R>(rhs[s * rhs_stride + r]) : zero;
    if (tid == 0) { shv[0] = 0; shv[1] = 0; }
    __syncthreads();
    tick(0);

    int rb = 0, cb = 0;
    for (int j0 = 0; j0 < N; j0 += NB) {
        const int nbk = imin(NB, N - j0);
        const bool more = j0 + nbk < N;
        auto rsl = [&](int i) { int t = rb + i; return t >= WR ? t - WR : t; };
        auto csl = [&](int c) { int t = cb + c; return t >= WC ? t - WC : t; };

        // ---------------- 1. panel factorization (warp 0) -----------------
        // The panel lives in registers: lane l holds rows l, l+32, .. of the
        // nbk panel columns (row k of step k is row k of slot 0, on lane k).
        if (warp == 0) {
            int ju = shv[0], inf = shv[1];
            T2 v[RS][NB];
            T2 rv[RS];
#pragma unroll
            for (int q = 0; q < RS; ++q) {
                const int i = lane + 32 * q;
                const bool ok = i < WR;
                const int ro = ok ? rsl(i) * P : 0;
#pragma unroll
                for (int c = 0; c < NB; ++c) v[q][c] = (ok && c < nbk) ? win[ro + csl(c)] : zero;
                if (FWD) rv[q] = ok ? rs[rsl(i)] : zero;
            }
#pragma unroll
            for (int k = 0; k < NB; ++k) {
                if (k >= nbk) break;
                const int jj = j0 + k;
                const int km = imin(KL, N - 1 - jj);
                // IZAMAX over rows k..k+km: the largest key, then the
                // smallest row holding it
                const int ip = warp_argmax_rows<R, RS>(v, k, km, lane);
                const int bt = ip - k, lp = ip & 31, qp = ip >> 5;
                const T2 piv = shfl_c<R>(pick<R, RS, NB>(v, qp, k), lp);
                if (lane == 0) pv[jj] = jj + bt + 1;
                if (cnz<R>(piv)) {
                    ju = imax(ju, imin(jj + KU + bt, N - 1));
                    if (bt != 0) {
#pragma unroll
                        for (int c = 0; c < NB; ++c) {
                            if (c < nbk) {
                                const T2 a = shfl_c<R>(v[0][c], k);
                                const T2 b = shfl_c<R>(pick<R, RS, NB>(v, qp, c), lp);
                                if (lane == k) v[0][c] = b;
                                if (lane == lp) put_slot<R, RS, NB>(v, qp, c, a);
                            }
                        }
                        if (FWD) {
                            const T2 a = shfl_c<R>(rv[0], k);
                            T2 bq = rv[0];
#pragma unroll
                            for (int q = 1; q < RS; ++q) if (qp == q) bq = rv[q];
                            const T2 b = shfl_c<R>(bq, lp);
                            if (lane == k) rv[0] = b;
                            if (lane == lp) {
#pragma unroll
                                for (int q = 0; q < RS; ++q) if (qp == q) rv[q] = a;
                            }
                        }
                    }
                    if (lane == 0) pvoff[k] = bt;
                    const T2 rp = crcp<R>(piv);
#pragma unroll
                    for (int q = 0; q < RS; ++q) {
                        const int i = lane + 32 * q;
                        if (i > k && i <= k + km) v[q][k] = cmul(v[q][k], rp);
                        if (i > k && i <= k + KL)
                            fl[(long long) jj * KL + (i - k - 1)] = (i <= k + km) ? v[q][k] : zero;
                    }
                    if (FWD) {
                        const T2 yj = shfl_c<R>(rv[0], k);
                        if (lane == 0) y[s * y_stride + jj] = yj;
#pragma unroll
                        for (int q = 0; q < RS; ++q) {
                            const int i = lane + 32 * q;
                            if (i > k && i <= k + km) rv[q] = cfnma(v[q][k], yj, rv[q]);
                        }
                    }
                    // rank-1 update of the remaining panel columns
#pragma unroll
                    for (int c = k + 1; c < NB; ++c) {
                        if (c < nbk) {
                            const T2 u = shfl_c<R>(v[0][c], k);
                            if (cnz<R>(u)) {
#pragma unroll
                                for (int q = 0; q < RS; ++q) {
                                    const int i = lane + 32 * q;
                                    if (i > k && i <= k + km) v[q][c] = cfnma(v[q][k], u, v[q][c]);
                                }
                            }
                        }
                    }
                } else {
                    if (inf == 0) inf = jj + 1;
                    if (lane == 0) pvoff[k] = 0;
#pragma unroll
                    for (int q = 0; q < RS; ++q) {
                        const int i = lane + 32 * q;
                        if (i > k && i <= k + KL) fl[(long long) jj * KL + (i - k - 1)] = zero;
                    }
                    if (FWD) {
                        const T2 yj = shfl_c<R>(rv[0], k);
                        if (lane == 0) y[s * y_stride + jj] = yj;
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < RS; ++q) {
                const int i = lane + 32 * q;
                if (i < WR) {
                    const int ro = rsl(i) * P;
#pragma unroll
                    for (int c = 0; c < NB; ++c)
                        if (c < nbk) win[ro + csl(c)] = v[q][c];
                    if (FWD) rs[rsl(i)] = rv[q];
                }
            }
            if (lane == 0) { shv[0] = ju; shv[1] = inf; }
        } else if constexpr (STAGE) {
            // the next nbk rows of A, at the next window's columns
            if (more) {
                for (int k = warp - 1; k < nbk; k += NW - 1) {
                    const int r = j0 + WR + k;
                    T2 *dst = stg + k * WC;
                    if (r < N) row_to(r, j0 + nbk, [&](int cc, T2 v) { dst[cc] = v; });
                    else for (int cc = lane; cc < WC; cc += 32) dst[cc] = zero;
                }
                if (FWD)
                    for (int k = tid - 32; k < nbk; k += NT - 32) {
                        const int r = j0 + WR + k;
                        stgr[k] = r < N ? from_z<R>(rhs[s * rhs_stride + r]) : zero;
                    }
            }
        }
        __syncthreads();
        tick(1);
        const int ju = shv[0];
        const int ce = ju - j0;              // last trailing column (relative), < WC
        const int ntr = ce - nbk + 1;

        // ---------------- 2. interchanges and U12, one column per thread ---
        for (int c = nbk + tid; c <= ce; c += NT) {
            const int cc = csl(c);
            for (int k = 0; k < nbk; ++k) {
                const int bt = pvoff[k];
                if (bt) {
                    T2 &a = win[rsl(k) * P + cc], &b = win[rsl(k + bt) * P + cc];
                    const T2 t = a; a = b; b = t;
                }
            }
            T2 u[NB];
#pragma unroll
            for (int k = 0; k < NB; ++k) {
                if (k < nbk) {
                    const int ro = rsl(k) * P;
                    T2 v = win[ro + cc];
#pragma unroll
                    for (int m = 0; m < NB; ++m)
                        if (m < k) v = cfnma(win[ro + csl(m)], u[m], v);
                    u[k] = v;
                    win[ro + cc] = v;
                }
            }
        }
        __syncthreads();
        tick(2);

        // ---------------- 3. A22 -= L21 U12 (register-tiled GEMM) -----------
        // and U rows out (rows < nbk, which the GEMM does not touch)
        if (ntr > 0) {
            const int rg = tid >> 3, cg = tid & 7;
            const int nrow = imin(KL, N - j0 - nbk);     // rows nbk .. nbk+nrow-1
            int roff[MAXTR];
#pragma unroll
            for (int t = 0; t < MAXTR; ++t) {
                const int i = rg + RGN * t;
                roff[t] = (i < nrow) ? rsl(nbk + i) * P : -1;
            }
            for (int c0 = 0; c0 < ntr; c0 += 8 * TC) {
                int coff[TC];
#pragma unroll
                for (int u = 0; u < TC; ++u) {
                    const int c = c0 + cg + 8 * u;
                    coff[u] = (c < ntr) ? csl(nbk + c) : -1;
                }
                T2 acc[MAXTR][TC];
#pragma unroll
                for (int t = 0; t < MAXTR; ++t)
#pragma unroll
                    for (int u = 0; u < TC; ++u)
                        acc[t][u] = (roff[t] >= 0 && coff[u] >= 0) ? win[roff[t] + coff[u]] : zero;
#pragma unroll
                for (int m = 0; m < NB; ++m) {
                    if (m < nbk) {
                        const int cm = csl(m), rm = rsl(m) * P;
                        T2 l[MAXTR], uu[TC];
#pragma unroll
                        for (int t = 0; t < MAXTR; ++t) l[t] = roff[t] >= 0 ? win[roff[t] + cm] : zero;
#pragma unroll
                        for (int u = 0; u < TC; ++u) uu[u] = coff[u] >= 0 ? win[rm + coff[u]] : zero;
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
                    for (int u = 0; u < TC; ++u)
                        if (roff[t] >= 0 && coff[u] >= 0) win[roff[t] + coff[u]] = acc[t][u];
            }
        }
        for (int k = warp; k < nbk; k += NW) {
            const int jj = j0 + k, ro = rsl(k) * P;
            for (int t = lane; t < UW; t += 32)
                fu[(long long) jj * UW + t] = win[ro + csl(k + t)];
        }
        __syncthreads();
        tick(3);

        // ---------------- 5. retire rows/columns, enter new ones ------------
        if (more) {
            // retired column slots (columns j0+WC.. next) of the rows that stay
            for (int idx = tid; idx < WR * NB; idx += NT) {
                const int i = idx >> LNB, c = idx & (NB - 1);
                if (i >= nbk && c < nbk) win[rsl(i) * P + csl(c)] = zero;
            }
            // retired row slots take rows j0+WR.. at columns j0+nbk ..
            for (int k = warp; k < nbk; k += NW) {
                T2 *dst = win + rsl(k) * P;
                auto put = [&](int cc, T2 v) {
                    int cs = cb + nbk + cc;          // < 3 WC: wrap at most twice
                    if (cs >= WC) cs -= WC;
                    if (cs >= WC) cs -= WC;
                    dst[cs] = v;
                };
                if constexpr (STAGE) {
                    for (int cc = lane; cc < WC; cc += 32) put(cc, stg[k * WC + cc]);
                } else {
                    const int r = j0 + WR + k;
                    if (r < N) row_to(r, j0 + nbk, put);
                    else for (int cc = lane; cc < WC; cc += 32) put(cc, zero);
                }
            }
            if (FWD)
                for (int k = tid; k < nbk; k += NT) {
                    if constexpr (STAGE) rs[rsl(k)] = stgr[k];
                    else {
                        const int r = j0 + WR + k;
                        rs[rsl(k)] = r < N ? from_z<R>(rhs[s * rhs_stride + r]) : zero;
                    }
                }
            __syncthreads();
        }
        tick(5);
        rb += NB; if (rb >= WR) rb -= WR;
        cb += NB; if (cb >= WC) cb -= WC;
    }
    if (tid == 0) info[fi] = shv[1];
    if (prof && tid == 0)
        for (int ph = 0; ph < 6; ++ph) atomicAdd(prof + ph, tph[ph]);
}

template <typename R, int NB, int NW, int MAXTR, bool MODEL, bool FWD>
cudaError_t launch_cta_one(const GbtrfArgs &a, cudaStream_t st)
{
    const int S = MODEL ? a.ms.cs.S : 1;
    const size_t smem = gbtrf_blk_smem_bytes(sizeof(R), a.g, S, NB, NW);
    auto kern = k_gbtrf_cta<R, NB, NW, MAXTR, MODEL, FWD>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
    if (e != cudaSuccess) return e;
    const int grid = a.sys_list ? a.nlist : a.nsys;
    if (grid == 0) return cudaSuccess;
    kern<<<grid, 32 * NW, smem, st>>>(a.g, a.nsys, a.src, a.ms,
                                      reinterpret_cast<cplx_t<R> *>(a.fac), a.fac_stride,
                                      a.ipiv, a.info, a.rhs, a.rhs_stride,
                                      reinterpret_cast<cplx_t<R> *>(a.y), a.y_stride,
                                      a.sys_list, a.d_count, a.slot_mode, a.prof);
    return cudaGetLastError();
}

template <typename R, int NB, int NW, int MAXTR>
cudaError_t launch_cta_r(const GbtrfArgs &a, cudaStream_t st)
{
    const bool fwd = a.rhs != nullptr;
    if (a.model) return fwd ? launch_cta_one<R, NB, NW, MAXTR, true, true>(a, st)
                            : launch_cta_one<R, NB, NW, MAXTR, true, false>(a, st);
    return fwd ? launch_cta_one<R, NB, NW, MAXTR, false, true>(a, st)
               : launch_cta_one<R, NB, NW, MAXTR, false, false>(a, st);
}

// Rows per GEMM thread for NW warps: KL <= (4 NW) * MAXTR.
template <typename R, int NB>
cudaError_t launch_cta_nw(const GbtrfArgs &a, int nw, cudaStream_t st)
{
    const int KL = a.g.KL;
    if (nw == 1) return KL <= 36 ? launch_cta_r<R, NB, 1, 9>(a, st) : launch_cta_r<R, NB, 1, 13>(a, st);
    if (nw == 2) return KL <= 40 ? launch_cta_r<R, NB, 2, 5>(a, st) : launch_cta_r<R, NB, 2, 7>(a, st);
    return KL <= 48 ? launch_cta_r<R, NB, 4, 3>(a, st) : launch_cta_r<R, NB, 4, 4>(a, st);
}

// One translation unit per (precision, NB) instantiates the kernels.
#define SGB_BLK_INSTANTIATE(R, NB, NAME)                                          \
    cudaError_t NAME(const GbtrfArgs &a, int nw, cudaStream_t st)                 \
    {                                                                             \
        return launch_cta_nw<R, NB>(a, nw, st);                                   \
    }

cudaError_t launch_blk_z4(const GbtrfArgs &, int, cudaStream_t);
cudaError_t launch_blk_z8(const GbtrfArgs &, int, cudaStream_t);
cudaError_t launch_blk_z16(const GbtrfArgs &, int, cudaStream_t);
cudaError_t launch_blk_c4(const GbtrfArgs &, int, cudaStream_t);
cudaError_t launch_blk_c8(const GbtrfArgs &, int, cudaStream_t);
cudaError_t launch_blk_c16(const GbtrfArgs &, int, cudaStream_t);

}  // namespace sgb
