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
// lanes of a warp spreads over the banks, and above WC, so that column WC of
// every row is a sink for the trailing update (below).
__host__ __device__ __forceinline__ int blk_pitch(int wc) { return (wc + 1) | 1; }

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


// Complex64 shared-memory accesses at explicit 32-bit shared-window byte
// addresses (one integer add per access in the trailing update).
__device__ __forceinline__ float2 lds_c(unsigned a, float2)
{ float2 v; asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(a)); return v; }
__device__ __forceinline__ void sts_c(unsigned a, float2 v)
{ asm volatile("st.shared.v2.f32 [%0], {%1, %2};" :: "r"(a), "f"(v.x), "f"(v.y) : "memory"); }

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

// Panel factorization of columns j0 .. j0+nbk-1 by one warp (zgbtf2 steps
// with the deferred trailing update).  The panel lives in registers: lane l
// holds panel rows l, l+32, .. (rows j0 + i at window slot rsl(i) for
// i < nrows, columns j0 + c at slot csl(c)); row k of step k is row k of slot
// 0, on lane k.  Writes the pivots, the L columns (zgbtf2's unswapped
// storage, column k at step k), pvoff (the interchange offsets, for the
// trailing columns), shv[0] = ju and shv[1] = info, and with FWD the forward
// elimination of the row-slot RHS rs into y.
template <typename R, int NB, int RS, bool FWD>
__device__ __forceinline__ void panel_factor(cplx_t<R> *__restrict__ win, int P, int WR, int WC,
                                             int rb, int cb, int nrows, cplx_t<R> *__restrict__ rs,
                                             int *__restrict__ pvoff, int *__restrict__ shv,
                                             int j0, int nbk, int N, int KL, int KU,
                                             cplx_t<R> *__restrict__ fl, int *__restrict__ pv,
                                             cplx_t<R> *__restrict__ ys, int lane,
                                             unsigned long long *__restrict__ clk = nullptr)
{
    using T2 = cplx_t<R>;
    const T2 zero = mk<R>(R(0), R(0));
    // optional sub-phase cycle counters (diagnostics, lane 0 with clk set,
    // in shared memory): pivot search, reciprocal + scale + L store, rank-1
    // update of the panel columns
    if (clk && lane == 0) clk[11] = clock64();
    auto stick = [&](int ph) {
        if (clk && lane == 0) {
            const unsigned long long t = clock64();
            clk[6 + ph] += t - clk[11];
            clk[11] = t;
        }
    };
    auto rsl = [&](int i) { int t = rb + i; return t >= WR ? t - WR : t; };
    auto csl = [&](int c) { int t = cb + c; return t >= WC ? t - WC : t; };
    int ju = shv[0], inf = shv[1];
    T2 v[RS][NB];
    T2 rv[RS];
#pragma unroll
    for (int q = 0; q < RS; ++q) {
        const int i = lane + 32 * q;
        const bool ok = i < nrows;
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
        stick(2);
        const int ip = warp_argmax_rows<R, RS>(v, k, km, lane);
        const int bt = ip - k, lp = ip & 31, qp = ip >> 5;
        const T2 piv = shfl_c<R>(pick<R, RS, NB>(v, qp, k), lp);
        stick(0);
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
                if (lane == 0) ys[jj] = yj;
#pragma unroll
                for (int q = 0; q < RS; ++q) {
                    const int i = lane + 32 * q;
                    if (i > k && i <= k + km) rv[q] = cfnma(v[q][k], yj, rv[q]);
                }
            }
            stick(1);
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
                if (lane == 0) ys[jj] = yj;
            }
        }
    }
#pragma unroll
    for (int q = 0; q < RS; ++q) {
        const int i = lane + 32 * q;
        if (i < nrows) {
            const int ro = rsl(i) * P;
#pragma unroll
            for (int c = 0; c < NB; ++c)
                if (c < nbk) win[ro + csl(c)] = v[q][c];
            if (FWD) rs[rsl(i)] = rv[q];
        }
    }
    if (lane == 0) { shv[0] = ju; shv[1] = inf; }
}

// Rows r0 .. r0+nr-1 of A (rows outside 0..N-1 read as zero) at columns
// cbase + cc, 0 <= cc < WC (columns outside 0..N-1 zero), handed to
// put(k, cc, value) for every k < nr, cc < WC.  One warp, lanes over cc.  The
// band reads of a group of GR rows x GC column passes of 32 are all issued
// before any value is formed, so the latency of the source (the float band
// copies in L2 for the model, HBM for a packed band) is paid once per group
// instead of once per entry; smaller groups hold fewer registers.
template <typename R, bool MODEL> struct BandRaw { using type = double2; };
template <> struct BandRaw<float, true> { using type = float4; };
template <> struct BandRaw<double, true> { using type = double3; };

template <typename R, bool MODEL, int GR = 2, int GC = 3, typename Put>
__device__ __forceinline__ void assemble_rows(const PackedSource &src, const ModelSource &ms,
                                              const cplx_t<R> *coef, unsigned magic, int s, int N,
                                              int KL, int KU, int WC, int r0, int nr, int cbase,
                                              int lane, Put &&put)
{
    using T2 = cplx_t<R>;
    using Raw = typename BandRaw<R, MODEL>::type;
    const int S = MODEL ? ms.cs.S : 1, SS = S * S;
    for (int k0 = 0; k0 < nr; k0 += GR) {
        for (int c0 = 0; c0 < WC; c0 += 32 * GC) {
            Raw raw[GR][GC];
            int tag[GR][GC];       // -1 zero, -2 one (wall diagonal), else coefficient index
            // per column: in range, block column q and equation f (model)
            int cq[GC], cf[GC];
            bool cok[GC];
#pragma unroll
            for (int ii = 0; ii < GC; ++ii) {
                const int cc = c0 + lane + 32 * ii, col = cbase + cc;
                cok[ii] = cc < WC && col >= 0 && col < N;
                cq[ii] = MODEL && cok[ii] ? div_small(col, magic) : 0;
                cf[ii] = col - cq[ii] * S;
            }
#pragma unroll
            for (int kk = 0; kk < GR; ++kk) {
                const int k = k0 + kk, r = r0 + k;
                const bool rv = k < nr && r >= 0 && r < N;
                int p = 0, e = 0;
                bool dir = false;
                if constexpr (MODEL) {
                    if (rv) {
                        p = div_small(r, magic);
                        e = r - p * S;
                        dir = ((ms.cs.dirichlet_mask >> e) & 1u) && (p == 0 || p == ms.cs.n - 1);
                    }
                }
#pragma unroll
                for (int ii = 0; ii < GC; ++ii) {
                    const int col = cbase + c0 + lane + 32 * ii;
                    int t = -1;
                    if (rv && cok[ii]) {
                        if constexpr (MODEL) {
                            if (dir) {
                                t = col == r ? -2 : -1;
                            } else {
                                const int q = cq[ii], d = p - q;
                                if (d <= ms.cs.kl && -d <= ms.cs.ku) {
                                    const int bk = ms.cs.ku + d + q * ms.cs.ld;
                                    t = e * S + cf[ii];
                                    if constexpr (sizeof(R) == 8)
                                        raw[kk][ii] = make_double3(__ldg(ms.cs.M + bk), __ldg(ms.cs.D1 + bk),
                                                                   __ldg(ms.cs.D2 + bk));
                                    else
                                        raw[kk][ii] = __ldg(ms.mdf + bk);
                                }
                            }
                        } else {
                            if (col - r <= KU && r - col <= KL) {
                                t = 0;
                                raw[kk][ii] = src.entry(s, KU, r, col);
                            }
                        }
                    }
                    tag[kk][ii] = t;
                }
            }
#pragma unroll
            for (int kk = 0; kk < GR; ++kk) {
#pragma unroll
                for (int ii = 0; ii < GC; ++ii) {
                    const int k = k0 + kk, cc = c0 + lane + 32 * ii;
                    if (k < nr && cc < WC) {
                        const int t = tag[kk][ii];
                        T2 v = mk<R>(t == -2 ? R(1) : R(0), R(0));
                        if (t >= 0) {
                            if constexpr (MODEL) {
                                const T2 a = coef[t], b = coef[SS + t], c = coef[2 * SS + t];
                                if constexpr (sizeof(R) == 8) {
                                    sgb_coef cM{a.x, a.y}, cD1{b.x, b.y}, cD2{c.x, c.y};
                                    double re, im;
                                    sgb_block_entry(cM, cD1, cD2, raw[kk][ii].x, raw[kk][ii].y,
                                                    raw[kk][ii].z, &re, &im);
                                    v = mk<R>(re, im);
                                } else {
                                    const float4 w = raw[kk][ii];
                                    v = mk<R>(fmaf(c.x, w.z, fmaf(b.x, w.y, a.x * w.x)),
                                              fmaf(c.y, w.z, fmaf(b.y, w.y, a.y * w.x)));
                                }
                            } else {
                                v = from_z<R>(raw[kk][ii]);
                            }
                        }
                        put(k, cc, v);
                    }
                }
            }
        }
    }
}

// Resident CTAs per SM the register budget is cut for: the window of one
// system (KL = KU = 34, NB = 4 or 8) leaves room for about 8 complex64 or 4
// complex128 systems per SM.
template <typename R, int NW>
constexpr int blk_min_blocks()
{
    // complex64 with three warps: registers are granted per scheduler in
    // whole warps, so 80 registers a thread keep 8 CTAs (24 warps) resident
    // and 81..96 only 6; asking for 7 gives 80 (a few spills), measured
    // faster than 6 CTAs without spills
    return sizeof(R) == 8 ? (NW == 4 ? 3 : 4) : (NW == 4 ? 4 : NW == 3 ? 7 : 8);
}

// The factor of one system s (factor, pivots and info at index fi) by the
// CTA: the body of the phased kernel below and of the ragged kernel.
// CKL, CKU > 0: the bandwidths fixed at compile time (they must equal g.KL,
// g.KU), so that the window's extents, pitch and wrap-arounds fold into
// immediates; NFULL: N is a multiple of NB, every panel is full.  Both only
// change the instruction stream, not the arithmetic: the factors are
// bit-identical to the generic instance's.  PROF: the per-phase cycle
// counters (diagnostics) are compiled in and kept when prof is set; without
// it the counting code and its branches are absent.  MST: how the model
// source is passed, by value (the phased kernel: a kernel parameter) or as
// a reference to the ragged kernel's shared-memory descriptor (fewer live
// registers).
template <typename R, int NB, int NW, int MAXTR, bool MODEL, bool FWD, typename MST = ModelSource,
          int CKL = 0, int CKU = 0, bool NFULL = false, bool PROF = false>
__device__ __forceinline__ void
gbtrf_cta_system(const FactorGeom g, int s, long long fi, const PackedSource src,
                 MST ms, cplx_t<R> *__restrict__ fac, long long fac_stride,
                 int *__restrict__ ipiv, int *__restrict__ info,
                 const double2 *__restrict__ rhs, long long rhs_stride,
                 cplx_t<R> *__restrict__ y, long long y_stride,
                 unsigned long long *__restrict__ prof)
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

    const int N = g.N, KL = CKL ? CKL : g.KL, KU = CKU ? CKU : g.KU, UW = KL + KU + 1;
    const int WR = KL + NB, WC = KL + KU + NB, P = blk_pitch(WC);
    const int S = MODEL ? ms.cs.S : 1;
    const unsigned magic = (MODEL && S > 1) ? (unsigned) ((0x100000000ull + S - 1) / S) : 0u;

    extern __shared__ __align__(16) unsigned char smem_raw[];
    // WR x WC, row pitch P, plus the sink row WR: the trailing update's
    // out-of-range rows and columns read and write row WR and column WC
    // instead of being predicated; nothing else reads the sinks.
    T2 *win = reinterpret_cast<T2 *>(smem_raw);
    T2 *rs = win + (WR + 1) * P;                      // RHS per row slot
    T2 *stg = rs + WR;                                // NB x WC staged rows (STAGE)
    T2 *stgr = stg + (STAGE ? NB * WC : 0);           // NB staged RHS entries (STAGE)
    T2 *coef = stgr + (STAGE ? NB : 0);               // 3 S^2 (model)
    int *pvoff = reinterpret_cast<int *>(coef + (MODEL ? 3 * S * S : 0));   // NB
    int *shv = pvoff + NB;                            // [0] ju, [1] info

    T2 *fu = fac + fi * fac_stride;
    T2 *fl = fu + (long long) N * UW;
    int *pv = ipiv + fi * N;
    const T2 zero = mk<R>(R(0), R(0));

    // Optional per-phase cycle counters (diagnostics), kept by thread 0 in
    // shared memory so that no registers are held for them: 0 init, 1 panel
    // (+ staging), 2 interchanges + U12, 3 GEMM + U rows out, 5 retire/enter;
    // 6..8 the panel's sub-phases; 10 and 11 the last marks.
    unsigned long long *clk = reinterpret_cast<unsigned long long *>(shv + 4);
    const bool timing = PROF && prof && tid == 0;
    if (timing) {
        for (int i = 0; i < 12; ++i) clk[i] = 0;
        clk[10] = clock64();
    }
    auto tick = [&](int ph) {
        if (timing) {
            const unsigned long long t = clock64();
            clk[ph] += t - clk[10];
            clk[10] = t;
        }
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

    // Initial window: rows 0..WR-1, columns 0..WC-1 (slots equal indices).
    {
        const int rb0 = WR * warp / NW, re0 = WR * (warp + 1) / NW;
        assemble_rows<R, MODEL>(src, ms, coef, magic, s, N, KL, KU, WC, rb0, re0 - rb0, 0, lane,
                                [&](int k, int cc, T2 v) { win[(rb0 + k) * P + cc] = v; });
    }
    if (FWD)
        for (int r = tid; r < WR; r += NT)
            rs[r] = r < N ? from_z<R>(rhs[s * rhs_stride + r]) : zero;
    if (tid == 0) { shv[0] = 0; shv[1] = 0; }
    __syncthreads();
    tick(0);

    int rb = 0, cb = 0;
    for (int j0 = 0; j0 < N; j0 += NB) {
        const int nbk = NFULL ? NB : imin(NB, N - j0);
        const bool more = j0 + nbk < N;
        auto rsl = [&](int i) { int t = rb + i; return t >= WR ? t - WR : t; };
        auto csl = [&](int c) { int t = cb + c; return t >= WC ? t - WC : t; };

        // ---------------- 1. panel factorization (warp 0) -----------------
        // The panel lives in registers: lane l holds rows l, l+32, .. of the
        // nbk panel columns (row k of step k is row k of slot 0, on lane k).
        if (warp == 0) {
            panel_factor<R, NB, RS, FWD>(win, P, WR, WC, rb, cb, WR, rs, pvoff, shv, j0, nbk, N, KL,
                                         KU, fl, pv, FWD ? y + s * y_stride : nullptr, lane,
                                         timing ? clk : nullptr);
        } else if constexpr (STAGE) {
            // the next nbk rows of A, at the next window's columns
            if (more) {
                const int kb = nbk * (warp - 1) / (NW - 1), ke = nbk * warp / (NW - 1);
                // three staging warps: one row and two column passes per
                // load group (fewer live registers: no spills at the
                // 80-register bound of the three-warp instances)
                assemble_rows<R, MODEL, (NW >= 3 ? 1 : 2), (NW >= 3 ? 2 : 3)>(
                    src, ms, coef, magic, s, N, KL, KU, WC, j0 + WR + kb, ke - kb, j0 + nbk, lane,
                    [&](int k, int cc, T2 v) { stg[(kb + k) * WC + cc] = v; });
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
        // The panel's interchange offsets, row offsets and L11 are read once
        // into registers; per column the interchanges are applied in order,
        // the nbk entries loaded together and U12 solved in registers (the
        // same multiply-adds in the same order as a column-by-column sweep).
        // Trailing columns exist only when column j0 + nbk exists, so then
        // the panel is full (nbk == NB): phases 2 and 3 need no nbk guards.
        if (ntr > 0) {
            int bts[NB], ro[NB];
            T2 l11[NB][NB];
#pragma unroll
            for (int k = 0; k < NB; ++k) {
                bts[k] = pvoff[k];
                ro[k] = rsl(k) * P;
#pragma unroll
                for (int m = 0; m < NB; ++m)
                    l11[k][m] = m < k ? win[ro[k] + csl(m)] : zero;
            }
            for (int c = nbk + tid; c <= ce; c += NT) {
                const int cc = csl(c);
#pragma unroll
                for (int k = 0; k < NB; ++k) {
                    if (bts[k]) {
                        T2 &a = win[ro[k] + cc], &b = win[rsl(k + bts[k]) * P + cc];
                        const T2 t = a; a = b; b = t;
                    }
                }
                T2 u[NB];
#pragma unroll
                for (int k = 0; k < NB; ++k) u[k] = win[ro[k] + cc];
#pragma unroll
                for (int k = 1; k < NB; ++k)
#pragma unroll
                    for (int m = 0; m < k; ++m) u[k] = cfnma(l11[k][m], u[m], u[k]);
#pragma unroll
                for (int k = 0; k < NB; ++k) win[ro[k] + cc] = u[k];
            }
        }
        __syncthreads();
        tick(2);

        // ---------------- 3. A22 -= L21 U12 (register-tiled GEMM) -----------
        // and U rows out (rows < nbk, which the GEMM does not touch)
        if (ntr > 0) {
            const int rg = tid >> 3, cg = tid & 7;
            const int nrow = imin(KL, N - j0 - nbk);     // rows nbk .. nbk+nrow-1
            // complex64: explicit shared-window byte addresses, one integer add
            // per access; complex128 (larger tiles, more live registers):
            // element offsets into win
            constexpr bool BYTE = sizeof(R) == 4;
            constexpr unsigned ES = BYTE ? sizeof(T2) : 1u;
            const unsigned wsh = BYTE ? (unsigned) __cvta_generic_to_shared(win) : 0u;
            auto ld = [&](unsigned a) -> T2 {
                if constexpr (BYTE) return lds_c(a, T2{});
                else return win[a];
            };
            auto st = [&](unsigned a, T2 v) {
                if constexpr (BYTE) sts_c(a, v);
                else win[a] = v;
            };
            unsigned rB[MAXTR];                           // address of each row
#pragma unroll
            for (int t = 0; t < MAXTR; ++t) {
                const int i = rg + RGN * t;
                rB[t] = wsh + (unsigned) ((i < nrow) ? rsl(nbk + i) * P : WR * P) * ES;
            }
            for (int c0 = 0; c0 < ntr; c0 += 8 * TC) {
                unsigned cB[TC];                          // offset of each column
#pragma unroll
                for (int u = 0; u < TC; ++u) {
                    const int c = c0 + cg + 8 * u;
                    cB[u] = (unsigned) ((c < ntr) ? csl(nbk + c) : WC) * ES;
                }
                T2 acc[MAXTR][TC];
#pragma unroll
                for (int t = 0; t < MAXTR; ++t)
#pragma unroll
                    for (int u = 0; u < TC; ++u)
                        acc[t][u] = ld(rB[t] + cB[u]);
#pragma unroll
                for (int m = 0; m < NB; ++m) {       // nbk == NB here
                    const unsigned cm = (unsigned) csl(m) * ES, rm = wsh + (unsigned) (rsl(m) * P) * ES;
                    T2 l[MAXTR], uu[TC];
#pragma unroll
                    for (int t = 0; t < MAXTR; ++t) l[t] = ld(rB[t] + cm);
#pragma unroll
                    for (int u = 0; u < TC; ++u) uu[u] = ld(rm + cB[u]);
                    if constexpr (sizeof(R) == 4) {
                        // complex64: two packed FMAs per complex multiply-add
                        float2 la[MAXTR], lb[MAXTR], us[TC];
#pragma unroll
                        for (int t = 0; t < MAXTR; ++t) {
                            la[t] = make_float2(-l[t].x, -l[t].x);
                            lb[t] = make_float2(l[t].y, -l[t].y);
                        }
#pragma unroll
                        for (int u = 0; u < TC; ++u) us[u] = make_float2(uu[u].y, uu[u].x);
#pragma unroll
                        for (int t = 0; t < MAXTR; ++t)
#pragma unroll
                            for (int u = 0; u < TC; ++u)
                                acc[t][u] = cfnma2(la[t], lb[t], uu[u], us[u], acc[t][u]);
                    } else {
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
                        st(rB[t] + cB[u], acc[t][u]);
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
            auto put = [&](int k, int cc, T2 v) {
                int cs = cb + nbk + cc;          // < 3 WC: wrap at most twice
                if (cs >= WC) cs -= WC;
                if (cs >= WC) cs -= WC;
                win[rsl(k) * P + cs] = v;
            };
            if constexpr (STAGE) {
                for (int k = warp; k < nbk; k += NW)
                    for (int cc = lane; cc < WC; cc += 32) put(k, cc, stg[k * WC + cc]);
            } else {
                const int kb = nbk * warp / NW, ke = nbk * (warp + 1) / NW;
                assemble_rows<R, MODEL>(src, ms, coef, magic, s, N, KL, KU, WC, j0 + WR + kb, ke - kb,
                                        j0 + nbk, lane,
                                        [&](int k, int cc, T2 v) { put(kb + k, cc, v); });
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
    if (timing)
        for (int ph = 0; ph < 9; ++ph) atomicAdd(prof + ph, clk[ph]);
}

template <typename R, int NB, int NW, int MAXTR, bool MODEL, bool FWD, int CKL = 0, int CKU = 0,
          bool NFULL = false, bool PROF = false>
__global__ void __launch_bounds__(32 * NW, (blk_min_blocks<R, NW>()))
k_gbtrf_cta(FactorGeom g, int nsys, PackedSource src, ModelSource ms,
            cplx_t<R> *__restrict__ fac, long long fac_stride,
            int *__restrict__ ipiv, int *__restrict__ info,
            const double2 *__restrict__ rhs, long long rhs_stride,
            cplx_t<R> *__restrict__ y, long long y_stride,
            const int *__restrict__ sys_list, const int *__restrict__ d_count,
            bool slot_mode, unsigned long long *__restrict__ prof)
{
    if (d_count && (int) blockIdx.x >= *d_count) return;
    const int s = sys_list ? sys_list[blockIdx.x] : (int) blockIdx.x;
    if (s < 0 || s >= nsys) return;
    const long long fi = slot_mode ? (long long) blockIdx.x : (long long) s;
    gbtrf_cta_system<R, NB, NW, MAXTR, MODEL, FWD, ModelSource, CKL, CKU, NFULL, PROF>(g, s, fi, src, ms, fac, fac_stride, ipiv, info, rhs,
                                                   rhs_stride, y, y_stride, prof);
}

// Ragged factor: one CTA per work item (plan d, list position k), the
// items in the order given (the largest plans' systems first, which the
// block scheduler dispatches first); each item is one system of one plan,
// of that plan's own geometry (KL <= 4 NW MAXTR; KL = CKL, KU = CKU and N a
// multiple of 4 in the specialized instances), or nothing when k is beyond
// the plan's active count.  The plan's descriptor is read once into shared
// memory (fewer live registers than a copy in registers).
// The shared memory is sized for the largest window of the batch.
template <int NW, int MAXTR, int CKL = 0, int CKU = 0, bool NFULL = false>
__global__ void __launch_bounds__(32 * NW, (blk_min_blocks<float, NW>()))
k_gbtrf_ragged(const RaggedDesc *__restrict__ descs, const int2 *__restrict__ items)
{
    __shared__ RaggedDesc sd;
    const int2 w = items[blockIdx.x];
    if (threadIdx.x == 0) sd = descs[w.x];
    __syncthreads();
    if (w.y >= *sd.d_count) return;
    const int s = sd.sys_list[w.y];
    gbtrf_cta_system<float, 4, NW, MAXTR, true, true, const ModelSource &, CKL, CKU, NFULL>(
        sd.g, s, s, PackedSource{}, sd.ms, sd.fac, sd.fac_stride, sd.ipiv, sd.info, sd.rhs,
        sd.rhs_stride, sd.y, sd.y_stride, nullptr);
}

// Lookahead form (NW >= 2): warp 0 factors panel J while warps 1..NW-1 apply
// panel J-1's deferred update to the columns beyond panel J, write panel
// J-1's U rows and assemble the rows that enter after panel J; the panel's
// sequential latency is hidden behind the trailing update.  Panel J-1's rows
// and columns therefore stay one panel longer: the window spans rows
// j0-NB .. j0+KL+NB-1 and columns j0-NB .. j0+KL+KU+NB-1 (logical row lr is
// row j0-NB+lr, logical column lc is column j0-NB+lc).  Per panel J:
//   A. warp 0: panel J;  workers: A(j0.., j0+NB..ju_{J-1}) -= L21_{J-1}
//      U12_{J-1}, U rows of panel J-1 out, rows j0+KL+NB.. staged;
//   B. all: panel J's interchanges and U12 on its trailing columns;
//   C. all: panel J+1's columns -= L21_J U12_J, panel J-1's columns retire
//      (zeroed), its row slots take the staged rows.
// Each element still receives the multiply-adds of zgbtf2 in zgbtf2's order:
// panel J-1's update of a column always precedes panel J's.
template <typename R, int NB, int NW, bool MODEL, bool FWD>
__global__ void __launch_bounds__(32 * NW, (blk_min_blocks<R, NW>()))
k_gbtrf_la(FactorGeom g, int nsys, PackedSource src, ModelSource ms,
           cplx_t<R> *__restrict__ fac, long long fac_stride,
           int *__restrict__ ipiv, int *__restrict__ info,
           const double2 *__restrict__ rhs, long long rhs_stride,
           cplx_t<R> *__restrict__ y, long long y_stride,
           const int *__restrict__ sys_list, const int *__restrict__ d_count,
           bool slot_mode, unsigned long long *__restrict__ prof)
{
    static_assert(NW >= 2, "the lookahead form needs worker warps");
    using T2 = cplx_t<R>;
    constexpr int NT = 32 * NW, NWK = NW - 1, NTK = 32 * NWK;
    constexpr int TC = sizeof(R) == 8 ? 3 : 5;      // worker GEMM columns per thread per pass
    constexpr int MT = 3;                             // worker GEMM rows per thread per pass
    constexpr int RGW = NTK / 8;                      // worker GEMM row groups
    constexpr int RS = 3;                             // panel rows per lane: KL + NB <= 96
    constexpr int LNB = NB == 4 ? 2 : NB == 8 ? 3 : 4;
    static_assert((1 << LNB) == NB, "NB must be 4, 8 or 16");
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (d_count && (int) blockIdx.x >= *d_count) return;
    const int s = sys_list ? sys_list[blockIdx.x] : (int) blockIdx.x;
    if (s < 0 || s >= nsys) return;
    const long long fi = slot_mode ? (long long) blockIdx.x : (long long) s;

    const int N = g.N, KL = g.KL, KU = g.KU, UW = g.UW();
    const int WR = KL + 2 * NB, WC = KL + KU + 2 * NB, P = blk_pitch(WC);
    const int S = MODEL ? ms.cs.S : 1;
    const unsigned magic = (MODEL && S > 1) ? (unsigned) ((0x100000000ull + S - 1) / S) : 0u;

    extern __shared__ __align__(16) unsigned char smem_raw[];
    T2 *win = reinterpret_cast<T2 *>(smem_raw);       // WR x WC, pitch P, + sink row WR
    T2 *rs = win + (WR + 1) * P;                      // RHS per row slot
    T2 *stg = rs + WR;                                // NB x WC staged rows
    T2 *stgr = stg + NB * WC;                         // NB staged RHS entries
    T2 *coef = stgr + NB;                             // 3 S^2 (model)
    int *pvoff = reinterpret_cast<int *>(coef + (MODEL ? 3 * S * S : 0));   // NB
    int *shv = pvoff + NB;                            // [0] ju, [1] info, [2] ju of panel J-1

    T2 *fu = fac + fi * fac_stride;
    T2 *fl = fu + (long long) N * UW;
    int *pv = ipiv + fi * N;
    const T2 zero = mk<R>(R(0), R(0));

    // Optional per-phase cycle counters (diagnostics), kept by thread 0 in
    // shared memory so that no registers are held for them: 0 init, 1 phase A,
    // 2 phase B, 3 phase C, 4 last U rows; 10 the last mark.
    unsigned long long *clk = reinterpret_cast<unsigned long long *>(shv + 4);
    const bool timing = prof && tid == 0;
    if (timing) {
        for (int i = 0; i < 12; ++i) clk[i] = 0;
        clk[10] = clock64();
    }
    auto tick = [&](int ph) {
        if (timing) {
            const unsigned long long t = clock64();
            clk[ph] += t - clk[10];
            clk[10] = t;
        }
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

    // Initial window (rb = cb = 0): slot lr holds row lr-NB, slot lc column
    // lc-NB; rows and columns before 0 are zero.
    {
        const int lb = WR * warp / NW, le = WR * (warp + 1) / NW;
        assemble_rows<R, MODEL>(src, ms, coef, magic, s, N, KL, KU, WC, lb - NB, le - lb, -NB, lane,
                                [&](int k, int cc, T2 v) { win[(lb + k) * P + cc] = v; });
    }
    if (FWD)
        for (int lr = tid; lr < WR; lr += NT) {
            const int r = lr - NB;
            rs[lr] = (r >= 0 && r < N) ? from_z<R>(rhs[s * rhs_stride + r]) : zero;
        }
    if (tid == 0) { shv[0] = 0; shv[1] = 0; shv[2] = 0; }
    __syncthreads();
    tick(0);

    int rb = 0, cb = 0, nbp = 0;      // nbp: columns of panel J-1 (0 before the first)
    int j0 = 0;
    for (; j0 < N; j0 += NB) {
        const int nbk = imin(NB, N - j0);
        const bool more = j0 + nbk < N;
        auto rsl = [&](int lr) { int t = rb + lr; return t >= WR ? t - WR : t; };
        auto csl = [&](int lc) { int t = cb + lc; return t >= WC ? t - WC : t; };

        // ---------------- A. panel J | update of panel J-1, staging --------
        if (warp == 0) {
            const int rbp = rsl(NB), cbp = csl(NB);
            panel_factor<R, NB, RS, FWD>(win, P, WR, WC, rbp, cbp, KL + NB, rs, pvoff, shv, j0, nbk,
                                         N, KL, KU, fl, pv, FWD ? y + s * y_stride : nullptr, lane);
        } else {
            const int wt = tid - 32;
            if (nbp > 0) {
                // A(j0+i, j0+NB .. ju_{J-1}) -= L21_{J-1} U12_{J-1}
                const int cep = shv[2] - (j0 - NB);      // last column, logical
                const int ntr = cep - 2 * NB + 1;
                const int nrow = imin(KL, N - j0);       // rows lr = NB + i
                const int rg = wt >> 3, cg = wt & 7;
                for (int r0 = 0; r0 < nrow && ntr > 0; r0 += RGW * MT) {
                    int roff[MT];
#pragma unroll
                    for (int t = 0; t < MT; ++t) {
                        const int i = r0 + rg + RGW * t;
                        roff[t] = (i < nrow) ? rsl(NB + i) * P : WR * P;
                    }
                    for (int c0 = 0; c0 < ntr; c0 += 8 * TC) {
                        int coff[TC];
#pragma unroll
                        for (int u = 0; u < TC; ++u) {
                            const int c = c0 + cg + 8 * u;
                            coff[u] = (c < ntr) ? csl(2 * NB + c) : WC;
                        }
                        T2 acc[MT][TC];
#pragma unroll
                        for (int t = 0; t < MT; ++t)
#pragma unroll
                            for (int u = 0; u < TC; ++u)
                                acc[t][u] = win[roff[t] + coff[u]];
#pragma unroll
                        for (int m = 0; m < NB; ++m) {
                            if (m < nbp) {
                                const int cm = csl(m), rm = rsl(m) * P;
                                T2 l[MT], uu[TC];
#pragma unroll
                                for (int t = 0; t < MT; ++t) l[t] = win[roff[t] + cm];
#pragma unroll
                                for (int u = 0; u < TC; ++u) uu[u] = win[rm + coff[u]];
                                if constexpr (sizeof(R) == 4) {
                                    // complex64: two packed FMAs per complex multiply-add
                                    float2 la[MT], lb[MT], us[TC];
#pragma unroll
                                    for (int t = 0; t < MT; ++t) {
                                        la[t] = make_float2(-l[t].x, -l[t].x);
                                        lb[t] = make_float2(l[t].y, -l[t].y);
                                    }
#pragma unroll
                                    for (int u = 0; u < TC; ++u) us[u] = make_float2(uu[u].y, uu[u].x);
#pragma unroll
                                    for (int t = 0; t < MT; ++t)
#pragma unroll
                                        for (int u = 0; u < TC; ++u)
                                            acc[t][u] = cfnma2(la[t], lb[t], uu[u], us[u], acc[t][u]);
                                } else {
#pragma unroll
                                    for (int t = 0; t < MT; ++t)
#pragma unroll
                                        for (int u = 0; u < TC; ++u)
                                            acc[t][u] = cfnma(l[t], uu[u], acc[t][u]);
                                }
                            }
                        }
#pragma unroll
                        for (int t = 0; t < MT; ++t)
#pragma unroll
                            for (int u = 0; u < TC; ++u)
                                win[roff[t] + coff[u]] = acc[t][u];
                    }
                }
                // U rows of panel J-1 (rows j0-NB+m, slot lr = m)
                for (int m = warp - 1; m < nbp; m += NWK) {
                    const long long jr = j0 - NB + m;
                    const int ro = rsl(m) * P;
                    for (int t = lane; t < UW; t += 32) fu[jr * UW + t] = win[ro + csl(m + t)];
                }
            }
            // rows j0+KL+NB+k enter after this panel, at the next window's
            // columns j0 .. j0+WC-1
            if (more) {
                const int kb = NB * (warp - 1) / NWK, ke = NB * warp / NWK;
                assemble_rows<R, MODEL>(src, ms, coef, magic, s, N, KL, KU, WC, j0 + KL + NB + kb,
                                        ke - kb, j0, lane,
                                        [&](int k, int cc, T2 v) { stg[(kb + k) * WC + cc] = v; });
                if (FWD)
                    for (int k = wt; k < NB; k += NTK) {
                        const int r = j0 + KL + NB + k;
                        stgr[k] = r < N ? from_z<R>(rhs[s * rhs_stride + r]) : zero;
                    }
            }
        }
        __syncthreads();
        tick(1);

        // ---------------- B. interchanges and U12 of panel J ---------------
        // Trailing columns exist only when column j0 + nbk does, so then the
        // panel is full (nbk == NB).  The interchange offsets, row offsets
        // and L11 are read once into registers; per column the interchanges
        // are applied in order and U12 solved in registers (the order of
        // multiply-adds of a column-by-column sweep).
        const int ju = shv[0];
        const int ce = ju - (j0 - NB);       // last trailing column, logical (< WC)
        if (ce >= NB + nbk) {
            int bts[NB], ro[NB];
            T2 l11[NB][NB];
#pragma unroll
            for (int k = 0; k < NB; ++k) {
                bts[k] = pvoff[k];
                ro[k] = rsl(NB + k) * P;
#pragma unroll
                for (int m = 0; m < NB; ++m) l11[k][m] = m < k ? win[ro[k] + csl(NB + m)] : zero;
            }
            for (int c = NB + nbk + tid; c <= ce; c += NT) {
                const int cc = csl(c);
#pragma unroll
                for (int k = 0; k < NB; ++k) {
                    if (bts[k]) {
                        T2 &a = win[ro[k] + cc], &b = win[rsl(NB + k + bts[k]) * P + cc];
                        const T2 t = a; a = b; b = t;
                    }
                }
                T2 u[NB];
#pragma unroll
                for (int k = 0; k < NB; ++k) u[k] = win[ro[k] + cc];
#pragma unroll
                for (int k = 1; k < NB; ++k)
#pragma unroll
                    for (int m = 0; m < k; ++m) u[k] = cfnma(l11[k][m], u[m], u[k]);
#pragma unroll
                for (int k = 0; k < NB; ++k) win[ro[k] + cc] = u[k];
            }
        }
        __syncthreads();
        if (tid == 0) shv[2] = ju;           // read by the workers in the next phase A
        tick(2);

        // ---------------- C. panel J+1's columns; retire / enter -----------
        if (more) {
            const int nrow = imin(KL, N - j0 - nbk);            // rows lr = NB + nbk + i
            const int ncol = imin(NB, ce - (NB + nbk) + 1);     // columns lc = NB + nbk + c
            for (int idx = tid; idx < nrow * NB; idx += NT) {
                const int i = idx >> LNB, c = idx & (NB - 1);
                if (c < ncol) {
                    const int ro = rsl(NB + nbk + i) * P, cc = csl(NB + nbk + c);
                    T2 acc = win[ro + cc];
#pragma unroll
                    for (int m = 0; m < NB; ++m)
                        if (m < nbk) acc = cfnma(win[ro + csl(NB + m)], win[rsl(NB + m) * P + cc], acc);
                    win[ro + cc] = acc;
                }
            }
            // panel J-1's columns (lc < NB) become columns j0+KL+KU+NB.. of the
            // staying rows: zero
            for (int idx = tid; idx < WR * NB; idx += NT) {
                const int lr = idx >> LNB, c = idx & (NB - 1);
                if (lr >= NB) win[rsl(lr) * P + csl(c)] = zero;
            }
            // panel J-1's row slots take rows j0+KL+NB+k (next columns j0 + cc)
            for (int k = warp; k < NB; k += NW) {
                T2 *dst = win + rsl(k) * P;
                for (int cc = lane; cc < WC; cc += 32) {
                    int cs = cb + NB + cc;           // < 3 WC: wrap at most twice
                    if (cs >= WC) cs -= WC;
                    if (cs >= WC) cs -= WC;
                    dst[cs] = stg[k * WC + cc];
                }
            }
            if (FWD)
                for (int k = tid; k < NB; k += NT) rs[rsl(k)] = stgr[k];
            __syncthreads();
        }
        tick(3);
        rb += NB; if (rb >= WR) rb -= WR;
        cb += NB; if (cb >= WC) cb -= WC;
        nbp = nbk;
    }
    // U rows of the last panel (rows j0-NB+m, slot lr = m after the shift)
    {
        auto rsl = [&](int lr) { int t = rb + lr; return t >= WR ? t - WR : t; };
        auto csl = [&](int lc) { int t = cb + lc; return t >= WC ? t - WC : t; };
        for (int m = warp; m < nbp; m += NW) {
            const long long jr = j0 - NB + m;
            const int ro = rsl(m) * P;
            for (int t = lane; t < UW; t += 32) fu[jr * UW + t] = win[ro + csl(m + t)];
        }
    }
    tick(4);
    if (tid == 0) info[fi] = shv[1];
    if (timing)
        for (int ph = 0; ph < 6; ++ph) atomicAdd(prof + ph, clk[ph]);
}

template <typename R, int NB, int NW, int MAXTR, bool LA, bool MODEL, bool FWD, int CKL = 0,
          int CKU = 0, bool NFULL = false>
cudaError_t launch_cta_one(const GbtrfArgs &a, cudaStream_t st)
{
    const int S = MODEL ? a.ms.cs.S : 1;
    const size_t smem = gbtrf_blk_smem_bytes(sizeof(R), a.g, S, NB, LA ? -NW : NW);
    // the phase counters: compiled into the generic packed-band instances
    // only (the diagnostic entry's), absent elsewhere
    constexpr bool CAN_PROF = LA || (!MODEL && !FWD && CKL == 0);
    if (!CAN_PROF && a.prof) return cudaErrorInvalidValue;
    auto kern = [&] {
        if constexpr (LA) return k_gbtrf_la<R, NB, NW, MODEL, FWD>;
        else if constexpr (CAN_PROF)
            return a.prof ? k_gbtrf_cta<R, NB, NW, MAXTR, MODEL, FWD, CKL, CKU, NFULL, true>
                          : k_gbtrf_cta<R, NB, NW, MAXTR, MODEL, FWD, CKL, CKU, NFULL, false>;
        else return k_gbtrf_cta<R, NB, NW, MAXTR, MODEL, FWD, CKL, CKU, NFULL>;
    }();
    cudaError_t e = smem_attr((const void *) kern, smem);
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

template <typename R, int NB, int NW, int MAXTR, bool LA>
cudaError_t launch_cta_r(const GbtrfArgs &a, cudaStream_t st)
{
    const bool fwd = a.rhs != nullptr;
    if (a.model) return fwd ? launch_cta_one<R, NB, NW, MAXTR, LA, true, true>(a, st)
                            : launch_cta_one<R, NB, NW, MAXTR, LA, true, false>(a, st);
    return fwd ? launch_cta_one<R, NB, NW, MAXTR, LA, false, true>(a, st)
               : launch_cta_one<R, NB, NW, MAXTR, LA, false, false>(a, st);
}

// The kernels of one (precision R, panel width NB, warp family FAM) are
// instantiated by one translation unit, gbtrf_blk_inst.cu compiled once per
// triple, so the build compiles them in parallel.  FAM 0 is the lookahead
// kernel (variant 2, nw = 2 or 4, which loops its worker update over row
// passes); FAM 1, 2, 4 the phased kernel with that many warps, KL <= (4 FAM)
// MAXTR rows of the trailing update per thread.
template <typename R, int NB, int FAM>
cudaError_t launch_blk_fam(const GbtrfArgs &a, int nw, cudaStream_t st);

// Bandwidths with compile-time instances of the complex64 phased kernel
// (NB = 4; N a multiple of 4): the geometries of the B-spline operators
// with S = 5 or 7 equations and order k = 6 or 8 whose window leaves room
// for 8 CTAs per SM (KL = KU = S (k - 1) - 1 = 24, 34).  Each has its own
// translation unit (gbtrf_blk_inst.cu with SGB_BLK_SPEC set).  Two warps
// use 5 x 5 register tiles; the three-warp shape (nw 3: 12 row groups x 3
// rows cover KL, 3 x 5 tiles) is the default for a packed band (10 % faster
// at N = 960, KL = 34) and, at KL = 34, for rows assembled from the model
// operator (5 % faster once the staging's load groups shrank to fit 80
// registers); model rows at KL = 24 keep two.  KL = 48 (S = 7, k = 8)
// takes the generic four-warp kernel: its 48 KB window allows 4 CTAs per SM,
// so four warps with 3 x 5 tiles fit without spills, measured 18 % (model
// rows) to 37 % (packed band) faster than two, and fixing KL there gains
// nothing.
constexpr int kSpecBands[] = {24, 34};
constexpr bool spec_has_w3(int kb) { return kb <= 36; }
template <int W> constexpr int spec_maxtr() { return W == 3 ? 3 : 5; }
template <int KB>
cudaError_t launch_blk_spec(const GbtrfArgs &a, int nw, cudaStream_t st);
// The specialized launch for a's geometry and warp count when one exists
// (complex64, NB 4, KL = KU in kSpecBands, N % 4 == 0, nw 2, or 3 where
// the band has that shape); *done false otherwise.
cudaError_t launch_blk_spec_any(const GbtrfArgs &a, int nw, cudaStream_t st, bool *done);

}  // namespace sgb
