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
//
// The sweeps are sequential in j, so each step's factor row (or column, and
// its pivot) must not wait on HBM: a ring of PD records in shared memory is
// filled PD records ahead of its use, by cp.async or, for the backward
// quad solve, by one bulk copy (1-D TMA) of two consecutive U rows per
// record completing on an mbarrier.
#include "sgb_internal.h"

#include <algorithm>

namespace sgb {

// Asynchronous global -> shared copy of one complex element (cp.async, 8 or
// 16 bytes) and of one int; groups committed per sweep step.
template <typename R>
__device__ __forceinline__ void cp_el(cplx_t<R> *dst, const cplx_t<R> *src)
{
    const unsigned d = (unsigned) __cvta_generic_to_shared(dst);
    if constexpr (sizeof(R) == 8)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_int(int *dst, const int *src)
{
    const unsigned d = (unsigned) __cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// One-dimensional bulk copy (TMA) of `bytes` (a multiple of 16, both
// addresses 16-byte aligned) from global into this CTA's shared memory,
// completing on the mbarrier at `bar` (the issuing lane declares the bytes).
__device__ __forceinline__ void bulk_to_smem(void *dst, const void *src, unsigned bytes, unsigned bar)
{
    const unsigned d = (unsigned) __cvta_generic_to_shared(dst);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n"
                 ::"r"(d), "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}
__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count) : "memory");
}
// Waits for phase `parity` of the mbarrier, at most `limit` polls; false on
// time-out (the caller records a fault and stops).
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity, int limit = 1 << 20)
{
    for (int i = 0; i < limit; ++i) {
        unsigned done;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                     " selp.u32 %0, 1, 0, p;\n}\n"
                     : "=r"(done) : "r"(bar), "r"(parity) : "memory");
        if (done) return true;
    }
    return false;
}

// Set by a kernel whose bounded wait on an asynchronous copy ran out (its
// results are then invalid); read and cleared by sgb_async_faults().
__device__ int g_async_fault = 0;

// Prefetch depth (sweep steps in flight) per precision.
template <typename R> __host__ __device__ constexpr int gbtrs_depth() { return sizeof(R) == 8 ? 4 : 8; }

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
    constexpr int PD = gbtrs_depth<R>();
    const int lane = threadIdx.x;
    if (d_count && (int) blockIdx.x >= *d_count) return;
    const int s = sys_list ? sys_list[blockIdx.x] : (int) blockIdx.x;
    if (s < 0 || s >= nsys) return;
    if (status && status[s] != status_want) return;
    const long long fi = slot_mode ? (long long) blockIdx.x : (long long) s;
    const int N = g.N, KL = g.KL, UW = g.UW(), KV = UW - 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T2 *xs = reinterpret_cast<T2 *>(smem_raw);        // N
    T2 *ru = xs + N;                                   // PD x UW ring of U rows
    T2 *rl = ru + PD * UW;                             // PD x KL ring of L columns
    int *rp = reinterpret_cast<int *>(rl + PD * KL);   // PD pivots
    const T2 *fu = fac + fi * fac_stride;
    const T2 *fl = fu + (long long) N * UW;
    const int *pv = ipiv + (fac_stride ? fi * N : 0);   // stride 0: one shared factor
    const bool cj = (TRANS == 2);

    // ring fillers: step t's data into slot t % PD (empty groups past the end)
    auto fetch_u = [&](int row) {
        if (row >= 0 && row < N) {
            T2 *d = ru + (row % PD) * UW;
            const T2 *src = fu + (long long) row * UW;
            for (int k = lane; k < UW; k += 32) cp_el<R>(d + k, src + k);
        }
        cp_commit();
    };
    auto fetch_l = [&](int col) {
        if (col >= 0 && col < N - 1) {
            T2 *d = rl + (col % PD) * KL;
            const T2 *src = fl + (long long) col * KL;
            for (int i = lane; i < KL; i += 32) cp_el<R>(d + i, src + i);
            if (lane == 0) cp_int(rp + col % PD, pv + col);
        }
        cp_commit();
    };

    for (int i = lane; i < N; i += 32)
        xs[i] = FWD_DONE ? yin[s * b_stride + i] : from_z<R>(b[s * b_stride + i]);
    __syncwarp();

    if (TRANS == 0) {
        if (!FWD_DONE && KL > 0) {
#pragma unroll 1
            for (int t = 0; t < PD; ++t) fetch_l(t);
            for (int j = 0; j < N - 1; ++j) {
                cp_wait<PD - 1>();
                __syncwarp();
                const T2 *lc = rl + (j % PD) * KL;
                const int lm = imin(KL, N - 1 - j);
                const int l = rp[j % PD] - 1;
                if (l != j) {
                    T2 a = xs[j], c = xs[l];
                    __syncwarp();
                    if (lane == 0) { xs[j] = c; xs[l] = a; }
                    __syncwarp();
                }
                const T2 xj = xs[j];
                for (int i = lane; i < lm; i += 32)
                    xs[j + 1 + i] = cfnma(lc[i], xj, xs[j + 1 + i]);
                __syncwarp();
                fetch_l(j + PD);
            }
            cp_wait<0>();
            __syncwarp();
        }
#pragma unroll 1
        for (int t = 0; t < PD; ++t) fetch_u(N - 1 - t);
        for (int j = N - 1; j >= 0; --j) {
            cp_wait<PD - 1>();
            __syncwarp();
            const T2 *ur = ru + (j % PD) * UW;
            T2 acc = mk<R>(R(0), R(0));
            for (int k = 1 + lane; k <= KV && j + k < N; k += 32)
                acc = cfma(ur[k], xs[j + k], acc);
            acc = warp_csum<R>(acc);
            if (lane == 0) xs[j] = cmul(csub(xs[j], acc), crcp<R>(ur[0]));
            __syncwarp();
            fetch_u(j - PD);
        }
    } else {
#pragma unroll 1
        for (int t = 0; t < PD; ++t) fetch_u(t);
        for (int j = 0; j < N; ++j) {
            cp_wait<PD - 1>();
            __syncwarp();
            const T2 *ur = ru + (j % PD) * UW;
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
            fetch_u(j + PD);
        }
        cp_wait<0>();
        __syncwarp();
        if (KL > 0) {
#pragma unroll 1
            for (int t = 0; t < PD; ++t) fetch_l(N - 2 - t);
            for (int j = N - 2; j >= 0; --j) {
                cp_wait<PD - 1>();
                __syncwarp();
                const T2 *lc = rl + (j % PD) * KL;
                const int lm = imin(KL, N - 1 - j);
                T2 acc = mk<R>(R(0), R(0));
                for (int i = lane; i < lm; i += 32) {
                    T2 l = lc[i];
                    if (cj) l = cconj(l);
                    acc = cfma(l, xs[j + 1 + i], acc);
                }
                acc = warp_csum<R>(acc);
                const int l = rp[j % PD] - 1;
                const T2 xj = csub(xs[j], acc);
                __syncwarp();
                if (lane == 0) {
                    if (l != j) { xs[j] = xs[l]; xs[l] = xj; }
                    else xs[j] = xj;
                }
                __syncwarp();
                fetch_l(j - PD);
            }
        }
    }
    cp_wait<0>();
    __syncwarp();
    for (int i = lane; i < N; i += 32) {
        const int o = unS ? (i % unS) * unn + i / unS : i;
        double2 *dst = x + s * x_stride + o;
        const double2 v = to_z<R>(xs[i]);
        if (ACCUM) { double2 t = *dst; t.x += v.x; t.y += v.y; *dst = t; }
        else *dst = v;
    }
}

// ---------------------------------------------------------------------------
// Quad solves for trans 'N' with a writable y buffer: four lanes per system,
// eight systems per warp, so that the sequential sweeps of eight systems
// share every instruction and the per-step dot products reduce over two
// shuffle levels instead of five.  Per system the shared memory holds a
// window of the vector (a power-of-two ring indexed by row & mask) and a ring
// of PD factor records fetched with cp.async PD steps ahead.
//   forward:  y = L^{-1} P b into ywork (column axpy; pivots and the entering
//             b entry travel in the record of their step)
//   backward: x = U^{-1} y, row dots over lanes k = 1+q, 5+q, ...; x_j is
//             written over the consumed y_j, then one coalesced pass moves
//             ywork to the FP64 output (written or accumulated, optionally
//             scattered to natural order).
// ---------------------------------------------------------------------------
constexpr int QSYS = 8;   // systems per warp (block)

__host__ __device__ inline int quad_pow2(int v)
{
    int p = 1;
    while (p < v) p <<= 1;
    return p;
}
// per-system stride in elements, = 4 (mod 16) so that the eight systems of a
// warp reading four consecutive elements each fill the banks twice
__host__ __device__ inline int quad_pad(int e) { return e + ((4 - e % 16) + 16) % 16; }

// Records in flight per system (forward, backward): template parameters of
// the kernels, chosen at launch from a process-wide setting
// (sgb_gbtrs_set_quad_depth); 2 and 2 unless set.  Shared memory bounds the
// warps per SM, and on the GB300 more resident warps with two records each
// beat fewer warps with deeper rings (N = 960, KL = KU = 34, complex64:
// forward + backward 4.6 ms at depth 2, 6.3 ms at 8 / 4, 8.6 ms at 16 / 8).
static int g_qdepth[2] = {2, 2};
static bool quad_depth_ok(int d) { return d == 2 || d == 4 || d == 8 || d == 16; }
// Backward quad solve: records of 1 row by 16-byte cp.async over the
// system's four lanes (g_qbulk 0 or 1), or of 2, 4 or 8 consecutive rows by
// one bulk copy (TMA) per record and system.  Measured on the GB300 at
// N = 960, KL = KU = 34, complex64, 24,768 systems (backsolve / correction
// solve): 1 row 2.83 / 4.75 ms, 2 rows 2.72 / 4.65 ms, 4 rows 3.25 / 5.21 ms,
// 8 rows 6.06 / 8.34 ms (larger records leave fewer warps per SM).
static int g_qbulk = 2;

// A factor segment of n complex elements starting at element e (from the
// base pointer `base`) is copied with 16-byte cp.async: complex128 element by
// element, complex64 in aligned pairs starting at e & ~1, so the segment
// lands at offset (e & 1) of the destination.  Lane q of a quad copies pairs
// q, q+4, ...; returns the offset.
template <typename R>
__device__ __forceinline__ int quad_copy(cplx_t<R> *dst, const cplx_t<R> *base, long long e, int n,
                                         int q)
{
    if constexpr (sizeof(R) == 8) {
        for (int k = q; k < n; k += 4) cp_el<R>(dst + k, base + e + k);
        return 0;
    } else {
        const int off = (int) (e & 1);
        const long long a0 = e - off;
        const int np = (n + off + 1) >> 1;
#pragma unroll 4
        for (int p = q; p < np; p += 4) {
            const unsigned d = (unsigned) __cvta_generic_to_shared(dst + 2 * p);
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(base + a0 + 2 * p)
                         : "memory");
        }
        return off;
    }
}
// Elements a quad_copy of n elements may write (pairs rounded up, offset).
template <typename R> __host__ __device__ constexpr int quad_span(int n)
{
    return sizeof(R) == 8 ? n : ((n + 2) & ~1);
}

template <typename R, int PD>
struct QuadFwdLayout {
    int XW, RL, SE;       // window (pow2 >= KL+2), L record (span), per-system stride
    __host__ __device__ QuadFwdLayout(const FactorGeom &g)
    {
        constexpr int EB = (int) sizeof(cplx_t<R>);
        XW = quad_pow2(g.KL + 2);
        RL = quad_span<R>(g.KL);
        RL += RL & 1;   // keep every record 16-byte aligned
        const int bytes = (XW + PD * RL) * EB + PD * (int) sizeof(double2) + PD * (int) sizeof(int);
        SE = quad_pad((bytes + EB - 1) / EB);
    }
};
template <typename R, int PD, int RB = 1>
struct QuadBwdLayout {
    int XW, SPAN, RP, SE; // mirrored window (2 x (KV+3) ring), rows' span, record, stride
    __host__ __device__ QuadBwdLayout(const FactorGeom &g)
    {
        XW = g.UW() + 2;
        SPAN = quad_span<R>(RB * g.UW());   // RB consecutive U rows, then their y
        RP = SPAN + RB;
        RP += RP & 1;
        SE = quad_pad(2 * XW + PD * RP);
    }
};

// System of lane group `sub` (list position pos): -1 when inactive.
__device__ __forceinline__ int quad_system(int pos, int nsys, const int *sys_list, int nlist,
                                           const int *d_count, const int *status, int status_want)
{
    int count = sys_list ? nlist : nsys;
    if (d_count) count = imin(count, *d_count);
    if (pos >= count) return -1;
    const int s = sys_list ? sys_list[pos] : pos;
    if (s < 0 || s >= nsys) return -1;
    if (status && status[s] != status_want) return -1;
    return s;
}

template <typename R, int PD>
__global__ void __launch_bounds__(32)
k_gbtrs_fwd_quad(FactorGeom g, int nsys, const cplx_t<R> *__restrict__ fac, long long fac_stride,
                 const int *__restrict__ ipiv, const double2 *__restrict__ b, long long b_stride,
                 cplx_t<R> *__restrict__ yw, const int *__restrict__ sys_list, int nlist,
                 const int *__restrict__ d_count, bool slot_mode, const int *__restrict__ status,
                 int status_want)
{
    using T2 = cplx_t<R>;
    const int lane = threadIdx.x, sub = lane >> 2, q = lane & 3;
    const int pos = blockIdx.x * QSYS + sub;
    const int s = quad_system(pos, nsys, sys_list, nlist, d_count, status, status_want);
    const bool act = s >= 0;
    if (!__any_sync(0xffffffffu, act)) return;
    const long long fi = slot_mode ? (long long) pos : (long long) s;
    const int N = g.N, KL = g.KL;
    const QuadFwdLayout<R, PD> L(g);
    const int m = L.XW - 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T2 *xw = reinterpret_cast<T2 *>(smem_raw) + sub * L.SE;
    T2 *rl = xw + L.XW;                                          // PD x RL
    double2 *rb = reinterpret_cast<double2 *>(rl + PD * L.RL);   // PD entering b
    int *rp = reinterpret_cast<int *>(rb + PD);                  // PD pivots
    const long long lbase = fi * fac_stride + (long long) N * g.UW();
    const int *pv = act ? ipiv + (fac_stride ? fi * N : 0) : nullptr;
    const double2 *bs = act ? b + s * b_stride : nullptr;
    T2 *ys = act ? yw + (long long) s * N : nullptr;

    auto fetch = [&](int j) {
        if (act && j < N - 1) {
            quad_copy<R>(rl + (j % PD) * L.RL, fac, lbase + (long long) j * KL, KL, q);
            if (q == 0) cp_int(rp + j % PD, pv + j);
            if (q == 1 && j + 1 + KL < N) cp_el<double>(rb + j % PD, bs + j + 1 + KL);
        }
        cp_commit();
    };
    if (act)
        for (int i = q; i <= KL && i < N; i += 4) xw[i & m] = from_z<R>(bs[i]);
#pragma unroll 1
    for (int t = 0; t < PD; ++t) fetch(t);
    for (int j = 0; j < N - 1; ++j) {
        cp_wait<PD - 1>();
        __syncwarp();
        const int l = rp[j % PD] - 1;
        if (act && q == 0 && l != j) {
            const T2 a = xw[j & m];
            xw[j & m] = xw[l & m];
            xw[l & m] = a;
        }
        __syncwarp();
        if (act) {
            const T2 yj = xw[j & m];
            if (q == 0) ys[j] = yj;
            const int lm = imin(KL, N - 1 - j);
            const T2 *lc = rl + (j % PD) * L.RL + (int) ((lbase + (long long) j * KL) & (sizeof(R) == 8 ? 0 : 1));
            int w = j + 1 + q;
            for (int i = q; i < lm; i += 4, w += 4) {
                T2 &y = xw[w & m];
                y = cfnma(lc[i], yj, y);
            }
            if (q == 1 && j + 1 + KL < N) xw[(j + 1 + KL) & m] = from_z<R>(rb[j % PD]);
        }
        __syncwarp();
        fetch(j + PD);
    }
    cp_wait<0>();
    __syncwarp();
    if (act && q == 0) ys[N - 1] = xw[(N - 1) & m];
}

template <typename R, bool ACCUM, int PD, int RB>
__global__ void __launch_bounds__(32)
k_gbtrs_bwd_quad(FactorGeom g, int nsys, const cplx_t<R> *__restrict__ fac, long long fac_stride,
                 cplx_t<R> *__restrict__ yw, double2 *__restrict__ x, long long x_stride,
                 const int *__restrict__ sys_list, int nlist, const int *__restrict__ d_count,
                 bool slot_mode, const int *__restrict__ status, int status_want, int unS, int unn)
{
    // RB == 1: each record (one U row and its y) by 16-byte cp.async over the
    // system's four lanes; RB > 1: each record holds RB consecutive rows,
    // fetched by one bulk copy (1-D TMA) issued by the system's lane 0 and
    // completing on the record slot's mbarrier, and their y by cp.async.
    constexpr bool BULK = RB > 1;
    using T2 = cplx_t<R>;
    const int lane = threadIdx.x, sub = lane >> 2, q = lane & 3;
    const int pos = blockIdx.x * QSYS + sub;
    const int s = quad_system(pos, nsys, sys_list, nlist, d_count, status, status_want);
    const bool act = s >= 0;
    if (!__any_sync(0xffffffffu, act)) return;
    const long long fi = slot_mode ? (long long) pos : (long long) s;
    const int N = g.N, UW = g.UW(), KV = UW - 1;
    const QuadBwdLayout<R, PD, RB> L(g);
    const int XW = L.XW;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // x window: ring of XW = KV+3 slots (row r at r mod XW), stored twice so
    // that rows j+1 .. j+KV+3 are contiguous from slot(j+1)
    T2 *xw = reinterpret_cast<T2 *>(smem_raw) + sub * L.SE;
    T2 *rec = xw + 2 * XW;                                        // PD x RP
    // BULK: one mbarrier per record slot of each system, after the systems' areas
    unsigned long long *mb = reinterpret_cast<unsigned long long *>(
        reinterpret_cast<T2 *>(smem_raw) + QSYS * L.SE) + sub * PD;
    const unsigned mb0 = (unsigned) __cvta_generic_to_shared(mb);
    const long long ubase = fi * fac_stride;
    T2 *ys = act ? yw + (long long) s * N : nullptr;
    const T2 zero = mk<R>(R(0), R(0));
    // offset of element e within its record: complex64 copies start at the
    // aligned pair holding e
    auto el_off = [&](long long e) { return (int) (e & (sizeof(R) == 8 ? 0 : 1)); };

    // record b: rows hi = N-1-b RB down to lo = max(0, hi-RB+1), into slot
    // b % PD; the rows' elements from offset el_off(e0), then y_lo .. y_hi
    auto fetch = [&](int b) {
        const int hi = N - 1 - b * RB, lo = imax(0, hi - RB + 1);
        if (act && hi >= 0) {
            T2 *d = rec + (b % PD) * L.RP;
            const long long e0 = ubase + (long long) lo * UW;
            const int cnt = (hi - lo + 1) * UW;
            if constexpr (BULK) {
                if (q == 0) {
                    const int off = el_off(e0);
                    const unsigned bytes = sizeof(R) == 8 ? (unsigned) cnt * 16u
                                                          : (unsigned) ((cnt + off + 1) >> 1) * 16u;
                    bulk_to_smem(d, fac + (e0 - off), bytes, mb0 + 8u * (unsigned) (b % PD));
                }
            } else {
                quad_copy<R>(d, fac, e0, cnt, q);
            }
            for (int r = q; r <= hi - lo; r += 4) cp_el<R>(d + L.SPAN + r, ys + lo + r);
        }
        cp_commit();
    };
    if constexpr (BULK) {
        if (q == 0)
            for (int p = 0; p < PD; ++p) mbar_init(mb0 + 8u * p, 1);
        __syncwarp();
    }
    // rows >= N (and never-written slots) read as zeros
    for (int i = q; i < 2 * XW; i += 4) xw[i] = zero;
#pragma unroll 1
    for (int b = 0; b < PD; ++b) fetch(b);
    const int T = (KV + 3) >> 2;          // terms per lane; only the last may pass KV
    const int nblk = (N + RB - 1) / RB;
    int slot = (N - 1) % XW;              // slot of row j
    for (int j = N - 1; j >= 0; --j) {
        const int tj = N - 1 - j, b = tj / RB, hi = N - 1 - b * RB, lo = imax(0, hi - RB + 1);
        if (j == hi) {                    // first row of record b: wait for it
            cp_wait<PD - 1>();
            if constexpr (BULK) {
                const bool ok = !act || mbar_wait(mb0 + 8u * (unsigned) (b % PD), (unsigned) ((b / PD) & 1));
                if (__any_sync(0xffffffffu, !ok)) {
                    // a copy did not complete: record the fault, let the
                    // copies still in flight land (bounded), and stop
                    if (lane == 0) atomicExch(&g_async_fault, 1);
                    if (act && q == 0)
                        for (int p = 1; p < PD && b + p < nblk; ++p)
                            mbar_wait(mb0 + 8u * (unsigned) ((b + p) % PD), (unsigned) (((b + p) / PD) & 1));
                    cp_wait<0>();
                    return;
                }
            }
            __syncwarp();
        }
        const T2 *rb = rec + (b % PD) * L.RP;
        const T2 *rj = rb + L.SPAN + (j - lo) - (L.RP - 1);   // rj[L.RP - 1] = y_j
        const T2 *ur = rb + el_off(ubase + (long long) lo * UW) + (j - lo) * UW;
        const int s1 = slot + 1 == XW ? 0 : slot + 1;
        const T2 *xr = xw + s1 - 1;                   // xr[k] = x_{j+k}, k = 1 .. KV+3
        T2 a0 = zero, a1 = zero, a2 = zero, a3 = zero;
        int t = 0, k = 1 + q;
        for (; t + 4 <= T; t += 4, k += 16) {
            a0 = cfma(ur[k], xr[k], a0);
            a1 = cfma(ur[k + 4], xr[k + 4], a1);
            a2 = cfma(ur[k + 8], xr[k + 8], a2);
            const T2 u3 = (k + 12 <= KV) ? ur[k + 12] : zero;
            a3 = cfma(u3, xr[k + 12], a3);
        }
        for (; t < T; ++t, k += 4) {
            const T2 u = (k <= KV) ? ur[k] : zero;
            a0 = cfma(u, xr[k], a0);
        }
        T2 acc = cadd(cadd(a0, a1), cadd(a2, a3));
        acc.x += __shfl_xor_sync(0xffffffffu, acc.x, 1);
        acc.y += __shfl_xor_sync(0xffffffffu, acc.y, 1);
        acc.x += __shfl_xor_sync(0xffffffffu, acc.x, 2);
        acc.y += __shfl_xor_sync(0xffffffffu, acc.y, 2);
        const T2 xj = cmul(csub(rj[L.RP - 1], acc), crcp<R>(ur[0]));
        if (q == 0) {
            xw[slot] = xj;
            xw[slot + XW] = xj;
            if (act) ys[j] = xj;
        }
        __syncwarp();
        if (j == lo) fetch(b + PD);       // record b consumed: its slot takes b + PD
        slot = slot == 0 ? XW - 1 : slot - 1;
    }
    cp_wait<0>();
    __syncwarp();
    // ywork (now x) -> FP64 output, one system at a time, lanes over rows
    for (int t = 0; t < QSYS; ++t) {
        const int st = __shfl_sync(0xffffffffu, s, 4 * t);
        if (st < 0) continue;
        const T2 *src = yw + (long long) st * N;
        for (int i = lane; i < N; i += 32) {
            const int o = unS ? (i % unS) * unn + i / unS : i;
            double2 *dst = x + st * x_stride + o;
            const double2 v = to_z<R>(src[i]);
            if (ACCUM) { double2 u = *dst; u.x += v.x; u.y += v.y; *dst = u; }
            else *dst = v;
        }
    }
}

template <typename R, int PB, int RB>
static cudaError_t launch_quad_bwd(const GbtrsArgs &a, cplx_t<R> *yw, int grid, cudaStream_t st)
{
    using T2 = cplx_t<R>;
    const QuadBwdLayout<R, PB, RB> L(a.g);
    const size_t smem = (size_t) QSYS * L.SE * sizeof(T2) + (size_t) QSYS * PB * 8;
    auto kern = a.accumulate ? k_gbtrs_bwd_quad<R, true, PB, RB> : k_gbtrs_bwd_quad<R, false, PB, RB>;
    cudaError_t e = smem_attr((const void *) kern, smem);
    if (e != cudaSuccess) return e;
    kern<<<grid, 32, smem, st>>>(a.g, a.nsys, reinterpret_cast<const T2 *>(a.fac), a.fac_stride, yw,
                                 a.x, a.x_stride, a.sys_list, a.nlist, a.d_count, a.slot_mode,
                                 a.status, a.status_want, a.unpermute_S, a.unpermute_n);
    return cudaGetLastError();
}

template <typename R, int PF, int PB>
static cudaError_t launch_quad_d(const GbtrsArgs &a, cudaStream_t st)
{
    const int count = a.sys_list ? a.nlist : a.nsys;
    if (count == 0) return cudaSuccess;
    const int grid = (count + QSYS - 1) / QSYS;
    using T2 = cplx_t<R>;
    T2 *yw = reinterpret_cast<T2 *>(a.ywork);
    cudaError_t e;
    if (!a.fwd_done) {
        const QuadFwdLayout<R, PF> L(a.g);
        const size_t smem = (size_t) QSYS * L.SE * sizeof(T2);
        e = smem_attr((const void *) k_gbtrs_fwd_quad<R, PF>, smem);
        if (e != cudaSuccess) return e;
        k_gbtrs_fwd_quad<R, PF><<<grid, 32, smem, st>>>(a.g, a.nsys, reinterpret_cast<const T2 *>(a.fac),
                                                         a.fac_stride, a.ipiv, a.b, a.b_stride, yw,
                                                         a.sys_list, a.nlist, a.d_count, a.slot_mode,
                                                         a.status, a.status_want);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    // multi-row records where the shared memory holds them, else one row
    // (the same results either way)
    auto fits = [&](size_t se) {
        return (size_t) QSYS * se * sizeof(T2) + (size_t) QSYS * PB * 8 <= 227 * 1024;
    };
    switch (g_qbulk) {
    case 2: if (fits(QuadBwdLayout<R, PB, 2>(a.g).SE)) return launch_quad_bwd<R, PB, 2>(a, yw, grid, st); break;
    case 4: if (fits(QuadBwdLayout<R, PB, 4>(a.g).SE)) return launch_quad_bwd<R, PB, 4>(a, yw, grid, st); break;
    case 8: if (fits(QuadBwdLayout<R, PB, 8>(a.g).SE)) return launch_quad_bwd<R, PB, 8>(a, yw, grid, st); break;
    default: break;
    }
    return launch_quad_bwd<R, PB, 1>(a, yw, grid, st);
}

template <typename R, int PF>
static cudaError_t launch_quad_b(const GbtrsArgs &a, cudaStream_t st)
{
    switch (g_qdepth[1]) {
    case 4: return launch_quad_d<R, PF, 4>(a, st);
    case 8: return launch_quad_d<R, PF, 8>(a, st);
    case 16: return launch_quad_d<R, PF, 16>(a, st);
    default: return launch_quad_d<R, PF, 2>(a, st);
    }
}

template <typename R>
static cudaError_t launch_quad(const GbtrsArgs &a, cudaStream_t st)
{
    switch (g_qdepth[0]) {
    case 4: return launch_quad_b<R, 4>(a, st);
    case 8: return launch_quad_b<R, 8>(a, st);
    case 16: return launch_quad_b<R, 16>(a, st);
    default: return launch_quad_b<R, 2>(a, st);
    }
}

template <typename R>
static size_t quad_fwd_se(const FactorGeom &g)
{
    switch (g_qdepth[0]) {
    case 4: return QuadFwdLayout<R, 4>(g).SE;
    case 8: return QuadFwdLayout<R, 8>(g).SE;
    case 16: return QuadFwdLayout<R, 16>(g).SE;
    default: return QuadFwdLayout<R, 2>(g).SE;
    }
}
template <typename R, int RB>
static size_t quad_bwd_se_rb(const FactorGeom &g)
{
    switch (g_qdepth[1]) {
    case 4: return QuadBwdLayout<R, 4, RB>(g).SE;
    case 8: return QuadBwdLayout<R, 8, RB>(g).SE;
    case 16: return QuadBwdLayout<R, 16, RB>(g).SE;
    default: return QuadBwdLayout<R, 2, RB>(g).SE;
    }
}
// the one-row layout: the backward solve falls back to it when larger
// records do not fit
template <typename R>
static size_t quad_bwd_se(const FactorGeom &g) { return quad_bwd_se_rb<R, 1>(g); }

// The quad path needs a writable y buffer (nsys x N, complex of prec) and,
// when forward elimination is already done, y already in it.
static bool quad_ok(const GbtrsArgs &a)
{
    if (a.trans != 'N' || !a.ywork) return false;
    if (a.fwd_done && a.yin != a.ywork) return false;
    const size_t el = a.prec == 'Z' ? 16 : 8;
    const size_t fwd = a.prec == 'Z' ? quad_fwd_se<double>(a.g) : quad_fwd_se<float>(a.g);
    const size_t bwd = a.prec == 'Z' ? quad_bwd_se<double>(a.g) : quad_bwd_se<float>(a.g);
    return (size_t) QSYS * std::max(fwd, bwd) * el + (size_t) QSYS * 16 * 8 <= 227 * 1024;
}

template <typename R, int TRANS, bool FWD_DONE, bool ACCUM>
static cudaError_t launch_t(const GbtrsArgs &a, cudaStream_t st)
{
    constexpr int PD = gbtrs_depth<R>();
    const size_t smem = ((size_t) a.g.N + (size_t) PD * (a.g.UW() + a.g.KL)) * sizeof(cplx_t<R>)
                      + PD * sizeof(int);
    auto kern = k_gbtrs<R, TRANS, FWD_DONE, ACCUM>;
    cudaError_t e = smem_attr((const void *) kern, smem);
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
    if (quad_ok(a)) return a.prec == 'Z' ? launch_quad<double>(a, st) : launch_quad<float>(a, st);
    return a.prec == 'Z' ? launch_r<double>(a, st) : launch_r<float>(a, st);
}

}  // namespace sgb

// Tuning knob: rows per record of the backward quad solve; 0 or 1: one row
// by 16-byte cp.async, 2 (the default), 4 or 8: that many rows by one bulk
// copy (TMA).
extern "C" int sgb_gbtrs_set_quad_bulk(int rows)
{
    if (rows != 0 && rows != 1 && rows != 2 && rows != 4 && rows != 8) return -1;
    sgb::g_qbulk = rows;
    return 0;
}

// Faults recorded by kernels whose bounded waits on asynchronous copies ran
// out since the last call (0 when none); clears the record.
extern "C" int sgb_async_faults(void)
{
    int h = 0;
    if (cudaMemcpyFromSymbol(&h, sgb::g_async_fault, sizeof h) != cudaSuccess) return -1;
    if (h) {
        const int z = 0;
        cudaMemcpyToSymbol(sgb::g_async_fault, &z, sizeof z);
    }
    return h;
}

// Tuning knob: records in flight per system of the quad-lane solves
// (2, 4, 8 or 16; 0 keeps the current value).
extern "C" int sgb_gbtrs_set_quad_depth(int fwd, int bwd)
{
    if ((fwd && !sgb::quad_depth_ok(fwd)) || (bwd && !sgb::quad_depth_ok(bwd))) return -1;
    if (fwd) sgb::g_qdepth[0] = fwd;
    if (bwd) sgb::g_qdepth[1] = bwd;
    return 0;
}
