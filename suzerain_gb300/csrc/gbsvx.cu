// Batched complex128 expert band driver with the semantics of LAPACK ZGBSVX
// (the method behind suzerain_lapack_zgbsvx, suzerain/blas_et_al/lapack.c:
// 548-574, and bsmbsm_solver_zgbsvx, suzerain/bsmbsm_solver.cpp:252-291):
//
//   ZGBEQU + ZLAQGB  equilibration (fact 'E'): row and column scales R, C,
//                    EQUED in {N, R, C, B}, the scaled band and right-hand side
//   ZGBTRF           partial-pivot LU of the (scaled) band
//   ZLANGB, ZGBCON   reciprocal condition number: Higham's 1-norm estimator
//                    (ZLACN2) driving solves with the factor
//   ZGBTRS           solve
//   ZGBRFS           iterative refinement (at most five corrections) with the
//                    componentwise backward error BERR, and the forward error
//                    bound FERR from the same estimator
//   unscaling of X, FERR; INFO = N+1 when RCOND < eps; RPVGRW
//
// Every system carries its own estimator state; the host loops until every
// system's estimator is done, launching the solves for the systems that ask
// for op(A)^{-1} and those that ask for op(A)^{-H} (device status filters).
// The triangular solves inside ZGBCON are plain solves: ZLATBS's
// overflow-guarding rescale (SCALE < 1) is not reproduced, so the estimate
// matches LAPACK's whenever LAPACK's SCALE stays 1.
#include "suzerain_gb300.h"
#include "sgb_internal.h"
#include "sgb_timer.h"

#include <cctype>
#include <cmath>
#include <cstring>
#include <vector>

namespace sgb {
namespace {

constexpr double kEps = 1.1102230246251565e-16;      // dlamch('E')
constexpr double kSafmin = 2.2250738585072014e-308;  // dlamch('S')
constexpr double kPrec = 2.220446049250313e-16;      // dlamch('P')

__device__ __forceinline__ double cabs1d(double2 z) { return fabs(z.x) + fabs(z.y); }
__device__ __forceinline__ double cmod(double2 z) { return hypot(z.x, z.y); }
__device__ __forceinline__ double wmax(double v)
{
    for (int o = 16; o; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ double wmin(double v)
{
    for (int o = 16; o; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ double wsum(double v)
{
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ int wimin(int v)
{
    for (int o = 16; o; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

struct SysScal {                 // per-system scalars
    double rowcnd, colcnd, amax, anorm, rcond, rpvgrw, ferr, berr, lstres, est, estold;
    int infequ, info, count, kase, jump, j, iter;
    char equed;
};

// ZGBEQU + ZLAQGB, one warp per system.  ab: packed band rows 0..LD-1 (ld
// ldab, stride per system); out: the (scaled) copy in LD x N (ld LD), with
// zeros outside the matrix.  fact 'F' (equed_in set): EQUED comes from the
// caller, ROWCND / COLCND from the given R / C, and the band is copied as is.
__global__ void k_gbequ(int nsys, int N, int KL, int KU, const double2 *__restrict__ ab, int ldab,
                        long long stride, double2 *__restrict__ as, double *__restrict__ R,
                        double *__restrict__ C, SysScal *__restrict__ sc, bool equil,
                        const char *__restrict__ equed_in)
{
    const int s = blockIdx.x, lane = threadIdx.x;
    if (s >= nsys) return;
    const int LD = KL + KU + 1;
    const double2 *a = ab + s * stride;
    double2 *o = as + (long long) s * LD * N;
    double *r = R + (long long) s * N, *c = C + (long long) s * N;
    const double smlnum = kSafmin, bignum = 1.0 / kSafmin;
    char equed = 'N';
    int infequ = 0;
    double rowcnd = 1, colcnd = 1, amax = 0;
    if (equed_in) {
        equed = equed_in[s];
        if (equed == 'R' || equed == 'B') {
            double mn = bignum, mx = 0;
            for (int i = lane; i < N; i += 32) { mn = fmin(mn, r[i]); mx = fmax(mx, r[i]); }
            mn = wmin(mn);
            mx = wmax(mx);
            rowcnd = fmax(mn, smlnum) / fmin(mx, bignum);
        }
        if (equed == 'C' || equed == 'B') {
            double mn = bignum, mx = 0;
            for (int j = lane; j < N; j += 32) { mn = fmin(mn, c[j]); mx = fmax(mx, c[j]); }
            mn = wmin(mn);
            mx = wmax(mx);
            colcnd = fmax(mn, smlnum) / fmin(mx, bignum);
        }
    } else if (equil) {
        double rmin = bignum, rmax = 0;
        int zr = N;
        for (int i = lane; i < N; i += 32) {
            double m = 0;
            for (int j = max(0, i - KL); j <= min(N - 1, i + KU); ++j)
                m = fmax(m, cabs1d(a[KU + i - j + (long long) j * ldab]));
            r[i] = m;
            rmin = fmin(rmin, m);
            rmax = fmax(rmax, m);
            if (m == 0 && i < zr) zr = i;
        }
        rmin = wmin(rmin);
        rmax = wmax(rmax);
        zr = wimin(zr);
        amax = rmax;
        if (rmin == 0) {
            infequ = zr + 1;
        } else {
            __syncwarp();
            for (int i = lane; i < N; i += 32) r[i] = 1.0 / fmin(fmax(r[i], smlnum), bignum);
            __syncwarp();
            rowcnd = fmax(rmin, smlnum) / fmin(rmax, bignum);
            double cmin = bignum, cmax = 0;
            int zc = N;
            for (int j = lane; j < N; j += 32) {
                double m = 0;
                for (int i = max(0, j - KU); i <= min(N - 1, j + KL); ++i)
                    m = fmax(m, cabs1d(a[KU + i - j + (long long) j * ldab]) * r[i]);
                c[j] = m;
                cmin = fmin(cmin, m);
                cmax = fmax(cmax, m);
                if (m == 0 && j < zc) zc = j;
            }
            cmin = wmin(cmin);
            cmax = wmax(cmax);
            zc = wimin(zc);
            if (cmin == 0) {
                infequ = N + zc + 1;
            } else {
                for (int j = lane; j < N; j += 32) c[j] = 1.0 / fmin(fmax(c[j], smlnum), bignum);
                colcnd = fmax(cmin, smlnum) / fmin(cmax, bignum);
                // ZLAQGB: THRESH 0.1, SMALL = safe minimum / precision
                const double small = kSafmin / kPrec, large = 1.0 / small;
                if (rowcnd >= 0.1 && amax >= small && amax <= large)
                    equed = colcnd >= 0.1 ? 'N' : 'C';
                else
                    equed = colcnd >= 0.1 ? 'R' : 'B';
            }
        }
    }
    __syncwarp();
    const bool scale = !equed_in && equed != 'N';
    for (int j = lane; j < N; j += 32) {
        for (int t = 0; t < LD; ++t) {
            const int i = j - KU + t;
            double2 v = make_double2(0, 0);
            if (i >= 0 && i < N) {
                v = a[t + (long long) j * ldab];
                if (scale) {
                    double f = 1;
                    if (equed == 'C') f = c[j];
                    else if (equed == 'R') f = r[i];
                    else f = c[j] * r[i];
                    v = make_double2(f * v.x, f * v.y);
                }
            }
            o[t + (long long) j * LD] = v;
        }
    }
    if (lane == 0) {
        SysScal &q = sc[s];
        q.rowcnd = rowcnd; q.colcnd = colcnd; q.amax = amax; q.infequ = infequ; q.equed = equed;
    }
}

// Norms of the scaled band: 'M' max modulus, '1' max column sum, 'I' max row
// sum (ZLANGB, modulus).  kind 0: anorm ('1' or 'I' by onenrm); also the
// reciprocal pivot growth ZLANGB('M') / ZLANTB('M', U) over the first info
// columns when singular (ZGBSVX).
__global__ void k_norms(int nsys, int N, int KL, int KU, const double2 *__restrict__ as,
                        const double2 *__restrict__ fac, const int *__restrict__ info, bool onenrm,
                        SysScal *__restrict__ sc)
{
    const int s = blockIdx.x, lane = threadIdx.x;
    if (s >= nsys) return;
    const int LD = KL + KU + 1, UW = LD;
    const FactorGeom g{N, KL, KU};
    const double2 *a = as + (long long) s * LD * N;
    const double2 *fu = fac + s * g.fac_elems();
    const int inf = info[s];
    const int ncol = inf > 0 ? inf : N;
    double nrm = 0, amx = 0, umx = 0;
    for (int j = lane; j < N; j += 32) {
        double cs = 0;
        for (int t = 0; t < LD; ++t) {
            const int i = j - KU + t;
            if (i < 0 || i >= N) continue;
            const double m = cmod(a[t + (long long) j * LD]);
            cs += m;
            if (j < ncol) amx = fmax(amx, m);
        }
        if (onenrm) nrm = fmax(nrm, cs);
    }
    if (!onenrm)
        for (int i = lane; i < N; i += 32) {
            double rsum = 0;
            for (int j = max(0, i - KL); j <= min(N - 1, i + KU); ++j)
                rsum += cmod(a[KU + i - j + (long long) j * LD]);
            nrm = fmax(nrm, rsum);
        }
    // U: rows j < ncol, columns j..min(ncol-1, j+KL+KU)
    for (int j = lane; j < ncol; j += 32)
        for (int t = 0; t < UW && j + t < ncol; ++t) umx = fmax(umx, cmod(fu[(long long) j * UW + t]));
    nrm = wmax(nrm);
    amx = wmax(amx);
    umx = wmax(umx);
    if (lane == 0) {
        sc[s].anorm = nrm;
        sc[s].rpvgrw = umx == 0 ? 1.0 : amx / umx;
        sc[s].info = inf;
    }
}

// B scaling (ZGBSVX): notran & rowequ -> R b; trans & colequ -> C b; x = b.
__global__ void k_scale_b(int nsys, int N, const double2 *__restrict__ b, double2 *__restrict__ bs,
                          double2 *__restrict__ x, const double *__restrict__ R,
                          const double *__restrict__ C, const SysScal *__restrict__ sc,
                          const int *__restrict__ info, bool notran)
{
    const long long t = (long long) blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long) nsys * N) return;
    const int s = (int) (t / N);
    const char e = sc[s].equed;
    double f = 1;
    if (notran && (e == 'R' || e == 'B')) f = R[t];
    if (!notran && (e == 'C' || e == 'B')) f = C[t];
    double2 v = b[t];
    if (f != 1) v = make_double2(f * v.x, f * v.y);
    bs[t] = v;
    if (info[s] == 0) x[t] = v;     // a singular system's x is left as it was
}

// ZLACN2 step for every system whose kase != 0 (x holds the applied vector);
// sets kase (1: apply op, 2: apply op^H, 0: done) and x for the next apply.
// est is in sc[].est; v (the estimate's vector) in vbuf.  mode 0: ZGBCON
// (kase1 = onenrm ? 1 : 2 decides which solve is op), mode 1: ZGBRFS.
__global__ void k_lacn2(int nsys, int N, double2 *__restrict__ xb, double2 *__restrict__ vb,
                        SysScal *__restrict__ sc, int *__restrict__ kase_out)
{
    const int s = blockIdx.x, lane = threadIdx.x;
    if (s >= nsys) return;
    SysScal &q = sc[s];
    if (q.kase == 0 && q.jump != 0) { if (lane == 0) kase_out[s] = 0; return; }
    double2 *x = xb + (long long) s * N, *v = vb + (long long) s * N;
    auto dzsum1 = [&]() {
        double acc = 0;
        for (int i = lane; i < N; i += 32) acc += cmod(x[i]);
        return wsum(acc);
    };
    auto sign_x = [&]() {
        for (int i = lane; i < N; i += 32) {
            const double a = cmod(x[i]);
            x[i] = a > kSafmin ? make_double2(x[i].x / a, x[i].y / a) : make_double2(1, 0);
        }
    };
    auto izmax1 = [&]() {       // first index of the largest modulus
        double best = -1;
        int bi = N;
        for (int i = lane; i < N; i += 32) {
            const double a = cmod(x[i]);
            if (a > best) { best = a; bi = i; }
        }
        for (int o = 16; o; o >>= 1) {
            const double ob = __shfl_xor_sync(0xffffffffu, best, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
        }
        return bi;
    };
    auto unit_x = [&](int j) {
        for (int i = lane; i < N; i += 32) x[i] = make_double2(i == j ? 1.0 : 0.0, 0);
    };
    auto alt_x = [&]() {
        for (int i = lane; i < N; i += 32) {
            const double sgn = (i & 1) ? -1.0 : 1.0;
            x[i] = make_double2(sgn * (1.0 + (double) i / (double) (N - 1)), 0);
        }
    };
    int kase = 0, jump = q.jump;
    switch (jump) {
    case 0:                                       // start
        for (int i = lane; i < N; i += 32) x[i] = make_double2(1.0 / N, 0);
        kase = 1; jump = 1;
        break;
    case 1:
        if (N == 1) {
            if (lane == 0) { v[0] = x[0]; }
            q.est = cmod(x[0]);
            kase = 0; jump = -1;
            break;
        }
        q.est = dzsum1();
        __syncwarp();
        sign_x();
        kase = 2; jump = 2;
        break;
    case 2: {
        const int j = izmax1();
        q.j = j; q.iter = 2;
        __syncwarp();
        unit_x(j);
        kase = 1; jump = 3;
        break;
    }
    case 3: {
        for (int i = lane; i < N; i += 32) v[i] = x[i];
        const double estold = q.est;
        const double est = dzsum1();
        __syncwarp();
        q.estold = estold;
        q.est = est;
        if (est <= estold) {
            alt_x();
            kase = 1; jump = 5;
        } else {
            sign_x();
            kase = 2; jump = 4;
        }
        break;
    }
    case 4: {
        const int jlast = q.j;
        const int j = izmax1();
        const double a = cmod(x[jlast]), b = cmod(x[j]);
        __syncwarp();
        q.j = j;
        if (a != b && q.iter < 5) {
            q.iter += 1;
            unit_x(j);
            kase = 1; jump = 3;
        } else {
            alt_x();
            kase = 1; jump = 5;
        }
        break;
    }
    case 5: {
        const double temp = 2.0 * (dzsum1() / (3.0 * N));
        if (temp > q.est) {
            for (int i = lane; i < N; i += 32) v[i] = x[i];
            q.est = temp;
        }
        kase = 0; jump = -1;
        break;
    }
    default:
        kase = 0; jump = -1;
    }
    __syncwarp();
    if (lane == 0) { q.kase = kase; q.jump = jump; kase_out[s] = kase; }
}

// ZGBRFS residual step: r = b - op(A) x, rw = |b| + |op(A)| |x|, berr; one
// warp per system for the systems with status == want.
__global__ void k_rfs_resid(int nsys, int N, int KL, int KU, int trans,
                            const double2 *__restrict__ as, const double2 *__restrict__ bs,
                            const double2 *__restrict__ x, double2 *__restrict__ r,
                            double *__restrict__ rw, SysScal *__restrict__ sc,
                            const int *__restrict__ status, int want)
{
    const int s = blockIdx.x, lane = threadIdx.x;
    if (s >= nsys || status[s] != want) return;
    const int LD = KL + KU + 1;
    const double2 *a = as + (long long) s * LD * N;
    const double2 *xs = x + (long long) s * N, *b = bs + (long long) s * N;
    double2 *rs = r + (long long) s * N;
    double *w = rw + (long long) s * N;
    const double nz = (double) min(KL + KU + 2, N + 1);
    const double safe1 = nz * kSafmin, safe2 = safe1 / kEps;
    double berr = 0;
    for (int i = lane; i < N; i += 32) {
        double2 acc = b[i];
        double ww = cabs1d(b[i]);
        if (trans == 0) {
            for (int j = max(0, i - KL); j <= min(N - 1, i + KU); ++j) {
                const double2 aij = a[KU + i - j + (long long) j * LD];
                acc = cfnma(aij, xs[j], acc);
                ww += cabs1d(aij) * cabs1d(xs[j]);
            }
        } else {
            // row i of op(A) = column i of A
            for (int k = max(0, i - KU); k <= min(N - 1, i + KL); ++k) {
                double2 aki = a[KU + k - i + (long long) i * LD];
                if (trans == 2) aki = cconj(aki);
                acc = cfnma(aki, xs[k], acc);
                ww += cabs1d(aki) * cabs1d(xs[k]);
            }
        }
        rs[i] = acc;
        w[i] = ww;
        const double ra = cabs1d(acc);
        berr = fmax(berr, ww > safe2 ? ra / ww : (ra + safe1) / (ww + safe1));
    }
    berr = wmax(berr);
    if (lane == 0) sc[s].berr = berr;
}

// ZGBRFS decision after a residual: correct again (status 1) or stop (2).
__global__ void k_rfs_decide(int nsys, SysScal *__restrict__ sc, int *__restrict__ status,
                             int *__restrict__ nactive)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsys || status[s] != 1) return;
    SysScal &q = sc[s];
    if (q.berr > kEps && 2.0 * q.berr <= q.lstres && q.count <= 5) {
        q.lstres = q.berr;
        q.count += 1;
        atomicAdd(nactive, 1);
    } else {
        status[s] = 2;
    }
}

// FERR weights: rw = |r| + nz eps rw (+ safe1 when small); starts the estimator
__global__ void k_rfs_weights(int nsys, int N, int KL, int KU, const double2 *__restrict__ r,
                              double *__restrict__ rw, const int *__restrict__ status)
{
    const long long t = (long long) blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long) nsys * N) return;
    const int s = (int) (t / N);
    if (status[s] != 2) return;
    const double nz = (double) min(KL + KU + 2, N + 1);
    const double safe1 = nz * kSafmin, safe2 = safe1 / kEps;
    const double w = rw[t];
    rw[t] = w > safe2 ? cabs1d(r[t]) + nz * kEps * w : cabs1d(r[t]) + nz * kEps * w + safe1;
}

__global__ void k_scale_by(int nsys, int N, double2 *__restrict__ x, const double *__restrict__ w,
                           const int *__restrict__ kase, int want)
{
    const long long t = (long long) blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long) nsys * N) return;
    const int s = (int) (t / N);
    if (kase[s] != want) return;
    x[t] = make_double2(w[t] * x[t].x, w[t] * x[t].y);
}

__global__ void k_start_est(int nsys, SysScal *__restrict__ sc, const int *__restrict__ info)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsys) return;
    sc[s].kase = 0;
    sc[s].jump = (info[s] > 0 || sc[s].anorm == 0) ? -1 : 0;   // -1: skip
    sc[s].est = 0;
}

// Finish: rcond, unscaling of x and ferr, info = N+1 for rcond < eps.
__global__ void k_finish(int nsys, int N, double2 *__restrict__ x, const double *__restrict__ R,
                         const double *__restrict__ C, SysScal *__restrict__ sc, bool notran)
{
    const int s = blockIdx.x, lane = threadIdx.x;
    if (s >= nsys) return;
    SysScal &q = sc[s];
    double2 *xs = x + (long long) s * N;
    const char e = q.equed;
    const bool scale = notran ? (e == 'C' || e == 'B') : (e == 'R' || e == 'B');
    const double *f = (notran ? C : R) + (long long) s * N;
    double xmax = 0;
    for (int i = lane; i < N; i += 32) xmax = fmax(xmax, cabs1d(xs[i]));
    xmax = wmax(xmax);
    __syncwarp();
    if (q.info == 0 && scale)
        for (int i = lane; i < N; i += 32) xs[i] = make_double2(f[i] * xs[i].x, f[i] * xs[i].y);
    if (lane == 0) {
        if (q.info == 0) {
            double fe = q.ferr;
            if (xmax != 0) fe /= xmax;
            if (scale) fe /= notran ? q.colcnd : q.rowcnd;
            q.ferr = fe;
            if (q.rcond < kEps) q.info = N + 1;
        }
    }
}

// LAPACK gbtrf storage (ld ldafb >= 2KL+KU+1, U in rows 0..KL+KU, L below)
// <-> row-panel factor (U as N rows of KL+KU+1, then L as N columns of KL).
__global__ void k_afb_to_fac(int nsys, FactorGeom g, const double2 *__restrict__ afb, int ldafb,
                             long long afb_stride, double2 *__restrict__ fac)
{
    const int s = (int) (blockIdx.x / g.N), j = (int) (blockIdx.x % g.N);
    if (s >= nsys) return;
    const int KL = g.KL, UW = g.UW(), KV = UW - 1;
    const double2 *col = afb + s * afb_stride + (long long) j * ldafb;
    double2 *fu = fac + s * g.fac_elems();
    double2 *fl = fu + (long long) g.N * UW;
    for (int t = threadIdx.x; t < UW + KL; t += blockDim.x) {
        if (t < UW) {            // U(j, j+t), column j+t row KV-t
            const int jj = j + t;
            fu[(long long) j * UW + t] =
                jj < g.N ? afb[s * afb_stride + (long long) jj * ldafb + KV - t] : make_double2(0, 0);
        } else {                 // L(j+i, j), i = t-UW+1
            const int i = t - UW + 1;
            fl[(long long) j * KL + i - 1] = j + i < g.N ? col[KV + i] : make_double2(0, 0);
        }
    }
}

__global__ void k_fac_to_afb(int nsys, FactorGeom g, const double2 *__restrict__ fac,
                             double2 *__restrict__ afb, int ldafb, long long afb_stride)
{
    const int s = (int) (blockIdx.x / g.N), j = (int) (blockIdx.x % g.N);
    if (s >= nsys || (afb_stride == 0 && s > 0)) return;   // stride 0: shared
    const int KL = g.KL, UW = g.UW(), KV = UW - 1;
    const double2 *fu = fac + s * g.fac_elems();
    const double2 *fl = fu + (long long) g.N * UW;
    double2 *col = afb + s * afb_stride + (long long) j * ldafb;
    for (int r = threadIdx.x; r <= KV + KL; r += blockDim.x) {
        double2 v = make_double2(0, 0);
        if (r <= KV) {
            const int i = j - KV + r;
            if (i >= 0) v = fu[(long long) i * UW + (j - i)];
        } else if (j + r - KV < g.N) {
            v = fl[(long long) j * KL + r - KV - 1];
        }
        col[r] = v;
    }
}

// Scaled band (LD x N) back into the caller's band storage, in-matrix
// entries only.
__global__ void k_band_back(int nsys, int N, int KL, int KU, const double2 *__restrict__ as,
                            double2 *__restrict__ ab, int ldab, long long stride)
{
    const int s = (int) (blockIdx.x / N), j = (int) (blockIdx.x % N);
    if (s >= nsys || (stride == 0 && s > 0)) return;   // stride 0: one shared band
    const int LD = KL + KU + 1;
    for (int t = threadIdx.x; t < LD; t += blockDim.x) {
        const int i = j - KU + t;
        if (i >= 0 && i < N)
            ab[s * stride + (long long) j * ldab + t] = as[((long long) s * N + j) * LD + t];
    }
}

}  // namespace

// Host driver (see GbsvxArgs).  Host synchronizations: one per estimator
// step and per refinement step (the loops end when no system asks for
// more), as LAPACK's reverse-communication estimator needs.
int zgbsvx_batched(const GbsvxArgs &A, cudaStream_t st)
{
    const int nsys = A.nsys, N = A.g.N, KL = A.g.KL, KU = A.g.KU;
    const char fact = A.fact, trans = A.trans;
    const bool equil = fact == 'E', notran = trans == 'N', given = fact == 'F';
    const int tcode = trans == 'N' ? 0 : (trans == 'T' ? 1 : 2);
    const int LD = KL + KU + 1;
    const FactorGeom g = A.g;
    const size_t vec = (size_t) nsys * N;
    if (nsys == 0) return 0;
    std::vector<void *> tmp;
    auto take = [&](size_t bytes) -> void * {
        void *p = nullptr;
        if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
        tmp.push_back(p);
        return p;
    };
    auto cleanup = [&]() { for (void *p : tmp) cudaFree(p); tmp.clear(); };
#define GX_TRY(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { cleanup(); return sgb_set_error(e_, #x, __FILE__, __LINE__); } } while (0)
    SysScal *sc = (SysScal *) take(nsys * sizeof(SysScal));
    double2 *as = (double2 *) take(vec * LD * sizeof(double2));
    double2 *bs = (double2 *) take(vec * sizeof(double2));
    double2 *fac = (double2 *) take((size_t) nsys * g.fac_elems() * sizeof(double2));
    double2 *r = (double2 *) take(vec * sizeof(double2));
    double2 *xe = (double2 *) take(vec * sizeof(double2));
    double2 *ve = (double2 *) take(vec * sizeof(double2));
    double *rw = (double *) take(vec * sizeof(double));
    int *status = (int *) take(nsys * sizeof(int));
    int *kase = (int *) take(nsys * sizeof(int));
    int *cnt = (int *) take(sizeof(int));
    if (tmp.size() != 11 || !sc || !as || !bs || !fac || !r || !xe || !ve || !rw || !status ||
        !kase || !cnt) {
        cleanup();
        return sgb_set_error(cudaErrorMemoryAllocation, "zgbsvx_batched workspace", __FILE__, __LINE__);
    }
    const unsigned EB = (unsigned) ((vec + 255) / 256);
    const int T = 128, B = (nsys + T - 1) / T;
    const unsigned cg = (unsigned) ((size_t) nsys * N);   // one block per column

    // equilibration (or the given one) and the scaled copy of the band
    count_launch(1);
    k_gbequ<<<nsys, 32, 0, st>>>(nsys, N, KL, KU, A.ab, A.ldab, A.ab_stride, as, A.R, A.C, sc,
                                 equil, given ? A.equed : nullptr);
    GX_TRY(cudaGetLastError());
    if (given) {
        count_launch(1);
        k_afb_to_fac<<<cg, 64, 0, st>>>(nsys, g, A.afb, A.ldafb, A.afb_stride, fac);
        GX_TRY(cudaGetLastError());
        GX_TRY(cudaMemsetAsync(A.info, 0, nsys * sizeof(int), st));
    } else {
        GbtrfArgs fa;
        fa.prec = 'Z'; fa.g = g; fa.nsys = nsys;
        fa.src = {as, (long long) LD * N, LD, 0};
        fa.fac = fac; fa.fac_stride = g.fac_elems(); fa.ipiv = A.ipiv; fa.info = A.info;
        count_launch(1);
        GX_TRY(launch_gbtrf(fa, st));
    }
    count_launch(2);
    k_norms<<<nsys, 32, 0, st>>>(nsys, N, KL, KU, as, fac, A.info, notran, sc);
    GX_TRY(cudaGetLastError());
    k_scale_b<<<EB, 256, 0, st>>>(nsys, N, A.b, bs, A.x, A.R, A.C, sc, A.info, notran);
    GX_TRY(cudaGetLastError());

    // one solve per estimator request: op(A)^{-1} or op(A)^{-H} per system
    auto apply = [&](char tr, int want) -> cudaError_t {
        GbtrsArgs a;
        a.prec = 'Z'; a.trans = tr; a.g = g; a.nsys = nsys; a.fac = fac;
        a.fac_stride = g.fac_elems(); a.ipiv = A.ipiv; a.b = xe; a.b_stride = N;
        a.x = xe; a.x_stride = N; a.status = kase; a.status_want = want;
        count_launch(1);
        return launch_gbtrs(a, st);
    };
    std::vector<int> hk(nsys);
    auto estimate = [&](auto do_apply) -> cudaError_t {
        for (int round = 0; round < 16; ++round) {
            count_launch(1);
            k_lacn2<<<nsys, 32, 0, st>>>(nsys, N, xe, ve, sc, kase);
            cudaError_t e = cudaGetLastError();
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(hk.data(), kase, nsys * sizeof(int), cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) return e;
            bool any = false;
            for (int k : hk) any |= k != 0;
            if (!any) break;
            e = do_apply();
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    };
    std::vector<SysScal> hs(nsys);
    auto pull = [&]() -> cudaError_t {
        cudaError_t e = cudaMemcpyAsync(hs.data(), sc, nsys * sizeof(SysScal), cudaMemcpyDeviceToHost, st);
        return e == cudaSuccess ? cudaStreamSynchronize(st) : e;
    };
    auto push = [&]() {
        return cudaMemcpyAsync(sc, hs.data(), nsys * sizeof(SysScal), cudaMemcpyHostToDevice, st);
    };

    // ZGBCON: ||A^{-1}|| in the norm of op (1-norm for 'N', infinity-norm
    // otherwise); the estimator's kase 1 applies A^{-1} for the 1-norm and
    // A^{-H} for the infinity-norm
    count_launch(1);
    k_start_est<<<B, T, 0, st>>>(nsys, sc, A.info);
    GX_TRY(cudaGetLastError());
    {
        const char op1 = notran ? 'N' : 'C', op2 = notran ? 'C' : 'N';
        GX_TRY(estimate([&]() -> cudaError_t {
            cudaError_t e = apply(op1, 1);
            return e != cudaSuccess ? e : apply(op2, 2);
        }));
    }
    GX_TRY(pull());
    std::vector<int> hst(nsys);
    for (int s = 0; s < nsys; ++s) {
        SysScal &q = hs[s];
        q.rcond = (q.info > 0 || q.anorm == 0 || q.est == 0) ? 0.0 : (1.0 / q.est) / q.anorm;
        q.ferr = 0; q.berr = 0; q.count = 1; q.lstres = 3.0;
        hst[s] = q.info > 0 ? 3 : 1;      // 1: solve and refine, 3: singular
    }
    GX_TRY(push());
    GX_TRY(cudaMemcpyAsync(status, hst.data(), nsys * sizeof(int), cudaMemcpyHostToDevice, st));
    {
        GbtrsArgs a;
        a.prec = 'Z'; a.trans = trans; a.g = g; a.nsys = nsys; a.fac = fac;
        a.fac_stride = g.fac_elems(); a.ipiv = A.ipiv; a.b = A.x; a.b_stride = N; a.x = A.x;
        a.x_stride = N; a.status = status; a.status_want = 1;
        count_launch(1);
        GX_TRY(launch_gbtrs(a, st));
    }
    // ZGBRFS: residual, BERR, and at most five corrections
    for (int it = 0; it <= 5; ++it) {
        count_launch(2);
        k_rfs_resid<<<nsys, 32, 0, st>>>(nsys, N, KL, KU, tcode, as, bs, A.x, r, rw, sc, status, 1);
        GX_TRY(cudaGetLastError());
        GX_TRY(cudaMemsetAsync(cnt, 0, sizeof(int), st));
        k_rfs_decide<<<B, T, 0, st>>>(nsys, sc, status, cnt);
        GX_TRY(cudaGetLastError());
        int h = 0;
        GX_TRY(cudaMemcpyAsync(&h, cnt, sizeof(int), cudaMemcpyDeviceToHost, st));
        GX_TRY(cudaStreamSynchronize(st));
        if (h == 0) break;
        GbtrsArgs a;
        a.prec = 'Z'; a.trans = trans; a.g = g; a.nsys = nsys; a.fac = fac;
        a.fac_stride = g.fac_elems(); a.ipiv = A.ipiv; a.b = r; a.b_stride = N; a.x = A.x;
        a.x_stride = N; a.accumulate = true; a.status = status; a.status_want = 1;
        count_launch(1);
        GX_TRY(launch_gbtrs(a, st));
    }
    // FERR: the estimator on diag(rw) inv(op(A)^H) (kase 1) and
    // inv(op(A)) diag(rw) (kase 2)
    count_launch(1);
    k_rfs_weights<<<EB, 256, 0, st>>>(nsys, N, KL, KU, r, rw, status);
    GX_TRY(cudaGetLastError());
    GX_TRY(pull());
    for (auto &q : hs) { q.jump = q.info > 0 ? -1 : 0; q.kase = 0; q.est = 0; }
    GX_TRY(push());
    {
        const char tn = notran ? 'N' : 'C', tt = notran ? 'C' : 'N';
        GX_TRY(estimate([&]() -> cudaError_t {
            cudaError_t e = apply(tt, 1);
            if (e != cudaSuccess) return e;
            count_launch(2);
            k_scale_by<<<EB, 256, 0, st>>>(nsys, N, xe, rw, kase, 1);
            k_scale_by<<<EB, 256, 0, st>>>(nsys, N, xe, rw, kase, 2);
            e = cudaGetLastError();
            return e != cudaSuccess ? e : apply(tn, 2);
        }));
    }
    GX_TRY(pull());
    for (auto &q : hs) q.ferr = q.est;
    GX_TRY(push());
    count_launch(1);
    k_finish<<<nsys, 32, 0, st>>>(nsys, N, A.x, A.R, A.C, sc, notran);
    GX_TRY(cudaGetLastError());
    // outputs: scaled band and b, the factor in LAPACK storage, scalars
    count_launch(2);
    k_band_back<<<cg, 64, 0, st>>>(nsys, N, KL, KU, as, A.ab_out, A.ldab, A.ab_stride);
    GX_TRY(cudaGetLastError());
    GX_TRY(cudaMemcpyAsync(A.b_out, bs, vec * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    if (!given && A.afb) {
        k_fac_to_afb<<<cg, 64, 0, st>>>(nsys, g, fac, A.afb, A.ldafb, A.afb_stride);
        GX_TRY(cudaGetLastError());
    }
    GX_TRY(pull());
    {
        std::vector<char> he(nsys);
        std::vector<double> h1(nsys), h2(nsys), h3(nsys), h4(nsys);
        std::vector<int> hi(nsys);
        for (int s = 0; s < nsys; ++s) {
            he[s] = hs[s].equed; h1[s] = hs[s].rcond; h2[s] = hs[s].ferr; h3[s] = hs[s].berr;
            h4[s] = hs[s].rpvgrw; hi[s] = hs[s].info;
        }
        auto put = [&](void *dst, const void *src, size_t bytes) -> cudaError_t {
            if (!dst) return cudaSuccess;
            return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, st);
        };
        GX_TRY(put(A.equed, he.data(), nsys));
        GX_TRY(put(A.rcond, h1.data(), nsys * sizeof(double)));
        GX_TRY(put(A.ferr, h2.data(), nsys * sizeof(double)));
        GX_TRY(put(A.berr, h3.data(), nsys * sizeof(double)));
        GX_TRY(put(A.rpvgrw, h4.data(), nsys * sizeof(double)));
        GX_TRY(put(A.info, hi.data(), nsys * sizeof(int)));
        GX_TRY(cudaStreamSynchronize(st));
    }
    cleanup();
#undef GX_TRY
    return 0;
}

// ZGBCON alone: the reciprocal condition number in the 1-norm (norm '1' or
// 'O') or the infinity-norm ('I') from a factor in LAPACK gbtrf storage
// (device afb, ipiv) and the norm of the unfactored matrix (host anorm, one
// per system); rcond out on the host.  The same estimator loop as the
// expert driver's condition estimate.
int zgbcon_batched(char norm, int nsys, const FactorGeom &g, const double2 *afb, int ldafb,
                   long long afb_stride, const int *ipiv, const double *anorm, double *rcond,
                   cudaStream_t st)
{
    const int N = g.N;
    if (nsys == 0) return 0;
    const bool onenrm = norm == '1' || norm == 'O';
    const size_t vec = (size_t) nsys * N;
    std::vector<void *> tmp;
    auto take = [&](size_t bytes) -> void * {
        void *p = nullptr;
        if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
        tmp.push_back(p);
        return p;
    };
    auto cleanup = [&]() { for (void *p : tmp) cudaFree(p); tmp.clear(); };
#define GC_TRY(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { cleanup(); return sgb_set_error(e_, #x, __FILE__, __LINE__); } } while (0)
    SysScal *sc = (SysScal *) take(nsys * sizeof(SysScal));
    double2 *fac = (double2 *) take((size_t) nsys * g.fac_elems() * sizeof(double2));
    double2 *xe = (double2 *) take(vec * sizeof(double2));
    double2 *ve = (double2 *) take(vec * sizeof(double2));
    int *kase = (int *) take(nsys * sizeof(int));
    int *info = (int *) take(nsys * sizeof(int));
    if (tmp.size() != 6) {
        cleanup();
        return sgb_set_error(cudaErrorMemoryAllocation, "zgbcon_batched workspace", __FILE__, __LINE__);
    }
    std::vector<SysScal> hs(nsys);
    std::memset(hs.data(), 0, nsys * sizeof(SysScal));
    for (int s = 0; s < nsys; ++s) hs[s].anorm = anorm[s];
    GC_TRY(cudaMemcpyAsync(sc, hs.data(), nsys * sizeof(SysScal), cudaMemcpyHostToDevice, st));
    GC_TRY(cudaMemsetAsync(info, 0, nsys * sizeof(int), st));
    const unsigned cg = (unsigned) ((size_t) nsys * N);
    count_launch(2);
    k_afb_to_fac<<<cg, 64, 0, st>>>(nsys, g, afb, ldafb, afb_stride, fac);
    GC_TRY(cudaGetLastError());
    const int T = 128, B = (nsys + T - 1) / T;
    k_start_est<<<B, T, 0, st>>>(nsys, sc, info);
    GC_TRY(cudaGetLastError());
    auto apply = [&](char tr, int want) -> cudaError_t {
        GbtrsArgs a;
        a.prec = 'Z'; a.trans = tr; a.g = g; a.nsys = nsys; a.fac = fac;
        a.fac_stride = g.fac_elems(); a.ipiv = ipiv; a.b = xe; a.b_stride = N;
        a.x = xe; a.x_stride = N; a.status = kase; a.status_want = want;
        count_launch(1);
        return launch_gbtrs(a, st);
    };
    // kase 1 applies A^{-1} for the 1-norm and A^{-H} for the infinity-norm
    const char op1 = onenrm ? 'N' : 'C', op2 = onenrm ? 'C' : 'N';
    std::vector<int> hk(nsys);
    for (int round = 0; round < 16; ++round) {
        count_launch(1);
        k_lacn2<<<nsys, 32, 0, st>>>(nsys, N, xe, ve, sc, kase);
        GC_TRY(cudaGetLastError());
        GC_TRY(cudaMemcpyAsync(hk.data(), kase, nsys * sizeof(int), cudaMemcpyDeviceToHost, st));
        GC_TRY(cudaStreamSynchronize(st));
        bool any = false;
        for (int k : hk) any |= k != 0;
        if (!any) break;
        GC_TRY(apply(op1, 1));
        GC_TRY(apply(op2, 2));
    }
    GC_TRY(cudaMemcpyAsync(hs.data(), sc, nsys * sizeof(SysScal), cudaMemcpyDeviceToHost, st));
    GC_TRY(cudaStreamSynchronize(st));
    for (int s = 0; s < nsys; ++s)
        rcond[s] = (anorm[s] == 0 || hs[s].est == 0) ? 0.0 : (1.0 / hs[s].est) / anorm[s];
    cleanup();
#undef GC_TRY
    return 0;
}

}  // namespace sgb

using namespace sgb;

// LAPACK ZGBCON (the routine suzerain_lapack_zgbcon forwards to,
// suzerain/blas_et_al/lapack.c): argument errors as LAPACK's -i, n = 0 gives
// rcond 1, anorm = 0 gives 0.  ab is the gbtrf factor (ld >= 2 kl + ku + 1),
// host or device; work and rwork are not used.
extern "C" int suzerain_lapack_zgbcon(const char norm_in, const int n, const int kl, const int ku,
                                      const sgb_complex_double *ab, const int ldab,
                                      const int *ipiv, const double anorm, double *rcond,
                                      sgb_complex_double *work, double *rwork)
{
    (void) work; (void) rwork;
    const char norm = (char) std::toupper((unsigned char) norm_in);
    if (norm != '1' && norm != 'O' && norm != 'I') return -1;
    if (n < 0) return -2;
    if (kl < 0) return -3;
    if (ku < 0) return -4;
    if (ldab < 2 * kl + ku + 1) return -6;
    if (anorm < 0) return -8;
    if (!rcond) return -9;
    *rcond = 0;
    if (n == 0) { *rcond = 1; return 0; }
    if (anorm == 0) return 0;
    if (kl + 1 > 64 || kl + ku + 1 > 192)
        return sgb_set_error(cudaErrorNotSupported, "suzerain_lapack_zgbcon: bandwidth beyond KL < 64, KL + KU < 192", __FILE__, __LINE__);
    const size_t fb = (size_t) ldab * n * sizeof(double2), pb = (size_t) n * sizeof(int);
    void *dab = nullptr, *dpv = nullptr;
    cudaPointerAttributes at;
    const bool dev_ab = cudaPointerGetAttributes(&at, ab) == cudaSuccess &&
                        (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged);
    cudaGetLastError();
    const bool dev_pv = cudaPointerGetAttributes(&at, ipiv) == cudaSuccess &&
                        (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged);
    cudaGetLastError();
    cudaError_t e = cudaSuccess;
    if (dev_ab) dab = (void *) ab;
    else if ((e = cudaMalloc(&dab, fb)) == cudaSuccess) e = cudaMemcpy(dab, ab, fb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        if (dev_pv) dpv = (void *) ipiv;
        else if ((e = cudaMalloc(&dpv, pb)) == cudaSuccess) e = cudaMemcpy(dpv, ipiv, pb, cudaMemcpyHostToDevice);
    }
    int rc = 0;
    if (e == cudaSuccess)
        rc = zgbcon_batched(norm, 1, FactorGeom{n, kl, ku}, (const double2 *) dab, ldab,
                            (long long) ldab * n, (const int *) dpv, &anorm, rcond, 0);
    if (!dev_ab && dab) cudaFree(dab);
    if (!dev_pv && dpv) cudaFree(dpv);
    if (e != cudaSuccess) return sgb_set_error(e, "suzerain_lapack_zgbcon", __FILE__, __LINE__);
    return rc;
}

extern "C" int sgb_zgbsvx_batched(char fact, char trans, int nsys, int n, int kl, int ku,
                                  sgb_complex_double *ab, int ldab, long long ab_stride,
                                  sgb_complex_double *afb, int ldafb, long long afb_stride,
                                  int *ipiv, char *equed, double *r, double *c,
                                  sgb_complex_double *b, sgb_complex_double *x, double *rcond,
                                  double *ferr, double *berr, double *rpvgrw, int *info,
                                  void *stream)
{
    fact = (char) std::toupper((unsigned char) fact);
    trans = (char) std::toupper((unsigned char) trans);
    if (fact != 'N' && fact != 'E' && fact != 'F') return -1;
    if (trans != 'N' && trans != 'T' && trans != 'C') return -2;
    if (nsys < 0) return -3;
    if (n < 1 || kl < 0 || ku < 0 || kl + 1 > 64 || kl + ku + 1 > 192) return -4;
    if (ldab < kl + ku + 1 || ab_stride < (long long) ldab * n) return -8;
    if ((afb || fact == 'F') && (ldafb < 2 * kl + ku + 1 || afb_stride < (long long) ldafb * n))
        return -11;
    if (!ab || !ipiv || !equed || !r || !c || !b || !x || !info || (fact == 'F' && !afb)) return -7;
    GbsvxArgs A;
    A.nsys = nsys; A.fact = fact; A.trans = trans; A.g = {n, kl, ku};
    A.ab = (const double2 *) ab; A.ab_out = (double2 *) ab; A.ldab = ldab; A.ab_stride = ab_stride;
    A.afb = (double2 *) afb; A.ldafb = ldafb; A.afb_stride = afb_stride;
    A.ipiv = ipiv; A.equed = equed; A.R = r; A.C = c;
    A.b = (const double2 *) b; A.b_out = (double2 *) b; A.x = (double2 *) x;
    A.rcond = rcond; A.ferr = ferr; A.berr = berr; A.rpvgrw = rpvgrw; A.info = info;
    return zgbsvx_batched(A, (cudaStream_t) stream);
}
