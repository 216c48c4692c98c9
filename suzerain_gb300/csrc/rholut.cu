// The production implicit operator of the perfect-gas formulation,
// M + phi L with L the linearisation about wall-normal reference profiles
// (suzerain/rholut_imexop.h, suzerain/rholut_imexop.def:41-594,
// suzerain/rholut_imexop.c:43-545), on the GPU:
//
//   * packc / packf: P (M + phi L)^T P^T as a packed complex128 band for
//     many wavenumber pairs at once, one warp per band column;
//   * accumulate: y <- (M + phi L) x + beta y, one warp per output element,
//     each entry of the operator formed on the fly (nothing assembled);
//   * the Giles non-reflecting upper boundary (the a, b, c 5 x 5 matrices)
//     as a correction of the last 15 x 5 block of the transpose.
//
// Every block of the operator is a sum over the collocation operators
// D_d (d = 0, 1, 2: M, D1, D2) right-scaled by a complex column factor
// t_{ij,d}(q) = sum over terms of coefficient(km, kn) x reference profile(q):
// entry (p, q) of block (i, j) of the transpose = sum_d D_d^T(p, q) t_d(q),
// then scaled by phi (mass added on the diagonal blocks).  rholut_terms
// below is that table, one case per block.
#include "suzerain_gb300.h"
#include "sgb_internal.h"
#include "sgb_timer.h"

#include <cctype>
#include <complex>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

using namespace sgb;

namespace {

// Reference profiles in the order of suzerain_rholut_imexop_ref's members.
enum Prof {
    UX, UY, UZ, U2, UXUX, UXUY, UXUZ, UYUY, UYUZ, UZUZ, NU, NUUX, NUUY, NUUZ, NUU2,
    NUUXUX, NUUXUY, NUUXUZ, NUUYUY, NUUYUZ, NUUZUZ, EX_GRADRHO, EY_GRADRHO, EZ_GRADRHO,
    E_DIVM, E_DELTARHO, NPROF
};
static_assert(sizeof(suzerain_rholut_imexop_ref) == NPROF * sizeof(double *),
              "profile table matches suzerain_rholut_imexop_ref");
static_assert(sizeof(suzerain_rholut_imexop_refld) == NPROF * sizeof(int),
              "stride table matches suzerain_rholut_imexop_refld");

// Equations in the reference's naming: E (total energy), u, v, w (momentum),
// rho (density).
enum Eq { EE = 0, EU = 1, EV = 2, EW = 3, ER = 4 };

}  // namespace

struct RholutDev {
    int n, kl, ku, ld;          // the workspace's max_kl / max_ku view of D_d^T
    int S;                      // equations present
    int ord[5], inv[5];         // ord[eq]: packed position or -1; inv[pos]: equation
    const double *band;         // 3 x ld x n: M^T, D1^T, D2^T
    const double *prof;         // NPROF x n
    const double *nrbc;         // a, b, c (5 x 5 column-major each) or null
    int has_a, has_b, has_c;
    double gm1, gm3, ap43, ap13, Ma2, invRe, invMa2, ginvPr, ginvRePr, gamma;
};

struct sgb_rholut {
    RholutDev d{};
    void *mem = nullptr;        // band + prof + nrbc, one allocation
};

namespace {

struct Z { double re, im; };
__device__ __forceinline__ Z zmk(double r, double i) { return Z{r, i}; }
__device__ __forceinline__ Z zadd(Z a, Z b) { return Z{a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ Z zmul(Z a, Z b)
{ return Z{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
__device__ __forceinline__ Z zscale(Z a, double s) { return Z{a.re * s, a.im * s}; }

// Column factors of block (i, j) (operator row equation i, input equation
// j) at point q: up to four passes (d, t) applied in order, and the finish
// kind: 0 zero block, 1 alpha times the sum, 2 the sum times phi plus M
// (the diagonal blocks of E, u, v, w: mass accumulated last).  The
// coefficients are suzerain/rholut_imexop.def:96-491's.
struct Passes {
    int np = 0;
    int d[4];
    Z t[4];
    int kind = 1;
    Z alpha;
};

__device__ void rholut_terms(const RholutDev &h, int i, int j, int q, double km, double kn,
                             Z phi, Passes &P)
{
    const double *pr = h.prof;
    const int n = h.n;
    auto R = [&](int k) { return pr[k * n + q]; };
    const Z ikm = zmk(0, km), ikn = zmk(0, kn);
    const double km2 = km * km, kn2 = kn * kn;
    const double gm1 = h.gm1, gm3 = h.gm3, ap43 = h.ap43, ap13 = h.ap13, Ma2 = h.Ma2,
                 invRe = h.invRe, invMa2 = h.invMa2, ginvPr = h.ginvPr, ginvRePr = h.ginvRePr,
                 g = h.gamma;
    auto add = [&](int d, Z t) { P.d[P.np] = d; P.t[P.np] = t; ++P.np; };
    P.np = 0;
    P.kind = 1;
    P.alpha = phi;
    if (i == EE) {
        if (j == EE) {
            P.kind = 2;
            add(0, zadd(zadd(zscale(zmul(zmk(-g, 0), ikm), R(UX)), zscale(zmul(zmk(-g, 0), ikn), R(UZ))),
                        zmk(-ginvRePr * (km2 + kn2) * R(NU), 0)));
            add(1, zmk(-g * R(UY), 0));
            add(2, zmk(ginvRePr * R(NU), 0));
        } else if (j == EU) {
            const double c_nuux = Ma2 * invRe * ((ginvPr - ap43) * km2 + (ginvPr - 1) * kn2);
            add(0, zadd(zmk(c_nuux * R(NUUX) + (-Ma2 * invRe * ap13 * km * kn) * R(NUUZ), 0),
                        zscale(zmk(0, -km), R(E_DIVM))));
            add(1, zscale(zmk(0, Ma2 * invRe * ap13 * km), R(NUUY)));
            add(2, zmk(Ma2 * invRe * (1 - ginvPr) * R(NUUX), 0));
        } else if (j == EV) {
            const double c_nuuy = Ma2 * invRe * (ginvPr - 1) * (km2 + kn2);
            add(0, zmk(c_nuuy * R(NUUY), 0));
            add(1, zadd(zadd(zscale(zmk(0, Ma2 * invRe * ap13 * km), R(NUUX)),
                             zscale(zmk(0, Ma2 * invRe * ap13 * kn), R(NUUZ))),
                        zmk(-R(E_DIVM), 0)));
            add(2, zmk(Ma2 * invRe * (ap43 - ginvPr) * R(NUUY), 0));
        } else if (j == EW) {
            const double c_nuuz = Ma2 * invRe * ((ginvPr - 1) * km2 + (ginvPr - ap43) * kn2);
            add(0, zadd(zmk((-Ma2 * invRe * ap13 * km * kn) * R(NUUX) + c_nuuz * R(NUUZ), 0),
                        zscale(zmk(0, -kn), R(E_DIVM))));
            add(1, zscale(zmk(0, Ma2 * invRe * ap13 * kn), R(NUUY)));
            add(2, zmk(Ma2 * invRe * (1 - ginvPr) * R(NUUZ), 0));
        } else {  // rho: the mass terms in two passes, as the reference
            add(0, zmk(Ma2 * invRe * (km2 + kn2) * R(NUU2) + Ma2 * invRe * ap13 * km2 * R(NUUXUX)
                       + Ma2 * invRe * ap13 * 2 * km * kn * R(NUUXUZ)
                       + Ma2 * invRe * ap13 * kn2 * R(NUUZUZ), 0));
            add(0, zadd(zadd(zscale(zmk(0, -km), R(EX_GRADRHO)), zscale(zmk(0, -kn), R(EZ_GRADRHO))),
                        zmk(-ginvRePr / gm1 * (km2 + kn2) * R(E_DELTARHO), 0)));
            add(1, zadd(zadd(zscale(zmk(0, -Ma2 * invRe * ap13 * 2 * km), R(NUUXUY)),
                             zscale(zmk(0, -Ma2 * invRe * ap13 * 2 * kn), R(NUUYUZ))),
                        zmk(-R(EY_GRADRHO), 0)));
            add(2, zmk(-Ma2 * invRe * R(NUU2) - Ma2 * invRe * ap13 * R(NUUYUY)
                       + ginvRePr / gm1 * R(E_DELTARHO), 0));
        }
    } else if (i == EU || i == EW) {
        // u and w rows are mirror images under (km, ux) <-> (kn, uz)
        const bool U = (i == EU);
        const double ka = U ? km : kn, kb = U ? kn : km, ka2 = ka * ka, kb2 = kb * kb;
        const int PA = U ? UX : UZ, PB = U ? UZ : UX;                  // along, across
        const int PAA = U ? UXUX : UZUZ, PAB = UXUZ, PAY = U ? UXUY : UYUZ;
        const int NA = U ? NUUX : NUUZ, NB = U ? NUUZ : NUUX;
        const Z ika = U ? ikm : ikn, ikb = U ? ikn : ikm;
        if (j == EE) {
            add(0, zscale(ika, -gm1 * invMa2));
        } else if (j == i) {
            P.kind = 2;
            add(0, zadd(zadd(zscale(zmul(zmk(gm3, 0), ika), R(PA)), zscale(zmk(-ikb.re, -ikb.im), R(PB))),
                        zmk(-invRe * (ap43 * ka2 + kb2) * R(NU), 0)));
            add(1, zmk(-R(UY), 0));
            add(2, zmk(invRe * R(NU), 0));
        } else if (j == EV) {
            add(0, zscale(zscale(ika, gm1), R(UY)));
            add(1, zadd(zmk(-R(PA), 0), zscale(zmk(0, ap13 * invRe * ka), R(NU))));
        } else if (j == (U ? EW : EU)) {
            add(0, zadd(zadd(zscale(zscale(ika, gm1), R(PB)), zscale(zmk(-ikb.re, -ikb.im), R(PA))),
                        zmk(-ap13 * invRe * km * kn * R(NU), 0)));
        } else {  // rho
            add(0, zadd(zadd(zadd(zscale(zscale(ika, -0.5 * gm1), R(U2)), zscale(ikm, R(U ? PAA : PAB))),
                             zscale(ikn, R(U ? PAB : PAA))),
                        zmk(invRe * (ap43 * ka2 + kb2) * R(NA) + ap13 * invRe * km * kn * R(NB), 0)));
            add(1, zadd(zmk(R(PAY), 0), zscale(zmk(0, -ap13 * invRe * ka), R(NUUY))));
            add(2, zmk(-invRe * R(NA), 0));
        }
    } else if (i == EV) {
        if (j == EE) {
            add(1, zmk(-gm1 * invMa2, 0));
        } else if (j == EU || j == EW) {
            const bool U = (j == EU);
            const double ka = U ? km : kn;
            add(0, zscale(zmk(0, -ka), R(UY)));
            add(1, zadd(zmk(gm1 * R(U ? UX : UZ), 0), zscale(zmk(0, ap13 * invRe * ka), R(NU))));
        } else if (j == EV) {
            P.kind = 2;
            add(0, zadd(zadd(zscale(zmk(0, -km), R(UX)), zscale(zmk(0, -kn), R(UZ))),
                        zmk(-invRe * (km2 + kn2) * R(NU), 0)));
            add(1, zmk(gm3 * R(UY), 0));
            add(2, zmk(ap43 * invRe * R(NU), 0));
        } else {  // rho
            add(0, zadd(zadd(zscale(ikm, R(UXUY)), zscale(ikn, R(UYUZ))),
                        zmk(invRe * (km2 + kn2) * R(NUUY), 0)));
            add(1, zadd(zadd(zmk(-0.5 * gm1 * R(U2) + R(UYUY), 0),
                             zscale(zmk(0, -ap13 * invRe * km), R(NUUX))),
                        zscale(zmk(0, -ap13 * invRe * kn), R(NUUZ))));
            add(2, zmk(-ap43 * invRe * R(NUUY), 0));
        }
    } else {  // density row: scaled collocation operators, no profiles
        if (j == EE) { P.kind = 0; return; }
        P.alpha = zmk(1, 0);
        if (j == EU) add(0, zmul(zmk(-phi.re, -phi.im), ikm));
        else if (j == EV) add(1, zmk(-phi.re, -phi.im));
        else if (j == EW) add(0, zmul(zmk(-phi.re, -phi.im), ikn));
        else add(0, zmk(1, 0));
    }
}

// Entry (p, q) of the block whose column factors are P (p, q points).
__device__ __forceinline__ Z rholut_apply(const RholutDev &h, const Passes &P, int p, int q, Z phi)
{
    const int dp = p - q;
    if (P.kind == 0 || dp > h.kl || -dp > h.ku) return zmk(0, 0);
    const long long k = (long long) h.ku + dp + (long long) q * h.ld;
    const long long bs = (long long) h.ld * h.n;
    Z b = zmk(0, 0);
    for (int t = 0; t < P.np; ++t) b = zadd(b, zscale(P.t[t], h.band[P.d[t] * bs + k]));
    if (P.kind == 2) return zadd(zmul(b, phi), zmk(h.band[k], 0));
    return zmul(P.alpha, b);
}

// Unmodified entry (R, C) of P (M + phi L)^T P^T (global permuted indices).
__device__ Z rholut_entry(const RholutDev &h, int R, int C, double km, double kn, Z phi)
{
    const int S = h.S;
    const int p = R / S, q = C / S;
    const int dp = p - q;
    if (dp > h.kl || -dp > h.ku) return zmk(0, 0);
    Passes P;
    rholut_terms(h, h.inv[C - q * S], h.inv[R - p * S], q, km, kn, phi, P);
    return rholut_apply(h, P, p, q, phi);
}

// The column factors of column C's S blocks (one per row equation), made by
// lanes 0..S-1 of the warp into the warp's table.
__device__ __forceinline__ void rholut_column_terms(const RholutDev &h, int C, double km, double kn,
                                                    Z phi, int lane, Passes *tab)
{
    const int q = C / h.S;
    if (lane < h.S) rholut_terms(h, h.inv[C - q * h.S], h.inv[lane], q, km, kn, phi, tab[lane]);
    __syncwarp();
}

// The 15 x 5 block X of the transpose at rows 5(n-3).., columns 5(n-1)..
// after the non-reflecting boundary correction (suzerain/rholut_imexop.def:
// 496-594): X + X (-C^T) + [0; C^T - i km phi A^T - i kn phi B^T].
__device__ Z rholut_nrbc_delta(const RholutDev &h, int r, int c, const Z *X, double km, double kn,
                               Z phi)
{
    Z d = zmk(0, 0);
    if (r >= 10) {
        const int e = 5 * (r - 10) + c;
        if (h.has_a) d = zadd(d, zscale(zmul(zmk(0, -km), phi), h.nrbc[e]));
        if (h.has_b) d = zadd(d, zscale(zmul(zmk(0, -kn), phi), h.nrbc[25 + e]));
        if (h.has_c) d = zadd(d, zmk(h.nrbc[50 + e], 0));
    }
    if (h.has_c)
        for (int k = 0; k < 5; ++k) d = zadd(d, zscale(X[r + 15 * k], -h.nrbc[50 + c + 5 * k]));
    return d;
}

__global__ void k_rholut_pack(RholutDev h, int nsys, Z phi, const double *__restrict__ km,
                              const double *__restrict__ kn, double2 *__restrict__ ab, int ldab,
                              long long stride, int off)
{
    const int warps = blockDim.x >> 5;
    const int C = blockIdx.x * warps + (threadIdx.x >> 5);
    const int s = blockIdx.y, lane = threadIdx.x & 31;
    const int N = h.S * h.n, KL = h.S * (h.kl + 1) - 1, KU = h.S * (h.ku + 1) - 1;
    if (C >= N || s >= nsys) return;
    __shared__ Passes tabs[4][5];
    Passes *tab = tabs[threadIdx.x >> 5];
    rholut_column_terms(h, C, km[s], kn[s], phi, lane, tab);
    const int q = C / h.S;
    double2 *col = ab + s * stride + (long long) C * ldab;
    for (int i = off + lane; i < ldab; i += 32) {     // rows above off are left alone
        const int R = C + i - off - KU;
        Z v = zmk(0, 0);
        if (i <= off + KL + KU && R >= 0 && R < N) {
            const int p = R / h.S;
            v = rholut_apply(h, tab[R - p * h.S], p, q, phi);
        }
        col[i] = make_double2(v.re, v.im);
    }
}

// One warp per system: the boundary correction of the packed transpose.
__global__ void k_rholut_pack_nrbc(RholutDev h, int nsys, Z phi, const double *__restrict__ km,
                                   const double *__restrict__ kn, double2 *__restrict__ ab,
                                   int ldab, long long stride, int off)
{
    const int s = blockIdx.x;
    if (s >= nsys) return;
    const int KU = h.S * (h.ku + 1) - 1, n = h.n;
    const int R0 = 5 * (n - 3), C0 = 5 * (n - 1);
    __shared__ Z X[75];
    double2 *base = ab + s * stride;
    auto at = [&](int r, int c) -> double2 & {
        const int R = R0 + r, C = C0 + c;
        return base[off + KU + R - C + (long long) C * ldab];
    };
    for (int t = threadIdx.x; t < 75; t += blockDim.x) {
        const double2 v = at(t % 15, t / 15);
        X[t] = zmk(v.x, v.y);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < 75; t += blockDim.x) {
        const int r = t % 15, c = t / 15;
        const Z d = rholut_nrbc_delta(h, r, c, X, km[s], kn[s], phi);
        double2 &e = at(r, c);
        e = make_double2(e.x + d.re, e.y + d.im);
    }
}

// y(C) <- sum_R A^T(R, C) x(R) + beta y(C), one warp per output C = (q, pos);
// x and y in natural order (position-major: pos n + q).  With the boundary
// correction, the last point's outputs add the correction's column.
__global__ void k_rholut_accumulate(RholutDev h, int nsys, Z phi, const double *__restrict__ km,
                                    const double *__restrict__ kn, const double2 *__restrict__ x,
                                    long long xs, Z beta, double2 *__restrict__ y, long long ys)
{
    const int warps = blockDim.x >> 5;
    const int C = blockIdx.x * warps + (threadIdx.x >> 5);
    const int s = blockIdx.y, lane = threadIdx.x & 31;
    const int S = h.S, n = h.n, N = S * n, KL = S * (h.kl + 1) - 1, KU = S * (h.ku + 1) - 1;
    if (C >= N || s >= nsys) return;
    const double kms = km[s], kns = kn[s];
    const double2 *xv = x + s * xs;
    __shared__ Passes tabs[4][5];
    Passes *tab = tabs[threadIdx.x >> 5];
    rholut_column_terms(h, C, kms, kns, phi, lane, tab);
    const int qc = C / S;
    Z acc = zmk(0, 0);
    const int Rlo = C - KU < 0 ? 0 : C - KU, Rhi = C + KL > N - 1 ? N - 1 : C + KL;
    for (int R = Rlo + lane; R <= Rhi; R += 32) {
        const int p = R / S, pos = R - p * S;
        const Z a = rholut_apply(h, tab[pos], p, qc, phi);
        const double2 xr = xv[pos * n + p];
        acc = zadd(acc, zmul(a, zmk(xr.x, xr.y)));
    }
    const bool nrbc = (h.has_a || h.has_b || h.has_c) && C >= 5 * (n - 1);
    if (nrbc) {
        // X column c = C - C0 over rows R0 .. R0 + 14 (unmodified), then the
        // correction's column applied to x
        const int R0 = 5 * (n - 3), c = C - 5 * (n - 1);
        Z X[75];
        for (int t = 0; t < 75; ++t)
            X[t] = rholut_entry(h, R0 + t % 15, 5 * (n - 1) + t / 15, kms, kns, phi);
        if (lane < 15) {
            const Z d = rholut_nrbc_delta(h, lane, c, X, kms, kns, phi);
            const int R = R0 + lane, p = R / S, pos = R - p * S;
            const double2 xr = xv[pos * n + p];
            acc = zadd(acc, zmul(d, zmk(xr.x, xr.y)));
        }
    }
    for (int o = 16; o; o >>= 1) {
        acc.re += __shfl_xor_sync(0xffffffffu, acc.re, o);
        acc.im += __shfl_xor_sync(0xffffffffu, acc.im, o);
    }
    if (lane == 0) {
        const int q = C / S, pos = C - q * S;
        double2 &yo = y[s * ys + pos * n + q];
        Z r = acc;
        if (beta.re != 0 || beta.im != 0) r = zadd(zmul(beta, zmk(yo.x, yo.y)), acc);
        yo = make_double2(r.re, r.im);
    }
}

thread_local std::string g_rerr;
int rfail(const char *msg)
{
    sgb_set_error(cudaErrorInvalidValue, msg, __FILE__, __LINE__);
    return -1;
}

// Equation order parameters -> (S, ord, inv); false if they are not a
// contiguous set starting at zero.
bool orders(const int o[5], int &S, int ord[5], int inv[5])
{
    S = 0;
    for (int e = 0; e < 5; ++e) {
        ord[e] = o[e] < 0 ? -1 : o[e];
        if (o[e] >= 0) ++S;
    }
    if (S == 0) return false;
    for (int p = 0; p < 5; ++p) inv[p] = -1;
    for (int e = 0; e < 5; ++e) {
        if (ord[e] < 0) continue;
        if (ord[e] >= S || inv[ord[e]] >= 0) return false;
        inv[ord[e]] = e;
    }
    return true;
}

}  // namespace

extern "C" sgb_rholut *sgb_rholut_create(const suzerain_rholut_imexop_scenario *s,
                                         const suzerain_rholut_imexop_ref *r,
                                         const suzerain_rholut_imexop_refld *ld,
                                         const suzerain_bsplineop_workspace *w, const int order[5],
                                         const double *a, const double *b, const double *c)
{
    if (!s || !r || !ld || !w || !order) { rfail("sgb_rholut_create: null argument"); return nullptr; }
    if (w->nderiv < 2 || w->n < 3) { rfail("sgb_rholut_create: workspace needs nderiv >= 2, n >= 3"); return nullptr; }
    int S, ord[5], inv[5];
    if (!orders(order, S, ord, inv)) {
        rfail("sgb_rholut_create: equation orders must be a contiguous set starting at zero");
        return nullptr;
    }
    if ((a || b || c) && !(S == 5 && ord[EE] == 0 && ord[EU] == 1 && ord[EV] == 2 && ord[EW] == 3
                          && ord[ER] == 4)) {
        rfail("sgb_rholut_create: the boundary matrices need all five equations in the order "
              "E, u, v, w, rho");
        return nullptr;
    }
    sgb_rholut *h = new (std::nothrow) sgb_rholut;
    if (!h) { rfail("sgb_rholut_create: out of host memory"); return nullptr; }
    RholutDev &d = h->d;
    d.n = w->n; d.kl = w->max_kl; d.ku = w->max_ku; d.ld = w->ld; d.S = S;
    for (int e = 0; e < 5; ++e) { d.ord[e] = ord[e]; d.inv[e] = inv[e]; }
    d.gamma = s->gamma;
    d.gm1 = s->gamma - 1; d.gm3 = s->gamma - 3;
    d.ap43 = s->alpha + 4.0 / 3.0; d.ap13 = s->alpha + 1.0 / 3.0;
    d.Ma2 = s->Ma * s->Ma; d.invRe = 1 / s->Re; d.invMa2 = 1 / d.Ma2;
    d.ginvPr = s->gamma / s->Pr; d.ginvRePr = s->gamma / (s->Re * s->Pr);
    d.has_a = a != nullptr; d.has_b = b != nullptr; d.has_c = c != nullptr;
    const size_t nb = (size_t) d.ld * d.n;
    std::vector<double> host(3 * nb + (size_t) NPROF * d.n + 75, 0.0);
    for (int k = 0; k < 3; ++k) {
        const double *view = w->D_T[k] - (w->max_ku - w->ku[k]);
        std::memcpy(&host[k * nb], view, nb * sizeof(double));
    }
    const double *const *rp = reinterpret_cast<const double *const *>(r);
    const int *lp = reinterpret_cast<const int *>(ld);
    double *pr = &host[3 * nb];
    for (int k = 0; k < NPROF; ++k)
        for (int q = 0; q < d.n; ++q) pr[(size_t) k * d.n + q] = rp[k] ? rp[k][(size_t) q * lp[k]] : 0.0;
    double *nr = pr + (size_t) NPROF * d.n;
    for (int t = 0; t < 25; ++t) {
        if (a) nr[t] = a[t];
        if (b) nr[25 + t] = b[t];
        if (c) nr[50 + t] = c[t];
    }
    cudaError_t e = cudaMalloc(&h->mem, host.size() * sizeof(double));
    if (e == cudaSuccess) e = cudaMemcpy(h->mem, host.data(), host.size() * sizeof(double),
                                         cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        sgb_set_error(e, "sgb_rholut_create", __FILE__, __LINE__);
        if (h->mem) cudaFree(h->mem);
        delete h;
        return nullptr;
    }
    double *dm = static_cast<double *>(h->mem);
    d.band = dm;
    d.prof = dm + 3 * nb;
    d.nrbc = dm + 3 * nb + (size_t) NPROF * d.n;
    return h;
}

extern "C" int sgb_rholut_destroy(sgb_rholut *h)
{
    if (!h) return 0;
    if (h->mem) cudaFree(h->mem);
    delete h;
    return 0;
}

extern "C" int sgb_rholut_geometry(const sgb_rholut *h, suzerain_bsmbsm *A)
{
    if (!h || !A) return rfail("sgb_rholut_geometry: null argument");
    *A = suzerain_bsmbsm_construct(h->d.S, h->d.n, h->d.kl, h->d.ku);
    return 0;
}

extern "C" int sgb_rholut_pack_batched(sgb_rholut *h, double phi_re, double phi_im, int nsys,
                                       const double *km, const double *kn, void *ab, int ldab,
                                       long long ab_stride, int off, void *stream)
{
    if (!h || !km || !kn || !ab || nsys < 0) return rfail("sgb_rholut_pack_batched: bad arguments");
    const RholutDev &d = h->d;
    const int N = d.S * d.n, KL = d.S * (d.kl + 1) - 1, KU = d.S * (d.ku + 1) - 1;
    if (off < 0 || ldab < off + KL + KU + 1 || ab_stride < (long long) ldab * N)
        return rfail("sgb_rholut_pack_batched: ldab must be >= off + KL + KU + 1 and "
                     "ab_stride >= ldab N");
    if (nsys == 0) return 0;
    cudaStream_t st = (cudaStream_t) stream;
    const Z phi{phi_re, phi_im};
    dim3 grd((unsigned) ((N + 3) / 4), (unsigned) nsys);
    count_launch(1);
    k_rholut_pack<<<grd, 128, 0, st>>>(d, nsys, phi, km, kn, reinterpret_cast<double2 *>(ab), ldab,
                                       ab_stride, off);
    SGB_CUDA_TRY(cudaGetLastError());
    if (d.has_a || d.has_b || d.has_c) {
        count_launch(1);
        k_rholut_pack_nrbc<<<nsys, 32, 0, st>>>(d, nsys, phi, km, kn, reinterpret_cast<double2 *>(ab),
                                               ldab, ab_stride, off);
        SGB_CUDA_TRY(cudaGetLastError());
    }
    return 0;
}

extern "C" int sgb_rholut_accumulate_batched(sgb_rholut *h, double phi_re, double phi_im, int nsys,
                                             const double *km, const double *kn, const void *x,
                                             long long x_stride, double beta_re, double beta_im,
                                             void *y, long long y_stride, void *stream)
{
    if (!h || !km || !kn || !x || !y || nsys < 0)
        return rfail("sgb_rholut_accumulate_batched: bad arguments");
    const RholutDev &d = h->d;
    const int N = d.S * d.n;
    if (x_stride < N || y_stride < N)
        return rfail("sgb_rholut_accumulate_batched: strides must be >= S n");
    if (nsys == 0) return 0;
    dim3 grd((unsigned) ((N + 3) / 4), (unsigned) nsys);
    count_launch(1);
    k_rholut_accumulate<<<grd, 128, 0, (cudaStream_t) stream>>>(
        d, nsys, Z{phi_re, phi_im}, km, kn, reinterpret_cast<const double2 *>(x), x_stride,
        Z{beta_re, beta_im}, reinterpret_cast<double2 *>(y), y_stride);
    SGB_CUDA_TRY(cudaGetLastError());
    return 0;
}

// ---------------------------------------------------------------------------
// Drop-ins with the reference's signatures (suzerain/rholut_imexop.h:175-470).
// Host or device pointers; one wavenumber pair per call; the work runs on the
// GPU.  The reference's buf argument is working storage these do not need.
// Errors (a bad argument, no device) leave the outputs untouched and set the
// library's last-error message (the reference asserts instead).
// ---------------------------------------------------------------------------
namespace {

bool dev_ptr(const void *p)
{
    if (!p) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return false; }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

struct Scratch1 {              // device km, kn and a buffer for one call
    double *k = nullptr;
    void *buf = nullptr;
    ~Scratch1() { if (k) cudaFree(k); if (buf) cudaFree(buf); }
};

int pack_one(sgb_complex_double phi, double km, double kn, const suzerain_rholut_imexop_scenario *s,
             const suzerain_rholut_imexop_ref *r, const suzerain_rholut_imexop_refld *ld,
             const suzerain_bsplineop_workspace *w, const int ord[5], suzerain_bsmbsm *A_T,
             sgb_complex_double *patpt, bool packf, const double *a, const double *b, const double *c)
{
    if (!patpt || !A_T) return rfail("rholut_imexop pack: null argument");
    sgb_rholut *h = sgb_rholut_create(s, r, ld, w, ord, a, b, c);
    if (!h) return -1;
    sgb_rholut_geometry(h, A_T);
    const int LD = A_T->LD, KL = A_T->KL, N = A_T->N;
    const int ldab = packf ? LD + KL : LD, off = packf ? KL : 0;
    const size_t bytes = (size_t) ldab * N * sizeof(double2);
    Scratch1 sc;
    const double kk[2] = {km, kn};
    cudaError_t e = cudaMalloc(&sc.k, sizeof kk);
    if (e == cudaSuccess) e = cudaMemcpy(sc.k, kk, sizeof kk, cudaMemcpyHostToDevice);
    const bool on_dev = dev_ptr(patpt);
    void *out = patpt;
    if (e == cudaSuccess && !on_dev) { e = cudaMalloc(&sc.buf, bytes); out = sc.buf; }
    if (e == cudaSuccess && !on_dev && packf)   // keep the caller's rows above the band
        e = cudaMemcpy(out, patpt, bytes, cudaMemcpyHostToDevice);
    int rc = e == cudaSuccess ? 0 : sgb_set_error(e, "rholut_imexop pack", __FILE__, __LINE__);
    if (!rc) {
        const std::complex<double> z(phi);
        rc = sgb_rholut_pack_batched(h, z.real(), z.imag(), 1, sc.k, sc.k + 1, out, ldab,
                                     (long long) ldab * N, off, nullptr);
    }
    if (!rc && !on_dev) {
        e = cudaMemcpy(patpt, out, bytes, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) rc = sgb_set_error(e, "rholut_imexop pack", __FILE__, __LINE__);
    }
    if (!rc && on_dev) {
        e = cudaDeviceSynchronize();
        if (e != cudaSuccess) rc = sgb_set_error(e, "rholut_imexop pack", __FILE__, __LINE__);
    }
    sgb_rholut_destroy(h);
    return rc;
}

int accumulate_one(sgb_complex_double phi, double km, double kn,
                   const suzerain_rholut_imexop_scenario *s, const suzerain_rholut_imexop_ref *r,
                   const suzerain_rholut_imexop_refld *ld, const suzerain_bsplineop_workspace *w,
                   const sgb_complex_double *const in[5], sgb_complex_double beta,
                   sgb_complex_double *const out[5], const double *a, const double *b,
                   const double *c)
{
    int ord[5], S = 0;
    for (int e = 0; e < 5; ++e) {
        if (!in[e] != !out[e]) return rfail("rholut_imexop accumulate: input and output must both be given or both NULL");
        ord[e] = in[e] ? S++ : -1;
    }
    if (!w) return rfail("rholut_imexop accumulate: null workspace");
    sgb_rholut *h = sgb_rholut_create(s, r, ld, w, ord, a, b, c);
    if (!h) return -1;
    const int n = w->n, N = S * n;
    const size_t vb = (size_t) n * sizeof(double2);
    Scratch1 sc;
    const double kk[2] = {km, kn};
    cudaError_t e = cudaMalloc(&sc.k, sizeof kk);
    if (e == cudaSuccess) e = cudaMemcpy(sc.k, kk, sizeof kk, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&sc.buf, 2 * (size_t) N * sizeof(double2));
    double2 *x = static_cast<double2 *>(sc.buf), *y = x + N;
    for (int k = 0; k < 5 && e == cudaSuccess; ++k) {
        if (ord[k] < 0) continue;
        e = cudaMemcpy(x + (size_t) ord[k] * n, in[k], vb, cudaMemcpyDefault);
        if (e == cudaSuccess) e = cudaMemcpy(y + (size_t) ord[k] * n, out[k], vb, cudaMemcpyDefault);
    }
    int rc = e == cudaSuccess ? 0 : sgb_set_error(e, "rholut_imexop accumulate", __FILE__, __LINE__);
    if (!rc) {
        const std::complex<double> z(phi), bt(beta);
        rc = sgb_rholut_accumulate_batched(h, z.real(), z.imag(), 1, sc.k, sc.k + 1, x, N,
                                           bt.real(), bt.imag(), y, N, nullptr);
    }
    for (int k = 0; k < 5 && !rc; ++k) {
        if (ord[k] < 0) continue;
        e = cudaMemcpy(out[k], y + (size_t) ord[k] * n, vb, cudaMemcpyDefault);
        if (e != cudaSuccess) rc = sgb_set_error(e, "rholut_imexop accumulate", __FILE__, __LINE__);
    }
    sgb_rholut_destroy(h);
    return rc;
}

}  // namespace

extern "C" void suzerain_rholut_imexop_accumulate(
    const sgb_complex_double phi, const double km, const double kn,
    const suzerain_rholut_imexop_scenario *s, const suzerain_rholut_imexop_ref *r,
    const suzerain_rholut_imexop_refld *ld, const suzerain_bsplineop_workspace *w,
    const sgb_complex_double *in_rho_E, const sgb_complex_double *in_rho_u,
    const sgb_complex_double *in_rho_v, const sgb_complex_double *in_rho_w,
    const sgb_complex_double *in_rho, const sgb_complex_double beta,
    sgb_complex_double *out_rho_E, sgb_complex_double *out_rho_u, sgb_complex_double *out_rho_v,
    sgb_complex_double *out_rho_w, sgb_complex_double *out_rho,
    const double *a, const double *b, const double *c)
{
    const sgb_complex_double *in[5] = {in_rho_E, in_rho_u, in_rho_v, in_rho_w, in_rho};
    sgb_complex_double *out[5] = {out_rho_E, out_rho_u, out_rho_v, out_rho_w, out_rho};
    accumulate_one(phi, km, kn, s, r, ld, w, in, beta, out, a, b, c);
}

extern "C" void suzerain_rholut_imexop_accumulate00(
    const sgb_complex_double phi, const suzerain_rholut_imexop_scenario *s,
    const suzerain_rholut_imexop_ref *r, const suzerain_rholut_imexop_refld *ld,
    const suzerain_bsplineop_workspace *w,
    const sgb_complex_double *in_rho_E, const sgb_complex_double *in_rho_u,
    const sgb_complex_double *in_rho_v, const sgb_complex_double *in_rho_w,
    const sgb_complex_double *in_rho, const sgb_complex_double beta,
    sgb_complex_double *out_rho_E, sgb_complex_double *out_rho_u, sgb_complex_double *out_rho_v,
    sgb_complex_double *out_rho_w, sgb_complex_double *out_rho, const double *c)
{
    const sgb_complex_double *in[5] = {in_rho_E, in_rho_u, in_rho_v, in_rho_w, in_rho};
    sgb_complex_double *out[5] = {out_rho_E, out_rho_u, out_rho_v, out_rho_w, out_rho};
    accumulate_one(phi, 0.0, 0.0, s, r, ld, w, in, beta, out, nullptr, nullptr, c);
}

extern "C" void suzerain_rholut_imexop_packc(
    const sgb_complex_double phi, const double km, const double kn,
    const suzerain_rholut_imexop_scenario *s, const suzerain_rholut_imexop_ref *r,
    const suzerain_rholut_imexop_refld *ld, const suzerain_bsplineop_workspace *w,
    const int rho_E, const int rho_u, const int rho_v, const int rho_w, const int rho,
    sgb_complex_double *buf, suzerain_bsmbsm *A_T, sgb_complex_double *patpt,
    const double *a, const double *b, const double *c)
{
    (void) buf;
    const int ord[5] = {rho_E, rho_u, rho_v, rho_w, rho};
    pack_one(phi, km, kn, s, r, ld, w, ord, A_T, patpt, false, a, b, c);
}

extern "C" void suzerain_rholut_imexop_packc00(
    const sgb_complex_double phi, const suzerain_rholut_imexop_scenario *s,
    const suzerain_rholut_imexop_ref *r, const suzerain_rholut_imexop_refld *ld,
    const suzerain_bsplineop_workspace *w,
    const int rho_E, const int rho_u, const int rho_v, const int rho_w, const int rho,
    sgb_complex_double *buf, suzerain_bsmbsm *A_T, sgb_complex_double *patpt, const double *c)
{
    (void) buf;
    const int ord[5] = {rho_E, rho_u, rho_v, rho_w, rho};
    pack_one(phi, 0.0, 0.0, s, r, ld, w, ord, A_T, patpt, false, nullptr, nullptr, c);
}

extern "C" void suzerain_rholut_imexop_packf(
    const sgb_complex_double phi, const double km, const double kn,
    const suzerain_rholut_imexop_scenario *s, const suzerain_rholut_imexop_ref *r,
    const suzerain_rholut_imexop_refld *ld, const suzerain_bsplineop_workspace *w,
    const int rho_E, const int rho_u, const int rho_v, const int rho_w, const int rho,
    sgb_complex_double *buf, suzerain_bsmbsm *A_T, sgb_complex_double *patpt,
    const double *a, const double *b, const double *c)
{
    (void) buf;
    const int ord[5] = {rho_E, rho_u, rho_v, rho_w, rho};
    pack_one(phi, km, kn, s, r, ld, w, ord, A_T, patpt, true, a, b, c);
}

extern "C" void suzerain_rholut_imexop_packf00(
    const sgb_complex_double phi, const suzerain_rholut_imexop_scenario *s,
    const suzerain_rholut_imexop_ref *r, const suzerain_rholut_imexop_refld *ld,
    const suzerain_bsplineop_workspace *w,
    const int rho_E, const int rho_u, const int rho_v, const int rho_w, const int rho,
    sgb_complex_double *buf, suzerain_bsmbsm *A_T, sgb_complex_double *patpt, const double *c)
{
    (void) buf;
    const int ord[5] = {rho_E, rho_u, rho_v, rho_w, rho};
    pack_one(phi, 0.0, 0.0, s, r, ld, w, ord, A_T, patpt, true, nullptr, nullptr, c);
}
