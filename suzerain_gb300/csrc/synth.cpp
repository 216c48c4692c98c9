// Seeded synthetic inputs for the benchmark configurations (host code).
//
// A case is the B-spline basis of the reference's create_bsplines
// (suzerain/support/support.cpp:245-322): nbreak = Ny - k + 2 breakpoints,
// linspace on [0,1] stretched by htstretch2(delta, 1, x) and mapped to
// [left, right], collocation at the Greville abscissae, plus the S x S block
// coefficients of the model operator: a, b, c ~ U(0.5, 1.5) on the block
// diagonal and offscale * U(-1, 1) off it, g = 0 (real blocks) or
// 0.1 * U(-1, 1) (complex coupling i phi g kx).
//
// Random numbers: SplitMix64 (Steele, Lea & Flood 2014) keyed by
// (seed, stream, counter), uniform doubles from the top 53 bits, normal
// pairs by the Box-Muller transform.  Every value is a pure function of its
// indices, so any subset of systems can be regenerated independently.
#include "suzerain_gb300.h"

#include <cmath>
#include <cstdint>
#include <vector>

namespace {

inline uint64_t splitmix64(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

inline double uniform(uint64_t seed, uint64_t stream, uint64_t ctr)
{
    const uint64_t h = splitmix64(splitmix64(seed ^ (stream * 0xD1B54A32D192ED03ull)) + ctr);
    return (double) (h >> 11) * (1.0 / 9007199254740992.0);   // [0, 1)
}

}  // namespace

extern "C" int sgb_synth_case(int S, int Ny, int k, double htdelta, double left,
                              double right, double offscale, int complex_coupling,
                              uint64_t seed, unsigned dirichlet_mask, int *kl_out,
                              int *ku_out, double *M, double *D1, double *D2, double *a,
                              double *b, double *c, double *g)
{
    (void) dirichlet_mask;
    if (S < 1 || k < 2 || Ny < k) return -1;
    const int nbreak = Ny - k + 2;
    std::vector<double> bp(nbreak);
    for (int i = 0; i < nbreak; ++i) {
        const double x = nbreak > 1 ? (double) i / (nbreak - 1) : 0.0;
        bp[i] = (right - left) * suzerain_htstretch2(htdelta, 1.0, x) + left;
    }
    bp[0] = left;
    bp[nbreak - 1] = right;
    int n = 0, kl = 0, ku = 0;
    if (sgb_bspline_collocation_bands(k, nbreak, bp.data(), 2, &n, &kl, &ku, nullptr, nullptr))
        return -2;
    if (kl_out) *kl_out = kl;
    if (ku_out) *ku_out = ku;
    if (M) {
        const int ld = kl + 1 + ku;
        std::vector<double> bands((size_t) 3 * ld * n);
        sgb_bspline_collocation_bands(k, nbreak, bp.data(), 2, &n, &kl, &ku, bands.data(), nullptr);
        for (size_t i = 0; i < (size_t) ld * n; ++i) {
            M[i] = bands[i];
            D1[i] = bands[(size_t) ld * n + i];
            D2[i] = bands[(size_t) 2 * ld * n + i];
        }
    }
    if (a) {
        for (int e = 0; e < S; ++e)
            for (int f = 0; f < S; ++f) {
                const int ef = e * S + f;
                const double u0 = uniform(seed, 1, ef), u1 = uniform(seed, 2, ef),
                             u2 = uniform(seed, 3, ef), u3 = uniform(seed, 4, ef);
                if (e == f) {
                    a[ef] = 0.5 + u0; b[ef] = 0.5 + u1; c[ef] = 0.5 + u2;
                } else {
                    a[ef] = offscale * (2 * u0 - 1);
                    b[ef] = offscale * (2 * u1 - 1);
                    c[ef] = offscale * (2 * u2 - 1);
                }
                g[ef] = complex_coupling ? 0.1 * (2 * u3 - 1) : 0.0;
            }
    }
    return 0;
}

extern "C" int suzerain_inorder_wavenumber(const int N, const int i)
{
    // suzerain/inorder.h:92-96
    return (i < N / 2 + 1) ? i : -N + i;
}

extern "C" int sgb_synth_wavenumbers(int Nx, int Nz, double Lx, double Lz, double *kx,
                                     double *kz)
{
    // R2C modes m = 0..Nx/2 along x, all Nz in-order modes along z; the
    // system index runs m fastest like the reference's (n, m) double loop
    // (apps/perfect/operator_hybrid_isothermal.cpp:612-613).
    if (Nx < 1 || Nz < 1) return -1;
    const int Mx = Nx / 2 + 1;
    const double twopi = 2 * std::acos(-1.0);
    for (int iz = 0; iz < Nz; ++iz)
        for (int m = 0; m < Mx; ++m) {
            kx[(size_t) iz * Mx + m] = twopi / Lx * m;
            kz[(size_t) iz * Mx + m] = twopi / Lz * suzerain_inorder_wavenumber(Nz, iz);
        }
    return 0;
}

extern "C" int sgb_synth_rhs(uint64_t seed, long long nsys, int N, double *u)
{
    // u[(s*N + i)*2 + {0,1}]: independent N(0,1) real and imaginary parts.
    const double twopi = 2 * std::acos(-1.0);
    for (long long s = 0; s < nsys; ++s)
        for (int i = 0; i < N; ++i) {
            const uint64_t ctr = (uint64_t) s * (uint64_t) N + (uint64_t) i;
            double u1 = uniform(seed, 11, ctr), u2 = uniform(seed, 12, ctr);
            if (u1 < 1e-300) u1 = 1e-300;
            const double rad = std::sqrt(-2 * std::log(u1));
            u[2 * ((size_t) s * N + i)] = rad * std::cos(twopi * u2);
            u[2 * ((size_t) s * N + i) + 1] = rad * std::sin(twopi * u2);
        }
    return 0;
}
