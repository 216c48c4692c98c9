// B-spline collocation operators at the Greville abscissae (host setup code).
//
// Restates what suzerain_bsplineop_alloc builds for
// SUZERAIN_BSPLINEOP_COLLOCATION_GREVILLE (suzerain/bsplineop.c:102-202,
// :403-519, :553-655) without GSL:
//   * knots from breakpoints with k-fold end knots, as gsl_bspline_knots
//     (suzerain/bspline.hpp:84-93): n = nbreak + k - 2 basis functions;
//   * Greville abscissa i = mean of knots i+1 .. i+k-1;
//   * basis derivatives by the recurrence of Piegl & Tiller, The NURBS Book,
//     2nd ed., algorithms A2.1 (span) and A2.3 (derivatives of the nonzero
//     basis functions), a restatement of de Boor's BSPLVD;
//   * band storage per derivative with kl/ku trimmed by exact-zero tests
//     (suzerain/bsplineop.c:479-510), operators stored transposed in the
//     reference-compatible workspace and non-transposed for the collocation
//     matrices the synthetic generator assembles.
#include "suzerain_gb300.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

namespace {

struct Basis {
    int k, n;
    std::vector<double> knots;
};

Basis make_basis(int k, int nbreak, const double *bp)
{
    Basis B;
    B.k = k;
    B.n = nbreak + k - 2;
    for (int i = 0; i < k; ++i) B.knots.push_back(bp[0]);
    for (int i = 1; i < nbreak - 1; ++i) B.knots.push_back(bp[i]);
    for (int i = 0; i < k; ++i) B.knots.push_back(bp[nbreak - 1]);
    return B;
}

double greville(const Basis &B, int i)
{
    double s = 0;
    for (int m = i + 1; m <= i + B.k - 1; ++m) s += B.knots[m];
    return s / (B.k - 1);
}

// A2.1: knot span index containing u (right end closed).
int find_span(const Basis &B, double u)
{
    const int p = B.k - 1, nn = B.n - 1;
    const std::vector<double> &U = B.knots;
    if (u >= U[nn + 1]) return nn;
    if (u <= U[p]) return p;
    int lo = p, hi = nn + 1, mid = (lo + hi) / 2;
    while (u < U[mid] || u >= U[mid + 1]) {
        if (u < U[mid]) hi = mid; else lo = mid;
        mid = (lo + hi) / 2;
    }
    return mid;
}

// A2.3: ders[d][j] = d-th derivative of basis function span-p+j at u.
void ders_basis(const Basis &B, int span, double u, int nd, std::vector<double> &ders)
{
    const int p = B.k - 1;
    const std::vector<double> &U = B.knots;
    std::vector<double> ndu((p + 1) * (p + 1)), left(p + 1), right(p + 1);
    auto NDU = [&](int a, int b) -> double & { return ndu[a * (p + 1) + b]; };
    NDU(0, 0) = 1.0;
    for (int j = 1; j <= p; ++j) {
        left[j] = u - U[span + 1 - j];
        right[j] = U[span + j] - u;
        double saved = 0.0;
        for (int r = 0; r < j; ++r) {
            NDU(j, r) = right[r + 1] + left[j - r];
            const double temp = NDU(r, j - 1) / NDU(j, r);
            NDU(r, j) = saved + right[r + 1] * temp;
            saved = left[j - r] * temp;
        }
        NDU(j, j) = saved;
    }
    ders.assign((nd + 1) * (p + 1), 0.0);
    auto D = [&](int a, int b) -> double & { return ders[a * (p + 1) + b]; };
    for (int j = 0; j <= p; ++j) D(0, j) = NDU(j, p);
    std::vector<double> a(2 * (p + 1));
    auto A = [&](int s, int j) -> double & { return a[s * (p + 1) + j]; };
    for (int r = 0; r <= p; ++r) {
        int s1 = 0, s2 = 1;
        A(0, 0) = 1.0;
        for (int kk = 1; kk <= nd && kk <= p; ++kk) {
            double d = 0.0;
            const int rk = r - kk, pk = p - kk;
            if (r >= kk) {
                A(s2, 0) = A(s1, 0) / NDU(pk + 1, rk);
                d = A(s2, 0) * NDU(rk, pk);
            }
            const int j1 = rk >= -1 ? 1 : -rk;
            const int j2 = (r - 1 <= pk) ? kk - 1 : p - r;
            for (int j = j1; j <= j2; ++j) {
                A(s2, j) = (A(s1, j) - A(s1, j - 1)) / NDU(pk + 1, rk + j);
                d += A(s2, j) * NDU(rk + j, pk);
            }
            if (r <= pk) {
                A(s2, kk) = -A(s1, kk - 1) / NDU(pk + 1, r);
                d += A(s2, kk) * NDU(r, pk);
            }
            D(kk, r) = d;
            std::swap(s1, s2);
        }
    }
    double rr = p;
    for (int kk = 1; kk <= nd && kk <= p; ++kk) {
        for (int j = 0; j <= p; ++j) D(kk, j) *= rr;
        rr *= (p - kk);
    }
}

// Dense collocation matrices D[m][i*n + j] = d^m B_j(xi_i), m = 0..nd.
bool collocation_dense(int k, int nbreak, const double *bp, int nd, int &n,
                       std::vector<double> &dense, std::vector<double> &xi)
{
    if (k < 2 || nbreak < 2 || nd < 0) return false;
    for (int i = 1; i < nbreak; ++i)
        if (!(bp[i] > bp[i - 1])) return false;
    Basis B = make_basis(k, nbreak, bp);
    n = B.n;
    dense.assign((size_t) (nd + 1) * n * n, 0.0);
    xi.resize(n);
    std::vector<double> ders;
    for (int i = 0; i < n; ++i) {
        xi[i] = greville(B, i);
        const int span = find_span(B, xi[i]);
        ders_basis(B, span, xi[i], nd, ders);
        for (int m = 0; m <= nd; ++m)
            for (int j = 0; j < k; ++j) {
                const int col = span - (k - 1) + j;
                if (col >= 0 && col < n) dense[((size_t) m * n + i) * n + col] = ders[m * k + j];
            }
    }
    return true;
}

// Exact-zero trimmed bandwidths of one dense n x n matrix.
void trimmed_band(const double *A, int n, int &kl, int &ku)
{
    kl = 0; ku = 0;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
            if (A[(size_t) i * n + j] != 0.0) {
                kl = std::max(kl, i - j);
                ku = std::max(ku, j - i);
            }
}

}  // namespace

extern "C" int sgb_bspline_collocation_bands(int k, int nbreak, const double *breakpts,
                                             int nderiv, int *n_out, int *kl_out,
                                             int *ku_out, double *bands, double *abscissae)
{
    int n = 0;
    std::vector<double> dense, xi;
    if (!collocation_dense(k, nbreak, breakpts, nderiv, n, dense, xi)) return -1;
    int kl = 0, ku = 0;
    for (int m = 0; m <= nderiv; ++m) {
        int a, b;
        trimmed_band(dense.data() + (size_t) m * n * n, n, a, b);
        kl = std::max(kl, a);
        ku = std::max(ku, b);
    }
    if (n_out) *n_out = n;
    if (kl_out) *kl_out = kl;
    if (ku_out) *ku_out = ku;
    const int ld = kl + 1 + ku;
    if (bands) {
        std::memset(bands, 0, sizeof(double) * (size_t) (nderiv + 1) * ld * n);
        for (int m = 0; m <= nderiv; ++m)
            for (int j = 0; j < n; ++j)
                for (int i = std::max(0, j - ku); i <= std::min(n - 1, j + kl); ++i)
                    bands[((size_t) m * n + j) * ld + ku + i - j] = dense[((size_t) m * n + i) * n + j];
    }
    if (abscissae) std::copy(xi.begin(), xi.end(), abscissae);
    return 0;
}

extern "C" suzerain_bsplineop_workspace *
sgb_bsplineop_alloc_breakpoints(int k, int nbreak, const double *breakpts, int nderiv)
{
    int n = 0;
    std::vector<double> dense, xi;
    if (!collocation_dense(k, nbreak, breakpts, nderiv, n, dense, xi)) return nullptr;
    const size_t hdr = sizeof(suzerain_bsplineop_workspace)
                     + 2 * (nderiv + 1) * sizeof(int) + (nderiv + 1) * sizeof(double *);
    char *mem = static_cast<char *>(std::calloc(1, hdr));
    if (!mem) return nullptr;
    auto *w = reinterpret_cast<suzerain_bsplineop_workspace *>(mem);
    w->method = SUZERAIN_BSPLINEOP_COLLOCATION_GREVILLE;
    w->k = k;
    w->n = n;
    w->nderiv = nderiv;
    w->kl = reinterpret_cast<int *>(mem + sizeof(*w));
    w->ku = w->kl + (nderiv + 1);
    w->D_T = reinterpret_cast<double **>(w->ku + (nderiv + 1));
    // The stored operators are transposes: D_T(j, i) = d^m B_j(xi_i), so
    // kl of D_T is ku of D and vice versa.
    for (int m = 0; m <= nderiv; ++m) {
        int a, b;
        trimmed_band(dense.data() + (size_t) m * n * n, n, a, b);
        w->kl[m] = b;
        w->ku[m] = a;
    }
    w->max_kl = *std::max_element(w->kl, w->kl + nderiv + 1);
    w->max_ku = *std::max_element(w->ku, w->ku + nderiv + 1);
    w->ld = w->max_ku + 1 + w->max_kl;
    double *store = static_cast<double *>(std::calloc((size_t) w->ld * n * (nderiv + 1), sizeof(double)));
    if (!store) { std::free(mem); return nullptr; }
    for (int m = 0; m <= nderiv; ++m) {
        // Each operator shares ld; its pointer steps past unused superdiagonals
        // (suzerain/bsplineop.c:180-186).
        w->D_T[m] = store + (size_t) m * w->ld * n + (w->max_ku - w->ku[m]);
        for (int col = 0; col < n; ++col)          // column of D_T = point index
            for (int row = 0; row < n; ++row) {    // row of D_T = basis index
                const double v = dense[((size_t) m * n + col) * n + row];
                if (v != 0.0) w->D_T[m][(size_t) col * w->ld + w->ku[m] + row - col] = v;
            }
    }
    return w;
}

extern "C" void suzerain_bsplineop_free(suzerain_bsplineop_workspace *w)
{
    if (!w) return;
    if (w->D_T && w->D_T[0]) std::free(w->D_T[0] - (w->max_ku - w->ku[0]));
    std::free(w);
}

extern "C" double suzerain_htstretch2(const double delta, const double L, const double x)
{
    // suzerain/htstretch.c:112-125
    if (delta == 0.0) return x / L;
    return 0.5 * (1 + std::tanh(delta * (x / L - 0.5)) / std::tanh(delta / 2.));
}
