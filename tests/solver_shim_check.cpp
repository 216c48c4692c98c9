// Drives include/suzerain_gb300_solver.hpp the way Suzerain's operators
// drive suzerain::bsmbsm_solver: pack S x S banded blocks into P A P^T,
// supply b, solve, demand x (twice: the second solve reuses the factor);
// checks A x = b against a dense copy of A for the zgbsv, zgbsvx (with and
// without equilibration) and zcgbsvx specifications.  Prints "OK ..." on
// success.
#include "suzerain_gb300_solver.hpp"

#include <cmath>
#include <cstdio>
#include <random>

using cd = std::complex<double>;

int main()
{
    const int S = 3, n = 24, kl = 2, ku = 2;
    const suzerain_bsmbsm A = suzerain_bsmbsm_construct(S, n, kl, ku);
    const int N = A.N, ld = kl + ku + 1;
    std::mt19937_64 rng(7);
    std::normal_distribution<double> nd;
    // blocks B^{ij}: ld x n LAPACK bands, dominant diagonal blocks
    std::vector<std::vector<cd>> B(S * S, std::vector<cd>((size_t) ld * n));
    std::vector<cd> dense((size_t) N * N, 0.0);
    for (int i = 0; i < S; ++i)
        for (int j = 0; j < S; ++j)
            for (int c = 0; c < n; ++c)
                for (int r = std::max(0, c - ku); r <= std::min(n - 1, c + kl); ++r) {
                    cd v(nd(rng), nd(rng));
                    if (i == j && r == c) v += 20.0;
                    if (i != j) v *= 0.2;
                    B[i * S + j][ku + r - c + (size_t) c * ld] = v;
                    dense[(size_t) (i * n + r) + (size_t) (j * n + c) * N] = v;
                }
    std::vector<cd> b(N), x(N);
    for (auto &v : b) v = cd(nd(rng), nd(rng));
    double worst = 0;
    for (const char *text : {"zgbsv", "zgbsvx,equil=true", "zgbsvx",
                             "zcgbsvx,aiter=5,siter=25,diter=5,tolsc=145"}) {
        suzerain_gb300::specification_zgbsv spec(text);
        auto solver = suzerain_gb300::bsmbsm_solver::build(A, spec, 1);
        for (int i = 0; i < S; ++i)
            for (int j = 0; j < S; ++j) {
                const int rc = spec.in_place()
                    ? suzerain_bsmbsm_zpackf(&A, i, j, cd(1), B[i * S + j].data(), solver->LU.data())
                    : suzerain_bsmbsm_zpackc(&A, i, j, cd(1), B[i * S + j].data(), solver->PAPT());
                if (rc) { std::printf("FAIL pack %d\n", rc); return 1; }
            }
        solver->supplied_PAPT();
        for (int rep = 0; rep < 2; ++rep) {
        if (solver->supply_b(b.data(), 0)) { std::printf("FAIL supply_b\n"); return 1; }
        solver->solve('N');
        if (solver->demand_x(x.data(), 0)) { std::printf("FAIL demand_x\n"); return 1; }
        double rmax = 0, amax = 0, xmax = 0, bmax = 0;
        for (int r = 0; r < N; ++r) {
            cd acc = 0;
            double arow = 0;
            for (int c = 0; c < N; ++c) {
                acc += dense[r + (size_t) c * N] * x[c];
                arow += std::abs(dense[r + (size_t) c * N]);
            }
            rmax = std::max(rmax, std::abs(acc - b[r]));
            amax = std::max(amax, arow);
            xmax = std::max(xmax, std::abs(x[r]));
            bmax = std::max(bmax, std::abs(b[r]));
        }
        const double berr = rmax / (amax * xmax + bmax);
        worst = std::max(worst, berr);
        for (const auto &line : solver->summarize_statistics()) std::printf("# %s\n", line.c_str());
        std::printf("%s berr=%.3e fact=%c\n", std::string(spec).c_str(), berr, solver->fact());
        }
    }
    if (worst > 1e-13) { std::printf("FAIL berr %.3e\n", worst); return 1; }
    // an invalid specification is rejected with the reference's message
    try {
        suzerain_gb300::specification_zgbsv bad("zcgbsvx,aiter");
        std::printf("FAIL no exception\n");
        return 1;
    } catch (const std::invalid_argument &e) {
        std::printf("# %s\n", e.what());
    }
    std::printf("OK worst berr %.3e\n", worst);
    return 0;
}
