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
                    : suzerain_bsmbsm_zpackc(solver.get(), i, j, cd(1), B[i * S + j].data(),
                                             solver->PAPT.data());
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

    // The production operator the way apps/perfect/operator_hybrid_isothermal.cpp
    // drives the solver (:636-661): pack (M + phi L)^T with the rholut drop-ins
    // straight into the solver's storage through solver.get() as the geometry
    // and LU.data() / PAPT.data(), supplied_PAPT(), solve with trans 'T';
    // the solution satisfies the operator's own accumulate.
    {
        const double bp[] = {0.0, 0.5, 1.5, 2.25, 2.5, 3.0, 3.35};
        suzerain_bsplineop_workspace *w = sgb_bsplineop_alloc_breakpoints(6, 7, bp, 2);
        const int nn = w->n, NN = 5 * nn;
        suzerain_rholut_imexop_scenario sc{3000, 0.7, 1.5, 3, 1.4};
        std::vector<double> prof(26 * nn);
        for (auto &v : prof) v = 0.5 + std::abs(nd(rng)) * 0.2;
        suzerain_rholut_imexop_ref ref;
        suzerain_rholut_imexop_refld rld;
        for (int k = 0; k < 26; ++k) {
            reinterpret_cast<double **>(&ref)[k] = prof.data() + k * nn;
            reinterpret_cast<int *>(&rld)[k] = 1;
        }
        const cd phi(0.02, 0.01);
        const double km = 2.5, kn = -1.5;
        std::vector<cd> u(NN), y(NN), xs(NN), y2(NN);
        for (auto &v : u) v = cd(nd(rng), nd(rng));
        suzerain_rholut_imexop_accumulate(phi, km, kn, &sc, &ref, &rld, w, &u[0], &u[nn], &u[2 * nn],
                                          &u[3 * nn], &u[4 * nn], cd(0), &y[0], &y[nn], &y[2 * nn],
                                          &y[3 * nn], &y[4 * nn], nullptr, nullptr, nullptr);
        const suzerain_bsmbsm AA = suzerain_bsmbsm_construct(5, nn, w->max_kl, w->max_ku);
        std::vector<cd> buf((size_t) std::max(75, nn * (w->max_kl + 1 + w->max_ku)));
        for (const char *text : {"zgbsv", "zcgbsvx,aiter=5,siter=25,diter=5,tolsc=0"}) {
            suzerain_gb300::specification_zgbsv spec(text);
            auto solver = suzerain_gb300::bsmbsm_solver::build(AA, spec, 1);
            if (solver->spec.in_place())
                suzerain_rholut_imexop_packf(phi, km, kn, &sc, &ref, &rld, w, 0, 1, 2, 3, 4,
                                             buf.data(), solver.get(), solver->LU.data(),
                                             nullptr, nullptr, nullptr);
            else
                suzerain_rholut_imexop_packc(phi, km, kn, &sc, &ref, &rld, w, 0, 1, 2, 3, 4,
                                             buf.data(), solver.get(), solver->PAPT.data(),
                                             nullptr, nullptr, nullptr);
            if (solver->PAPT.colStride() != (solver->spec.in_place() ? AA.KL + AA.LD : AA.LD)) {
                std::printf("FAIL PAPT colStride\n");
                return 1;
            }
            solver->supplied_PAPT();
            solver->supply_b(y.data(), 0);
            solver->solve('T');
            solver->demand_x(xs.data(), 0);
            suzerain_rholut_imexop_accumulate(phi, km, kn, &sc, &ref, &rld, w, &xs[0], &xs[nn],
                                              &xs[2 * nn], &xs[3 * nn], &xs[4 * nn], cd(0),
                                              &y2[0], &y2[nn], &y2[2 * nn], &y2[3 * nn],
                                              &y2[4 * nn], nullptr, nullptr, nullptr);
            double r = 0, ym = 0;
            for (int i = 0; i < NN; ++i) { r = std::max(r, std::abs(y2[i] - y[i])); ym = std::max(ym, std::abs(y[i])); }
            std::printf("rholut %s: |A x - y| / |y| = %.3e\n", text, r / ym);
            if (!(r <= 1e-12 * ym)) { std::printf("FAIL rholut %s\n", text); return 1; }
        }
        suzerain_bsplineop_free(w);
    }
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
