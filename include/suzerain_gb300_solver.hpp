// Header-only C++ counterpart of suzerain::bsmbsm_solver
// (suzerain/bsmbsm_solver.hpp:70-330, suzerain/bsmbsm_solver.cpp:58-414) over
// the C ABI of suzerain_gb300.h: the same protocol (supply_b/B -> optional
// supplied_PAPT()/apprx() -> solve -> demand_x/X), the same storage roles
// (LU, PAPT, PB, PX, ipiv; column-major, PAPT in bsmbsm packed band order),
// the same specification strings and the same error messages.  The solves run
// on the GPU through the drop-in entry points (suzerain_lapackext_zgbsv,
// suzerain_lapack_zgbsvx, suzerain_lapackext_zcgbsvx); the storage here is
// host memory, as the reference's Eigen members are.
//
// Difference: errors throw std::runtime_error (the reference calls
// SUZERAIN_ERROR, whose default handler aborts).
#ifndef SUZERAIN_GB300_SOLVER_HPP
#define SUZERAIN_GB300_SOLVER_HPP

#include <algorithm>
#include <cctype>
#include <complex>
#include <cstdio>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "suzerain_gb300.h"

namespace suzerain_gb300 {

/** A solver specification string with the reference's grammar. */
class specification_zgbsv {
public:
    explicit specification_zgbsv(const std::string &text = "")
    {
        char err[512];
        if (sgb_solver_spec_parse(text.c_str(), &s_, err, sizeof err) != 0)
            throw std::invalid_argument(err);
    }
    int method() const { return s_.method; }
    bool equil() const { return s_.equil != 0; }
    bool reuse() const { return s_.reuse != 0; }
    int aiter() const { return s_.aiter; }
    int siter() const { return s_.siter; }
    int diter() const { return s_.diter; }
    double tolsc() const { return s_.tolsc; }
    bool in_place() const { return s_.method == SGB_METHOD_ZGBSV; }
    const char *mname() const
    {
        switch (s_.method) {
        case SGB_METHOD_ZGBSV: return "suzerain_lapackext_zgbsv";
        case SGB_METHOD_ZGBSVX: return "suzerain_lapack_zgbsvx";
        case SGB_METHOD_ZCGBSVX: return "suzerain_lapackext_zcgbsvx";
        default: return "UNKNOWN";
        }
    }
    operator std::string() const
    {
        char buf[256];
        sgb_solver_spec_format(&s_, buf, sizeof buf);
        return buf;
    }

private:
    sgb_solver_spec s_;
};

/** Column-major complex storage with the members of the reference's Eigen
 *  matrices that Suzerain's operators use on a solver's LU, PAPT, PB and PX
 *  (data(), colStride(), rows(), cols(), element access,
 *  apps/perfect/operator_hybrid_isothermal.cpp:643-661): it owns its
 *  elements, or views another's (the in-place solver's PAPT inside LU). */
class cmatrix {
public:
    using value_type = std::complex<double>;
    cmatrix() = default;
    cmatrix(int rows, int cols, value_type fill = value_type(0))
        : own_((size_t) rows * cols, fill), p_(own_.data()), rows_(rows), cols_(cols), ld_(rows)
    {
    }
    static cmatrix view(value_type *p, int rows, int cols, int ld)
    {
        cmatrix m;
        m.p_ = p; m.rows_ = rows; m.cols_ = cols; m.ld_ = ld;
        return m;
    }
    cmatrix(cmatrix &&o) noexcept { *this = std::move(o); }
    cmatrix &operator=(cmatrix &&o) noexcept
    {
        const bool owned = o.p_ == o.own_.data() && !o.own_.empty();
        own_ = std::move(o.own_);
        p_ = owned ? own_.data() : o.p_;
        rows_ = o.rows_; cols_ = o.cols_; ld_ = o.ld_;
        return *this;
    }
    cmatrix(const cmatrix &) = delete;
    cmatrix &operator=(const cmatrix &) = delete;
    value_type *data() { return p_; }
    const value_type *data() const { return p_; }
    int rows() const { return rows_; }
    int cols() const { return cols_; }
    int colStride() const { return ld_; }
    value_type &operator()(int i, int j) { return p_[i + (size_t) j * ld_]; }
    const value_type &operator()(int i, int j) const { return p_[i + (size_t) j * ld_]; }
    void setConstant(value_type v)
    {
        for (int j = 0; j < cols_; ++j) std::fill(p_ + (size_t) j * ld_, p_ + (size_t) j * ld_ + rows_, v);
    }

private:
    std::vector<value_type> own_;
    value_type *p_ = nullptr;
    int rows_ = 0, cols_ = 0, ld_ = 0;
};

/** suzerain::bsmbsm_solver: the solver is the BSMBSM geometry (as the
 *  reference's derives from suzerain_bsmbsm, so a solver pointer is passed
 *  where the packing routines take the geometry) plus its storage. */
class bsmbsm_solver : public suzerain_bsmbsm {
public:
    using complex_double = std::complex<double>;

    virtual ~bsmbsm_solver() = default;

    /** zgbsv, zgbsvx or zcgbsvx per the specification (nrhs right hand sides). */
    static std::unique_ptr<bsmbsm_solver> build(const suzerain_bsmbsm &A,
                                                const specification_zgbsv &spec, int nrhs);

    /** The geometry (this object viewed as its suzerain_bsmbsm base). */
    const suzerain_bsmbsm &A;
    const specification_zgbsv spec;

    // Storage (column-major), the reference's public members: LU holds the
    // factor; PAPT the packed band P A P^T that callers fill (e.g. with
    // suzerain_bsmbsm_zpackc/zpackf or suzerain_rholut_imexop_packc/packf,
    // writing through PAPT.data() with leading dimension PAPT.colStride():
    // rows KL.. of LU for the in-place zgbsv, its own LD x N otherwise)
    // before calling supplied_PAPT(); PB the permuted right hand sides, PX
    // the permuted solutions (PB itself for zgbsv); ipiv the pivots.
    cmatrix LU, PAPT, PB, PX;
    std::vector<int> ipiv;
    int nrhs() const { return nrhs_; }

    /** PB(:, j) = P b */
    int supply_b(const complex_double *b, int j, int incb = 1)
    {
        check_col(j);
        return suzerain_bsmbsm_zaPxpby('N', A.S, A.n, complex_double(1), b, incb,
                                       complex_double(0), PB.data() + (size_t) j * A.N, 1);
    }
    int supply_B(const complex_double *B, int ldB, int incB = 1)
    {
        int info = 0;
        for (int j = 0; !info && j < nrhs_; ++j) info = supply_b(B + (size_t) j * ldB, j, incB);
        return info;
    }
    int supply_B(const complex_double *B) { return supply_B(B, A.N, 1); }

    char fact() const { return fact_; }
    char default_fact() const { return spec.equil() ? 'E' : 'N'; }
    bool apprx() const { return apprx_ != 0; }

    /** PAPT was (re)written: refactor on the next solve, or, when the
     *  specification allows reuse, keep the factor as an approximation. */
    virtual bsmbsm_solver &supplied_PAPT()
    {
        if (spec.reuse()) apprx_ = fact_ != default_fact();
        else fact_ = default_fact();
        return *this;
    }
    /** Whether a reused factor is still acceptable; returns the old flag. */
    bool apprx(bool acceptable)
    {
        const bool old = apprx_ != 0;
        if (spec.reuse()) {
            apprx_ = (apprx_ && acceptable) ? 1 : 0;
            if (!apprx_) fact_ = default_fact();
        }
        return old;
    }

    int solve(char trans, int nrhs)
    {
        if (nrhs == 0) return 0;
        if (nrhs < 1 || nrhs > nrhs_) throw std::invalid_argument("Invalid nrhs supplied to solve()");
        const int info = solve_hook(trans, nrhs);
        if (info == 0) return 0;
        char buf[256];
        if (info < 0)
            std::snprintf(buf, sizeof buf, "%s reported error in argument %d", spec.mname(), -info);
        else if (info <= A.N)
            std::snprintf(buf, sizeof buf,
                          "%s reported singularity in PAP^T row %d corresponding to A row %d"
                          " for state scalar %d",
                          spec.mname(), info - 1, suzerain_bsmbsm_q(A.S, A.n, info - 1),
                          suzerain_bsmbsm_q(A.S, A.n, info - 1) / A.n);
        else
            std::snprintf(buf, sizeof buf, "%s reported unknown error %d", spec.mname(), info);
        throw std::runtime_error(buf);
    }
    int solve(char trans) { return solve(trans, nrhs_); }

    /** x = P^T PX(:, j) */
    int demand_x(complex_double *x, int j, int incx = 1) const
    {
        check_col(j);
        return suzerain_bsmbsm_zaPxpby('T', A.S, A.n, complex_double(1),
                                       PX.data() + (size_t) j * A.N, 1, complex_double(0), x, incx);
    }
    int demand_X(complex_double *X, int ldX, int incX = 1) const
    {
        int info = 0;
        for (int j = 0; !info && j < nrhs_; ++j) info = demand_x(X + (size_t) j * ldX, j, incX);
        return info;
    }
    int demand_X(complex_double *X) const { return demand_X(X, A.N, 1); }

    virtual std::vector<std::string> summarize_statistics() const
    {
        return {"Employed bsmbsm_solver per specification " + std::string(spec)};
    }

protected:
    bsmbsm_solver(const suzerain_bsmbsm &a, const specification_zgbsv &s, int nrhs)
        : suzerain_bsmbsm(a), A(*this), spec(s), PB(a.N, nrhs), ipiv(a.N), nrhs_(nrhs),
          fact_(s.equil() ? 'E' : 'N'), apprx_(0)
    {
        if (nrhs < 1) throw std::invalid_argument("nrhs must be positive");
    }
    bsmbsm_solver(const bsmbsm_solver &) = delete;
    bsmbsm_solver &operator=(const bsmbsm_solver &) = delete;
    virtual int solve_hook(char trans, int nrhs) = 0;
    void check_col(int j) const
    {
        if (j < 0 || j >= nrhs_) throw std::out_of_range("right hand side column");
    }

    int nrhs_;
    char fact_;
    int apprx_;
};

/** Plain complex128 band LU, in place: LU is (KL + LD) x N, PAPT aliases its
 *  rows KL.., PX aliases PB (suzerain/bsmbsm_solver.cpp:155-182). */
class bsmbsm_solver_zgbsv : public bsmbsm_solver {
public:
    bsmbsm_solver_zgbsv(const suzerain_bsmbsm &a, const specification_zgbsv &s, int nrhs)
        : bsmbsm_solver(a, s, nrhs)
    {
        if (!s.in_place()) throw std::invalid_argument("Invalid method in bsmbsm_solver_zgbsv");
        LU = cmatrix(a.KL + a.LD, a.N, complex_double(std::numeric_limits<double>::quiet_NaN()));
        PAPT = cmatrix::view(LU.data() + a.KL, a.LD, a.N, a.KL + a.LD);
        PX = cmatrix::view(PB.data(), a.N, nrhs, a.N);
    }

protected:
    int solve_hook(char trans, int nrhs) override
    {
        return suzerain_lapackext_zgbsv(&fact_, trans, A.N, A.KL, A.KU, nrhs, LU.data(),
                                        A.KL + A.LD, ipiv.data(), PB.data(), A.N);
    }
};

/** LAPACK's expert driver, out of place: PAPT is LD x N, LU (2KL + KU + 1) x N
 *  holds the factor; the first solve equilibrates (equil=true) or not and
 *  factors, later ones reuse the factor with fact 'F' until PAPT is supplied
 *  again (suzerain/bsmbsm_solver.cpp:184-291).  Every right hand side
 *  records equed, 1/rcond, ferr and berr. */
class bsmbsm_solver_zgbsvx : public bsmbsm_solver {
public:
    struct stat { char equed; double rcond_inv, ferr, berr; };
    std::vector<stat> stats;

    bsmbsm_solver_zgbsvx(const suzerain_bsmbsm &a, const specification_zgbsv &s, int nrhs)
        : bsmbsm_solver(a, s, nrhs), r_(a.N), c_(a.N), rwork_(a.N), ferr_(nrhs), berr_(nrhs),
          work_((size_t) 2 * a.N)
    {
        if (s.method() != SGB_METHOD_ZGBSVX)
            throw std::invalid_argument("Invalid method in bsmbsm_solver_zgbsvx");
        LU = cmatrix(2 * a.KL + a.KU + 1, a.N);
        PAPT = cmatrix(a.LD, a.N);
        PX = cmatrix(a.N, nrhs);
    }
    char equed() const { return equed_; }
    double rcond() const { return rcond_; }
    std::vector<std::string> summarize_statistics() const override
    {
        auto out = bsmbsm_solver::summarize_statistics();
        if (!stats.empty()) {
            double mr = 0, mf = 0, mb = 0;
            int eq = 0;
            for (const stat &x : stats) {
                mr = std::max(mr, x.rcond_inv); mf = std::max(mf, x.ferr); mb = std::max(mb, x.berr);
                eq += x.equed != 'N';
            }
            char buf[256];
            std::snprintf(buf, sizeof buf,
                          "solves %zu, equilibrated %d, max 1/rcond %.3g, max ferr %.3g, max berr %.3g",
                          stats.size(), eq, mr, mf, mb);
            out.push_back(buf);
        }
        return out;
    }

protected:
    int solve_hook(char trans, int nrhs) override
    {
        const int info = suzerain_lapack_zgbsvx(fact_, trans, A.N, A.KL, A.KU, nrhs, PAPT.data(),
                                                A.LD, LU.data(), 2 * A.KL + A.KU + 1, ipiv.data(),
                                                &equed_, r_.data(), c_.data(), PB.data(), A.N,
                                                PX.data(), A.N,
                                                &rcond_, ferr_.data(), berr_.data(), work_.data(),
                                                rwork_.data());
        fact_ = 'F';
        for (int j = 0; j < nrhs; ++j) stats.push_back({equed_, 1 / rcond_, ferr_[j], berr_[j]});
        return info;
    }

private:
    std::vector<double> r_, c_, rwork_, ferr_, berr_;
    std::vector<complex_double> work_;
    char equed_ = 'N';
    double rcond_ = 0;
};

/** Complex64 factor + complex128 refinement, out of place: PAPT is LD x N,
 *  LU (2KL + KU + 1) x N holds the factor (suzerain/bsmbsm_solver.cpp:293-414).
 *  Every right hand side runs the driver with the specification's siter,
 *  diter, tolsc and records them with fact, apprx, afrob and res. */
class bsmbsm_solver_zcgbsvx : public bsmbsm_solver {
public:
    struct stat { char fact; int apprx; double afrob; int siter, diter; double tolsc, res; };
    std::vector<stat> stats;

    bsmbsm_solver_zcgbsvx(const suzerain_bsmbsm &a, const specification_zgbsv &s, int nrhs)
        : bsmbsm_solver(a, s, nrhs), r_(a.N)
    {
        if (s.method() != SGB_METHOD_ZCGBSVX)
            throw std::invalid_argument("Invalid method in bsmbsm_solver_zcgbsvx");
        LU = cmatrix(2 * a.KL + a.KU + 1, a.N);
        PAPT = cmatrix(a.LD, a.N);
        PX = cmatrix(a.N, nrhs);
    }
    bsmbsm_solver &supplied_PAPT() override
    {
        afrob_ = -1;
        return bsmbsm_solver::supplied_PAPT();
    }
    std::vector<std::string> summarize_statistics() const override
    {
        auto out = bsmbsm_solver::summarize_statistics();
        if (!stats.empty()) {
            int s = 0, d = 0;
            double t = 0;
            for (const stat &x : stats) { s += x.siter; d += x.diter; t = std::max(t, x.tolsc); }
            char buf[256];
            std::snprintf(buf, sizeof buf, "solves %zu, mean siter %.3g, mean diter %.3g, max tolsc %.3g",
                          stats.size(), (double) s / stats.size(), (double) d / stats.size(), t);
            out.push_back(buf);
        }
        return out;
    }

protected:
    int solve_hook(char trans, int nrhs) override
    {
        int info = 0;
        for (int j = 0; !info && j < nrhs; ++j) {
            int siter = spec.siter(), diter = spec.diter();
            double tolsc = spec.tolsc(), res = 0;
            info = suzerain_lapackext_zcgbsvx(&fact_, &apprx_, spec.aiter(), trans, A.N, A.KL, A.KU,
                                              PAPT.data(), &afrob_, LU.data(), ipiv.data(),
                                              PB.data() + (size_t) j * A.N,
                                              PX.data() + (size_t) j * A.N, &siter, &diter, &tolsc,
                                              r_.data(), &res);
            stats.push_back({fact_, apprx_, afrob_, siter, diter, tolsc, res});
        }
        return info;
    }

private:
    std::vector<complex_double> r_;
    double afrob_ = -1;
};

inline std::unique_ptr<bsmbsm_solver> bsmbsm_solver::build(const suzerain_bsmbsm &A,
                                                           const specification_zgbsv &spec,
                                                           int nrhs)
{
    switch (spec.method()) {
    case SGB_METHOD_ZGBSV: return std::make_unique<bsmbsm_solver_zgbsv>(A, spec, nrhs);
    case SGB_METHOD_ZGBSVX: return std::make_unique<bsmbsm_solver_zgbsvx>(A, spec, nrhs);
    case SGB_METHOD_ZCGBSVX: return std::make_unique<bsmbsm_solver_zcgbsvx>(A, spec, nrhs);
    default:
        throw std::invalid_argument(std::string("bsmbsm_solver::build: method not provided: ") +
                                    std::string(spec));
    }
}

}  // namespace suzerain_gb300

#endif  // SUZERAIN_GB300_SOLVER_HPP
