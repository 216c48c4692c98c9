/*
 * The synthetic S x S block operator solved on every (kx, kz) pair, shared
 * verbatim by host code (generator, tests) and device code (fused assembly,
 * structured apply/residual) so both evaluate it bit for bit.
 *
 *   Block(e,f) = cM(e,f) M + cD1(e,f) D1 + cD2(e,f) D2
 *   cM(e,f)    = delta_ef - phi c_ef (kx^2 + kz^2) + i phi g_ef kx
 *   cD1(e,f)   = phi a_ef,      cD2(e,f) = phi b_ef
 *
 * M, D1, D2 are the 0th/1st/2nd derivative B-spline collocation matrices at
 * the Greville abscissae (suzerain/bsplineop.c:553-655), stored as LAPACK
 * bands with kl subdiagonals, ku superdiagonals and leading dimension ld.
 * This is the generator of the benchmark configurations; with g == 0 every
 * block is real-valued in complex storage, g != 0 exercises complex
 * coefficients the way suzerain/rholut_imexop.def:110-140 couples i*km.
 * Rows (e, p) for equations e in dirichlet_mask and p in {0, n-1} are
 * identity rows, as IsothermalPATPTEnforcer imposes no-slip walls
 * (apps/perfect/operator_hybrid_isothermal.cpp:471-515).
 */
#ifndef SGB_MODEL_H
#define SGB_MODEL_H

#include <math.h>
#include "suzerain_gb300.h"

#ifdef __CUDACC__
#define SGB_MODEL_HD __host__ __device__ __forceinline__
#else
#define SGB_MODEL_HD static inline
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sgb_coef { double re, im; } sgb_coef;

/** Coefficients of block (e, f) for one wavenumber pair and scale phi. */
SGB_MODEL_HD void sgb_block_coefs(const sgb_case *cs, int e, int f,
                                  double phi, double kx, double kz,
                                  sgb_coef *cM, sgb_coef *cD1, sgb_coef *cD2)
{
    const int ef = e * cs->S + f;
    const double ksq = fma(kx, kx, kz * kz);
    const double pc = phi * cs->c[ef];
    cM->re  = fma(-pc, ksq, e == f ? 1.0 : 0.0);
    cM->im  = (phi * cs->g[ef]) * kx;
    cD1->re = phi * cs->a[ef];
    cD1->im = 0.0;
    cD2->re = phi * cs->b[ef];
    cD2->im = 0.0;
}

/** Entry of block (e,f) at band offset k of M/D1/D2 given its coefficients. */
SGB_MODEL_HD void sgb_block_entry(sgb_coef cM, sgb_coef cD1, sgb_coef cD2,
                                  double m, double d1, double d2,
                                  double *re, double *im)
{
    *re = fma(cD2.re, d2, fma(cD1.re, d1, cM.re * m));
    *im = fma(cD2.im, d2, fma(cD1.im, d1, cM.im * m));
}

/** Is packed row I = p*S + e a Dirichlet identity row? */
SGB_MODEL_HD int sgb_is_dirichlet_row(const sgb_case *cs, int I)
{
    const int e = I % cs->S, p = I / cs->S;
    return ((cs->dirichlet_mask >> e) & 1u) && (p == 0 || p == cs->n - 1);
}

/* SMR91 low-storage Runge-Kutta coefficients, numerators over 480
 * (suzerain/lowstorage.hpp:1242-1305). */
#define SGB_SMR91_DENOM 480
static const int sgb_smr91_alpha[3] = { 29 * (480 / 96), -3 * (480 / 40), 1 * (480 / 6) };
static const int sgb_smr91_beta[3]  = { 37 * (480 / 160), 5 * (480 / 24), 1 * (480 / 6) };
static const int sgb_smr91_gamma[3] = { 8 * (480 / 15), 5 * (480 / 12), 3 * (480 / 4) };

#ifdef __cplusplus
}
#endif

#endif /* SGB_MODEL_H */
