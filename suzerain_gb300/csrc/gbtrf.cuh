// Batched partial-pivot band LU (zgbtrf / cgbtrf semantics) for sm_103a.
//
// One warp factors one system.  The live part of the band -- logical rows
// j..j+KL (the pivot candidates of column j) by columns j..j+KL+KU -- sits in
// a shared-memory window of R = KL+1 row slots by C = KL+KU+1 circular
// columns.  Row interchanges are not performed physically: each slot carries
// the logical row it currently represents, and the interchange of LAPACK's
// zgbtf2 (swap rows j and p) becomes a relabel of two slots.  After the rank-1
// update the pivot slot is retired (its contents are row j of U) and refilled
// with the next row of A, entering pristine.
//
// Pivot choice reproduces reference LAPACK's IZAMAX exactly: largest
// |re|+|im| among candidates, the smallest logical row on ties, a NaN first
// candidate wins, NaNs elsewhere never do.  `ju` (the last column touched)
// follows zgbtf2 so the same entries are updated.
//
// Output layout per system ("row-panel factor"):
//   U:  N rows of UW = KL+KU+1 entries, U(j, j+k) at u[j*UW + k]
//   L:  N columns of KL multipliers, L(j+1+i, j) at l[j*KL + i]
//   ipiv[j] 1-based row interchanged with j (LAPACK convention), info as
//   zgbtrf: 0, or the 1-based index of the first exactly-zero pivot.
// The forward elimination y = L^{-1} P b of one right-hand side can be fused
// into the sweep (the RHS entry travels with its row slot).
#pragma once
#include "sgb_common.cuh"
#include "sgb_model.h"

namespace sgb {

struct FactorGeom {
    int N, KL, KU;        // banded system size and bandwidths
    __host__ __device__ int R() const { return KL + 1; }
    __host__ __device__ int C() const { return KL + KU + 1; }
    __host__ __device__ int UW() const { return KL + KU + 1; }
    // elements (complex) of one system's row-panel factor
    __host__ __device__ long long fac_elems() const
    { return (long long) N * (UW() + KL); }
};

// Row source: packed P A P^T in LAPACK band storage, complex128,
// A(i,j) at ab[off + KU + i - j + j*ldab] of system s (stride per system).
struct PackedSource {
    const double2 *ab;
    long long stride;
    int ldab, off;
    __device__ double2 entry(int s, int KU, int i, int j) const
    {
        return __ldg(ab + s * stride + off + KU + i - j + (long long) j * ldab);
    }
};

// Row source: the synthetic operator of sgb_model.h, assembled on the fly.
struct ModelSource {
    sgb_case cs;
    const double *kx, *kz;   // per system wavenumbers
    const int *case_of;      // per system case index (unused: one case)
    double phi;
    // (float) M, (float) D1, (float) D2 per band slot, for complex64 assembly
    const float4 *mdf = nullptr;
};

template <typename R>
struct SmemLayout {
    int R_, C_;
    __host__ __device__ size_t win_bytes() const { return (size_t) R_ * C_ * sizeof(cplx_t<R>); }
    __host__ __device__ size_t bytes(int S) const
    {
        return win_bytes() + 2 * R_ * sizeof(cplx_t<R>) + 2 * R_ * sizeof(int)
             + 3 * (size_t) S * S * sizeof(cplx_t<R>) + 16;
    }
};

}  // namespace sgb
