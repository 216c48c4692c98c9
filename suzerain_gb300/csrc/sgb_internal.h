// Internal launch interfaces shared by the .cu translation units.
#pragma once
#include <cuda_runtime.h>
#include "gbtrf.cuh"

namespace sgb {

// cudaFuncSetAttribute(MaxDynamicSharedMemorySize) once per (kernel, device,
// size): later launches (including those recorded into a CUDA graph) make no
// driver call for it.
cudaError_t smem_attr(const void *kernel, size_t bytes);

struct GbtrfArgs {
    char prec = 'Z';             // 'Z' complex128 factor, 'C' complex64
    FactorGeom g{};
    int nsys = 0;
    bool model = false;
    PackedSource src{};
    ModelSource ms{};
    void *fac = nullptr;         // row-panel factor, complex of prec
    long long fac_stride = 0;    // complex elements between systems
    int *ipiv = nullptr;         // nsys x N
    int *info = nullptr;         // nsys
    const double2 *rhs = nullptr;    // optional permuted RHS (fuses forward elimination)
    long long rhs_stride = 0;
    void *y = nullptr;           // forward-eliminated RHS (complex of prec)
    long long y_stride = 0;
    const int *sys_list = nullptr;   // optional subset of systems
    int nlist = 0;                   // grid size when sys_list is set
    const int *d_count = nullptr;    // optional device count bounding the list
    bool slot_mode = false;          // factor/ipiv/info indexed by list position
    int variant = 0;                 // 0 blocked (default), 1 unblocked, 2 blocked with lookahead
    int nb = 0;                      // panel width of the blocked kernel (4, 8, 16; 0 = default)
    int nw = 0;                      // warps per system of the blocked kernel (1, 2, 4; 0 = default)
    unsigned long long *prof = nullptr;  // optional per-phase cycle counters (6)
};
// One system of a ragged batch: the factor inputs and outputs of the plan
// it belongs to (complex64, assembled from the plan's model operator, the
// forward elimination of its right-hand side fused).
struct RaggedDesc {
    FactorGeom g;
    ModelSource ms;
    float2 *fac;
    long long fac_stride;
    int *ipiv, *info;
    const double2 *rhs;
    long long rhs_stride;
    float2 *y;
    long long y_stride;
    const int *sys_list;       // the plan's active list and its device count
    const int *d_count;
};
// The ragged factor over descriptors and (descriptor, list position) items
// in device memory, one CTA per item; kind (ragged_kind of every item's
// geometry) KB for the compile-time bandwidth instances (two warps), -25,
// -43, -44 for the generic ones (two warps KL <= 40, four warps KL <= 48,
// KL <= 56); smem the largest window's bytes.
cudaError_t launch_gbtrf_ragged(const RaggedDesc *descs, const int2 *items, int nitems, int kind,
                                size_t smem, cudaStream_t st);
int ragged_kind(const FactorGeom &g);
// The compile-time bandwidth of the complex64 phased factor's instance for
// g (KL = KU in 24, 34 and N % 4 == 0), or 0 for the generic instance;
// gbtrf_set_specialized(0) makes every geometry take the generic one.
int gbtrf_spec_band(const FactorGeom &g);
void gbtrf_set_specialized(int on);

cudaError_t launch_gbtrf(const GbtrfArgs &a, cudaStream_t st);
cudaError_t launch_gbtrf_blk(const GbtrfArgs &a, int nb, int nw, cudaStream_t st);
bool gbtrf_blk_supported(const FactorGeom &g, int nb, int nw);
// Fills nb / nw left at 0 from the tuned table, else the built-in default
// (model: rows assembled from the model operator rather than read from a
// packed band; the default warp count of the specialized instances differs).
void gbtrf_blk_choice(char prec, const FactorGeom &g, int &nb, int &nw, bool model = false);
void gbtrf_blk_set_choice(char prec, const FactorGeom &g, int nb, int nw);
size_t gbtrf_blk_smem_bytes(int prec_bytes, const FactorGeom &g, int S, int nb, int nw);
size_t gbtrf_smem_bytes(int prec_bytes, const FactorGeom &g, int S);

// Triangular solves with the row-panel factor.
struct GbtrsArgs {
    char prec = 'Z';
    char trans = 'N';
    FactorGeom g{};
    int nsys = 0;
    const void *fac = nullptr;
    long long fac_stride = 0;    // 0: every system solves with one factor and its pivots
    const int *ipiv = nullptr;
    bool fwd_done = false;       // input already forward-eliminated (trans N only)
    const double2 *b = nullptr;  // FP64 input when !yin
    const void *yin = nullptr;   // input in factor precision (fwd_done)
    long long b_stride = 0;
    double2 *x = nullptr;        // FP64 output
    long long x_stride = 0;
    bool accumulate = false;     // x += solution instead of x = solution
    const int *sys_list = nullptr;
    int nlist = 0;
    const int *d_count = nullptr;
    bool slot_mode = false;      // factor/ipiv indexed by list position
    const int *status = nullptr; // optional: skip systems whose status != status_want
    int status_want = 0;
    // optional natural-order scatter of the output: x[q(i)] instead of x[i]
    int unpermute_S = 0, unpermute_n = 0;
    // optional writable nsys x N buffer (complex of prec, row s at s*N) that
    // enables the quad-lane solve for trans 'N'; with fwd_done it must be yin
    void *ywork = nullptr;
};
cudaError_t launch_gbtrs(const GbtrsArgs &a, cudaStream_t st);

// Packed band residual r = b - op(A) x (FP64), with per-system norms.
struct ResidualArgs {
    char trans = 'N';
    int nsys = 0, N = 0, KL = 0, KU = 0;
    bool model = false;
    PackedSource src{};          // packed LD x N band (off = 0)
    ModelSource ms{};
    const double2 *b = nullptr; long long b_stride = 0;
    const double2 *x = nullptr; long long x_stride = 0;
    double2 *r = nullptr; long long r_stride = 0;
    double *rnorm2 = nullptr;    // ||r||_2 per system (may be null)
    double *xnorm2 = nullptr;    // ||x||_2 per system (may be null)
    const int *sys_list = nullptr;
    int nlist = 0;
    const int *d_count = nullptr;
    const int *status = nullptr;
    int status_want = 0;
};
cudaError_t launch_residual(const ResidualArgs &a, cudaStream_t st);

// Explicit operator apply of the synthetic model: y = P (M + phi L) u with
// Dirichlet rows zeroed; u natural order, y permuted order.
struct ApplyArgs {
    int nsys = 0;
    ModelSource ms{};
    const double2 *u = nullptr; long long u_stride = 0;
    double2 *y = nullptr; long long y_stride = 0;
    double beta = 0;             // y = A u + beta * y_prev (permuted) when nonzero
};
cudaError_t launch_model_apply(const ApplyArgs &a, cudaStream_t st);

// Batched complex128 expert driver (LAPACK zgbsvx semantics, one right-hand
// side per system).  Device pointers unless noted; per-system strides are
// in complex elements (b, x: N per system; ipiv, R, C: N per system).
struct GbsvxArgs {
    int nsys = 0;
    char fact = 'N';             // 'N' factor, 'E' equilibrate and factor, 'F' factor given
    char trans = 'N';
    FactorGeom g{};
    const double2 *ab = nullptr; // band rows 0..KL+KU (ld ldab)
    double2 *ab_out = nullptr;   // equilibrated band written back (may equal ab)
    int ldab = 0;
    long long ab_stride = 0;
    double2 *afb = nullptr;      // LAPACK gbtrf storage: input for 'F', output otherwise (may be null)
    int ldafb = 0;
    long long afb_stride = 0;
    int *ipiv = nullptr;         // input for 'F', output otherwise
    char *equed = nullptr;       // input for 'F', output otherwise
    double *R = nullptr, *C = nullptr;   // input for 'F', output for 'E'
    const double2 *b = nullptr;
    double2 *b_out = nullptr;    // scaled right-hand side (may equal b)
    double2 *x = nullptr;
    double *rcond = nullptr, *ferr = nullptr, *berr = nullptr, *rpvgrw = nullptr;  // host or device
    int *info = nullptr;         // device
};
int zgbsvx_batched(const GbsvxArgs &a, cudaStream_t st);
// Batched ZGBCON from gbtrf storage (device afb, ipiv); anorm and rcond on
// the host, one per system.
int zgbcon_batched(char norm, int nsys, const FactorGeom &g, const double2 *afb, int ldafb,
                   long long afb_stride, const int *ipiv, const double *anorm, double *rcond,
                   cudaStream_t st);

}  // namespace sgb
