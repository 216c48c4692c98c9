// Batched mixed-precision solve driver (zcgbsvx semantics), internal API.
#pragma once
#include "sgb_internal.h"

namespace sgb {
struct PhaseTimer;

// Per-system refinement state (device arrays of length nsys).
struct RefineState {
    double *res = nullptr, *lastres = nullptr, *tolconst = nullptr, *tol = nullptr,
           *tolsc = nullptr;
    int *status = nullptr, *siter = nullptr, *diter = nullptr, *info = nullptr;
    char *fact = nullptr;
    bool use_eps = false;
};

struct RefineProblem {
    int nsys = 0;
    FactorGeom g{};
    char trans = 'N';            // solve op(A) x = b
    char resid_trans = 'N';      // op used by the residual (reference gbmv maps 'C' to 'T')
    bool model = false;
    PackedSource src{};          // packed LD x N complex128 band (packc layout)
    ModelSource ms{};            // synthetic operator
    const double *gram = nullptr;// per-case band Gram sums (model ||A||_F)
    const double2 *b = nullptr; long long b_stride = 0;   // permuted RHS
    double2 *x = nullptr; long long x_stride = 0;         // permuted solution
    int aiter = 5, siter = 25, diter = 5;
    double tolsc = 1.0;
    double afrob_in = -1;        // ||A||_F supplied by the caller when >= 0
    int nslot64 = 1;             // complex128 factor slots for the fallback
    int *host_count = nullptr;   // pinned host int for list counts
    struct PhaseTimer *timer = nullptr;   // optional per-phase event timing
    // Capturable form (no host synchronization, no host-to-device copies):
    // the complex64 loop runs exactly graph_siter correction solves whose
    // grids are bounded by device counts (systems still refining then leave
    // as if siter were exhausted; graph_siter = siter + 1 is the reference's
    // own bound), and the complex128 fallback runs one chunk of at most
    // nslot64 systems for graph_diter iterations (diter + 2 is the
    // reference's bound); systems beyond the chunk are counted in
    // RefineOutputs::d_unserved (device int) and keep status "needs
    // complex128".
    bool graph = false;
    int graph_siter = 0, graph_diter = 0;
    // 0: the whole solve; 1: up to the complex64 factor (initial state,
    // norms, active list); 2: from the factor's results on (the caller ran
    // the factor, e.g. as part of a ragged batch)
    int stage = 0;
};

struct RefineOutputs {
    RefineState state;
    double *rnorm = nullptr, *xnorm = nullptr;
    double2 *r = nullptr;
    int *info32 = nullptr;
    double *afrob = nullptr;
    void *fac32 = nullptr, *fac64 = nullptr;     // row-panel factors (slot 0 first)
    int *ipiv32 = nullptr, *ipiv64 = nullptr;
    int single_iters = 0, double_iters = 0, n_double = 0;
    int *d_unserved = nullptr;   // capturable form: fallback systems beyond the chunk
};

size_t refine_workspace_bytes(const RefineProblem &P);
// Argument checks of the batched zcgbsvx entry points (capi.cu): 0 or the
// negative error code, with the library's last-error message set.
int zcgbsvx_batched_check(const char *who, int nsys, int N, int KL, int KU, char trans, int ldab,
                          const sgb_refine_spec *spec);
int refine_batched(const RefineProblem &P, void *workspace, size_t workspace_bytes,
                   RefineOutputs &out, cudaStream_t st);
struct RaggedDesc;
// Fills d with the complex64 factor's inputs and outputs of problem P in its
// workspace (model operator, trans 'N', siter >= 0 only).
int refine_ragged_desc(const RefineProblem &P, void *workspace, RaggedDesc &d);

}  // namespace sgb
