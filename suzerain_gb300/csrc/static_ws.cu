// sgb_zcgbsvx_batched_static: the batched mixed-precision band solve for
// callers that cannot allocate device memory.
//
// Some hosts own every byte of device memory: a simulation code that reserves
// its whole HBM budget up front in its own arena, or a solver loop that must
// not call into the driver's allocator once time stepping has begun (a
// cudaMalloc there can fail against the reserved budget, fragment the arena,
// or stall the loop while the driver maps pages).  sgb_zcgbsvx_batched cannot
// serve them because it allocates its workspace on first use.  This variant
// runs the same kernels with their scratch memory taken from a fixed array
// compiled into the library instead.
//
// The array is SGB_STATIC_WS_BYTES (64 MiB) of file-scope __device__ storage:
// every GPU that loads this library holds it until the process exits, whether
// or not this entry point is called.  A problem whose workspace exceeds it
// (refine_workspace_bytes with SGB_STATIC_SLOTS64 complex128 fallback slots,
// through which the fallback systems pass in chunks; at N = 960,
// KL = KU = 34 that is 6.3 MB plus about 0.82 MB per system, so up to 74
// systems per call) is rejected.
#include "suzerain_gb300.h"
#include "sgb_internal.h"
#include "sgb_refine.h"

#include <cctype>
#include <cstdio>
#include <mutex>

using namespace sgb;

#define SGB_STATIC_WS_BYTES (64ull << 20)
#define SGB_STATIC_SLOTS64 4
#define SGB_STATIC_MAX_DEVICES 64

static __device__ __align__(256) unsigned char g_sgb_static_ws[SGB_STATIC_WS_BYTES];

namespace {
std::mutex g_static_mu;
// Device address of g_sgb_static_ws per device, looked up once with that
// device current.  The host-side name g_sgb_static_ws is a stand-in only and
// must never be handed to a kernel.
void *g_static_addr[SGB_STATIC_MAX_DEVICES];
// Pageable host landing spot for the driver's active-list counts.
int g_static_count[SGB_STATIC_MAX_DEVICES];

int static_fail(const char *msg)
{
    sgb_set_error(cudaErrorInvalidValue, msg, __FILE__, __LINE__);
    return -1;
}
}  // namespace

__global__ void k_static_report(int nsys, RefineState st, int *info, int *siter, int *diter,
                                double *res, double *tolsc, char *fact)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsys) return;
    if (info) info[s] = st.info[s];
    if (siter) siter[s] = st.siter[s];
    if (diter) diter[s] = st.diter[s];
    if (res) res[s] = st.res[s];
    if (tolsc) tolsc[s] = st.tolsc[s];
    if (fact) fact[s] = st.fact[s];
}

extern "C" int sgb_zcgbsvx_batched_static(int nsys, int N, int KL, int KU, char trans,
                                          const void *ab, int ldab, long long ab_stride,
                                          const void *b, void *x, const sgb_refine_spec *spec,
                                          const sgb_refine_report *report, void *stream)
{
    trans = (char) std::toupper((unsigned char) trans);
    const int bad = zcgbsvx_batched_check("sgb_zcgbsvx_batched_static", nsys, N, KL, KU, trans,
                                          ldab, spec);
    if (bad) return bad;
    if (nsys == 0) return 0;

    RefineProblem P;
    P.nsys = nsys; P.g = {N, KL, KU}; P.trans = trans;
    P.resid_trans = (trans == 'C') ? 'T' : trans;   // reference gbmv: 'C' == 'T'
    P.model = false;
    P.src = {reinterpret_cast<const double2 *>(ab), ab_stride, ldab, 0};
    P.b = reinterpret_cast<const double2 *>(b); P.b_stride = N;
    P.x = reinterpret_cast<double2 *>(x); P.x_stride = N;
    P.aiter = spec->aiter; P.siter = spec->siter; P.diter = spec->diter; P.tolsc = spec->tolsc;
    // complex128 fallback slots: the fallback runs in chunks of this many
    // systems, so a few slots serve any number of fallback systems
    P.nslot64 = nsys < SGB_STATIC_SLOTS64 ? nsys : SGB_STATIC_SLOTS64;
    const size_t need = refine_workspace_bytes(P);
    if (need > SGB_STATIC_WS_BYTES) {
        char msg[256];
        std::snprintf(msg, sizeof msg,
                      "sgb_zcgbsvx_batched_static: %d systems of N=%d, KL=%d, KU=%d need %zu bytes "
                      "of scratch; the static workspace holds %llu bytes",
                      nsys, N, KL, KU, need, (unsigned long long) SGB_STATIC_WS_BYTES);
        return static_fail(msg);
    }

    std::lock_guard<std::mutex> lk(g_static_mu);
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return sgb_set_error(e, "cudaGetDevice", __FILE__, __LINE__);
    if (dev < 0 || dev >= SGB_STATIC_MAX_DEVICES)
        return static_fail("sgb_zcgbsvx_batched_static: device ordinal out of range");
    if (!g_static_addr[dev]) {
        // One-time set-up on this device (the current device).
        void *ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_sgb_static_ws);
        if (e != cudaSuccess || !ptr)
            return sgb_set_error(e != cudaSuccess ? e : cudaErrorInvalidSymbol,
                                 "cudaGetSymbolAddress(g_sgb_static_ws)", __FILE__, __LINE__);
        g_static_addr[dev] = ptr;
    }
    P.host_count = &g_static_count[dev];

    // The driver initialises everything it reads (counters are cleared, x is
    // zeroed, r is copied from b), so the previous call's contents of the
    // shared array never leak into this one.
    RefineOutputs out;
    const int rc = refine_batched(P, g_static_addr[dev], SGB_STATIC_WS_BYTES, out,
                                  (cudaStream_t) stream);
    if (rc) return sgb_set_error((cudaError_t) rc, "refine_batched (static workspace)", __FILE__, __LINE__);
    if (report) {
        k_static_report<<<(nsys + 127) / 128, 128, 0, (cudaStream_t) stream>>>(
            nsys, out.state, report->info, report->siter, report->diter, report->res,
            report->tolsc, report->fact);
        e = cudaGetLastError();
        if (e != cudaSuccess) return sgb_set_error(e, "k_static_report", __FILE__, __LINE__);
    }
    return 0;
}
