// C-ABI of the batched device API: error reporting, batched gbtrf/gbtrs,
// batched zcgbsvx, and the resident-batch plan driving whole substeps.
#include "suzerain_gb300.h"
#include "sgb_internal.h"
#include "sgb_refine.h"
#include "sgb_timer.h"

#include <algorithm>
#include <map>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

using namespace sgb;

namespace sgb { std::atomic<long long> g_launches{0}; }

namespace {
thread_local std::string g_err;
}

extern "C" long long sgb_launch_count(void) { return g_launches.load(); }

int sgb_set_error(cudaError_t e, const char *what, const char *file, int line)
{
    char buf[512];
    std::snprintf(buf, sizeof buf, "%s: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
    g_err = buf;
    return (int) e;
}

static int fail(const char *msg, int code = -1)
{
    g_err = msg;
    return code;
}

extern "C" const char *sgb_last_error(void) { return g_err.c_str(); }

extern "C" int sgb_device_ok(void)
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return sgb_set_error(e, "cudaGetDevice", __FILE__, __LINE__);
    int major = 0, minor = 0;
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
    if (major != 10 || minor != 3) return fail("device is not compute capability 10.3 (GB300)", -2);
    return 0;
}

extern "C" long long sgb_factor_elems(int N, int KL, int KU)
{
    return FactorGeom{N, KL, KU}.fac_elems();
}

static bool geom_ok(int N, int KL, int KU)
{
    return N >= 1 && KL >= 0 && KU >= 0 && KL + 1 <= 64 && KL + KU + 1 <= 192;
}

namespace sgb {
cudaError_t smem_attr(const void *kernel, size_t bytes)
{
    static std::mutex mu;
    static std::map<std::pair<const void *, int>, size_t> done;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(mu);
    size_t &have = done[{kernel, dev}];
    if (bytes <= have) return cudaSuccess;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) bytes);
    if (e == cudaSuccess) have = bytes;
    return e;
}
}  // namespace sgb

extern "C" int sgb_gbtrf_batched(char prec, int nsys, int N, int KL, int KU, const void *ab,
                                 int ldab, long long ab_stride, void *fac, int *ipiv,
                                 int *info, void *stream)
{
    if (prec != 'Z' && prec != 'C') return fail("sgb_gbtrf_batched: prec must be 'Z' or 'C'");
    if (!geom_ok(N, KL, KU) || ldab < KL + KU + 1 || nsys < 0)
        return fail("sgb_gbtrf_batched: bad geometry");
    GbtrfArgs a;
    a.prec = prec; a.g = {N, KL, KU}; a.nsys = nsys;
    a.src = {reinterpret_cast<const double2 *>(ab), ab_stride, ldab, 0};
    a.fac = fac; a.fac_stride = a.g.fac_elems(); a.ipiv = ipiv; a.info = info;
    count_launch(1);
    SGB_CUDA_TRY(launch_gbtrf(a, (cudaStream_t) stream));
    return 0;
}

extern "C" int sgb_gbtrf_batched_ex(char prec, int nsys, int N, int KL, int KU, const void *ab,
                                    int ldab, long long ab_stride, void *fac, int *ipiv,
                                    int *info, int variant, int nb, int nw, void *stream)
{
    if (prec != 'Z' && prec != 'C') return fail("sgb_gbtrf_batched_ex: prec must be 'Z' or 'C'");
    if (!geom_ok(N, KL, KU) || ldab < KL + KU + 1 || nsys < 0)
        return fail("sgb_gbtrf_batched_ex: bad geometry");
    if (variant < 0 || variant > 2) return fail("sgb_gbtrf_batched_ex: variant must be 0, 1 or 2");
    if (variant != 1) {
        gbtrf_blk_choice(prec, {N, KL, KU}, nb, nw);
        if (nw < 0) { variant = 2; nw = -nw; }
        if (!gbtrf_blk_supported({N, KL, KU}, nb, nw))
            return fail("sgb_gbtrf_batched_ex: blocked kernel needs nb in {4,8,16}, nw in {1,2,4}, "
                        "KL <= 52/56/64 for nw 1/2/4 and N < 65536 (nw 3: nb 4, KL = KU = 24 or "
                        "34, N a multiple of 4)");
    }
    GbtrfArgs a;
    a.prec = prec; a.g = {N, KL, KU}; a.nsys = nsys;
    a.src = {reinterpret_cast<const double2 *>(ab), ab_stride, ldab, 0};
    a.fac = fac; a.fac_stride = a.g.fac_elems(); a.ipiv = ipiv; a.info = info;
    a.variant = variant; a.nb = nb; a.nw = nw;
    count_launch(1);
    SGB_CUDA_TRY(launch_gbtrf(a, (cudaStream_t) stream));
    return 0;
}

extern "C" int sgb_gbtrf_phase_cycles(char prec, int nsys, int N, int KL, int KU, const void *ab,
                                      int ldab, long long ab_stride, void *fac, int *ipiv,
                                      int *info, int nb, int nw, unsigned long long *cycles_dev,
                                      void *stream)
{
    if (prec != 'Z' && prec != 'C') return fail("sgb_gbtrf_phase_cycles: prec must be 'Z' or 'C'");
    gbtrf_blk_choice(prec, {N, KL, KU}, nb, nw);
    const int variant = nw < 0 ? 2 : 0;     // negative nw: the lookahead form
    if (nw < 0) nw = -nw;
    if (!geom_ok(N, KL, KU) || ldab < KL + KU + 1 || !gbtrf_blk_supported({N, KL, KU}, nb, nw))
        return fail("sgb_gbtrf_phase_cycles: bad geometry");
    GbtrfArgs a;
    a.prec = prec; a.g = {N, KL, KU}; a.nsys = nsys;
    a.src = {reinterpret_cast<const double2 *>(ab), ab_stride, ldab, 0};
    a.fac = fac; a.fac_stride = a.g.fac_elems(); a.ipiv = ipiv; a.info = info;
    a.variant = variant; a.nb = nb; a.nw = nw; a.prof = cycles_dev;
    count_launch(1);
    SGB_CUDA_TRY(launch_gbtrf(a, (cudaStream_t) stream));
    return 0;
}

extern "C" int sgb_gbtrf_set_shape(char prec, int N, int KL, int KU, int nb, int nw)
{
    if (prec != 'Z' && prec != 'C') return fail("sgb_gbtrf_set_shape: prec must be 'Z' or 'C'");
    if (!geom_ok(N, KL, KU) || nw == -1 || nw == -3 || (nw == 3 && prec != 'C') ||
        !gbtrf_blk_supported({N, KL, KU}, nb, nw < 0 ? -nw : nw))
        return fail("sgb_gbtrf_set_shape: unsupported (N, KL, KU, nb, nw)");
    gbtrf_blk_set_choice(prec, {N, KL, KU}, nb, nw);
    return 0;
}

extern "C" int sgb_gbtrf_get_shape(char prec, int N, int KL, int KU, int *nb, int *nw)
{
    int b = 0, w = 0;
    gbtrf_blk_choice(prec, {N, KL, KU}, b, w);
    if (nb) *nb = b;
    if (nw) *nw = w;
    return 0;
}

extern "C" int sgb_gbtrs_batched(char prec, char trans, int nsys, int N, int KL, int KU,
                                 const void *fac, const int *ipiv, const void *b, void *x,
                                 void *stream)
{
    trans = (char) toupper(trans);
    if (prec != 'Z' && prec != 'C') return fail("sgb_gbtrs_batched: prec must be 'Z' or 'C'");
    if (trans != 'N' && trans != 'T' && trans != 'C') return fail("sgb_gbtrs_batched: bad trans");
    if (!geom_ok(N, KL, KU) || nsys < 0) return fail("sgb_gbtrs_batched: bad geometry");
    GbtrsArgs a;
    a.prec = prec; a.trans = trans; a.g = {N, KL, KU}; a.nsys = nsys; a.fac = fac;
    a.fac_stride = a.g.fac_elems(); a.ipiv = ipiv;
    a.b = reinterpret_cast<const double2 *>(b); a.b_stride = N;
    a.x = reinterpret_cast<double2 *>(x); a.x_stride = N;
    SGB_CUDA_TRY(launch_gbtrs(a, (cudaStream_t) stream));
    return 0;
}

extern "C" int sgb_gbtrs_batched_ws(char prec, char trans, int nsys, int N, int KL, int KU,
                                    const void *fac, const int *ipiv, const void *b, void *x,
                                    void *ywork, void *stream)
{
    trans = (char) toupper(trans);
    if (prec != 'Z' && prec != 'C') return fail("sgb_gbtrs_batched_ws: prec must be 'Z' or 'C'");
    if (trans != 'N' && trans != 'T' && trans != 'C') return fail("sgb_gbtrs_batched_ws: bad trans");
    if (!geom_ok(N, KL, KU) || nsys < 0) return fail("sgb_gbtrs_batched_ws: bad geometry");
    GbtrsArgs a;
    a.prec = prec; a.trans = trans; a.g = {N, KL, KU}; a.nsys = nsys; a.fac = fac;
    a.fac_stride = a.g.fac_elems(); a.ipiv = ipiv;
    a.b = reinterpret_cast<const double2 *>(b); a.b_stride = N;
    a.x = reinterpret_cast<double2 *>(x); a.x_stride = N;
    a.ywork = ywork;
    SGB_CUDA_TRY(launch_gbtrs(a, (cudaStream_t) stream));
    return 0;
}

// One factor, many right-hand sides: the wavenumber-independent operator
// factored once and solved for every wavenumber's right-hand side
// (apps/perfect/operator_hybrid_isothermal.cpp:691-760, bsmbsm_solver with
// nrhs > 1 and a reused factor, suzerain/bsmbsm_solver.cpp:80-102).
extern "C" int sgb_gbtrs_shared(char prec, char trans, int nrhs, int N, int KL, int KU,
                                const void *fac, const int *ipiv, const void *b, long long ldb,
                                void *x, long long ldx, void *ywork, void *stream)
{
    trans = (char) toupper(trans);
    if (prec != 'Z' && prec != 'C') return fail("sgb_gbtrs_shared: prec must be 'Z' or 'C'");
    if (trans != 'N' && trans != 'T' && trans != 'C') return fail("sgb_gbtrs_shared: bad trans");
    if (!geom_ok(N, KL, KU) || nrhs < 0) return fail("sgb_gbtrs_shared: bad geometry");
    if (ldb < N || ldx < N) return fail("sgb_gbtrs_shared: ldb and ldx must be >= N");
    GbtrsArgs a;
    a.prec = prec; a.trans = trans; a.g = {N, KL, KU}; a.nsys = nrhs; a.fac = fac;
    a.fac_stride = 0; a.ipiv = ipiv;
    a.b = reinterpret_cast<const double2 *>(b); a.b_stride = ldb;
    a.x = reinterpret_cast<double2 *>(x); a.x_stride = ldx;
    a.ywork = ywork;
    SGB_CUDA_TRY(launch_gbtrs(a, (cudaStream_t) stream));
    return 0;
}

template <typename T2>
__global__ void k_factor_to_lapack(int nsys, FactorGeom g, const T2 *__restrict__ fac,
                                   T2 *__restrict__ ab)
{
    const int s = blockIdx.y;
    const int j = blockIdx.x * blockDim.y + threadIdx.y;
    if (s >= nsys || j >= g.N) return;
    const int KL = g.KL, UW = g.UW(), KV = UW - 1, LDAB = 2 * KL + g.KU + 1;
    const T2 *fu = fac + s * g.fac_elems();
    const T2 *fl = fu + (long long) g.N * UW;
    T2 *col = ab + (long long) s * LDAB * g.N;
    // column j of LAPACK storage: U(j-KV..j, j) rows 0..KV, L(j+1..j+KL, j) rows KV+1..
    for (int r = threadIdx.x; r < LDAB; r += blockDim.x) {
        T2 v; v.x = 0; v.y = 0;
        if (r <= KV) {
            const int i = j - KV + r;       // U(i, j) = fu[i*UW + (j - i)]
            if (i >= 0) v = fu[(long long) i * UW + (j - i)];
        } else {
            const int i = r - KV;           // L(j+i, j)
            if (j + i < g.N) v = fl[(long long) j * KL + i - 1];
        }
        col[(long long) j * LDAB + r] = v;
    }
}

extern "C" int sgb_factor_to_lapack(char prec, int nsys, int N, int KL, int KU,
                                    const void *fac, void *ab, void *stream)
{
    if (!geom_ok(N, KL, KU)) return fail("sgb_factor_to_lapack: bad geometry");
    if (nsys == 0) return 0;
    FactorGeom g{N, KL, KU};
    dim3 blk(32, 4), grd((N + 3) / 4, nsys);
    if (prec == 'Z')
        k_factor_to_lapack<double2><<<grd, blk, 0, (cudaStream_t) stream>>>(
            nsys, g, (const double2 *) fac, (double2 *) ab);
    else if (prec == 'C')
        k_factor_to_lapack<float2><<<grd, blk, 0, (cudaStream_t) stream>>>(
            nsys, g, (const float2 *) fac, (float2 *) ab);
    else return fail("sgb_factor_to_lapack: prec must be 'Z' or 'C'");
    SGB_CUDA_TRY(cudaGetLastError());
    return 0;
}

// ---------------------------------------------------------------------------
// Small elementwise kernels
// ---------------------------------------------------------------------------
// dir 'N': dst[i] = src[q(i)]  (natural -> permuted); 'T': dst[i] = src[qinv(i)]
__global__ void k_permute(long long nsys, int S, int n, const double2 *__restrict__ src,
                          double2 *__restrict__ dst, int to_natural)
{
    const long long N = (long long) S * n;
    const long long t = (long long) blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nsys * N) return;
    const long long s = t / N;
    const int i = (int) (t - s * N);
    const int o = to_natural ? (i % n) * S + i / n : (i % S) * n + i / S;
    dst[t] = src[s * N + o];
}

// ---------------------------------------------------------------------------
// Batched zcgbsvx over packed bands
// ---------------------------------------------------------------------------
namespace {
struct Scratch {
    void *p = nullptr; size_t bytes = 0;
    int *hcount = nullptr;
    std::mutex mu;
    int ensure(size_t b)
    {
        if (!hcount) {
            cudaError_t e = cudaMallocHost(&hcount, sizeof(int));
            if (e != cudaSuccess) return sgb_set_error(e, "cudaMallocHost", __FILE__, __LINE__);
        }
        if (b <= bytes) return 0;
        if (p) cudaFree(p);
        p = nullptr; bytes = 0;
        cudaError_t e = cudaMalloc(&p, b);
        if (e != cudaSuccess) return sgb_set_error(e, "cudaMalloc(zcgbsvx workspace)", __FILE__, __LINE__);
        bytes = b;
        return 0;
    }
};
Scratch g_zc;
}  // namespace

__global__ void k_report_copy(int nsys, RefineState st, int *info, int *siter, int *diter,
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

namespace sgb {
// Argument checks shared by the batched zcgbsvx entry points: 0, or the
// negative code with the message set (-4 trans, -5 geometry or ldab,
// -16 tolsc, -99 siter and diter both negative, -1 nsys < 0).
int zcgbsvx_batched_check(const char *who, int nsys, int N, int KL, int KU, char trans, int ldab,
                          const sgb_refine_spec *spec)
{
    std::string w(who);
    if (trans != 'N' && trans != 'T' && trans != 'C') return fail((w + ": bad trans").c_str(), -4);
    if (!geom_ok(N, KL, KU) || ldab < KL + KU + 1) return fail((w + ": bad geometry").c_str(), -5);
    if (!spec || spec->tolsc < 0) return fail((w + ": bad tolsc").c_str(), -16);
    if (spec->siter < 0 && spec->diter < 0) return fail((w + ": siter and diter < 0").c_str(), -99);
    if (nsys < 0) return fail((w + ": nsys < 0").c_str(), -1);
    return 0;
}
}  // namespace sgb

extern "C" int sgb_zcgbsvx_batched(int nsys, int N, int KL, int KU, char trans, const void *ab,
                                   int ldab, long long ab_stride, const void *b, void *x,
                                   const sgb_refine_spec *spec, const sgb_refine_report *report,
                                   void *stream)
{
    trans = (char) toupper(trans);
    const int bad = zcgbsvx_batched_check("sgb_zcgbsvx_batched", nsys, N, KL, KU, trans, ldab, spec);
    if (bad) return bad;
    if (nsys == 0) return 0;
    std::lock_guard<std::mutex> lk(g_zc.mu);
    RefineProblem P;
    P.nsys = nsys; P.g = {N, KL, KU}; P.trans = trans;
    P.resid_trans = (trans == 'C') ? 'T' : trans;   // reference gbmv: 'C' == 'T'
    P.model = false;
    P.src = {reinterpret_cast<const double2 *>(ab), ab_stride, ldab, 0};
    P.b = reinterpret_cast<const double2 *>(b); P.b_stride = N;
    P.x = reinterpret_cast<double2 *>(x); P.x_stride = N;
    P.aiter = spec->aiter; P.siter = spec->siter; P.diter = spec->diter; P.tolsc = spec->tolsc;
    P.nslot64 = std::min(nsys, 4096);
    int rc = g_zc.ensure(refine_workspace_bytes(P));
    if (rc) return rc;
    P.host_count = g_zc.hcount;
    RefineOutputs out;
    rc = refine_batched(P, g_zc.p, g_zc.bytes, out, (cudaStream_t) stream);
    if (rc) return sgb_set_error((cudaError_t) rc, "refine_batched", __FILE__, __LINE__);
    if (report) {
        k_report_copy<<<(nsys + 127) / 128, 128, 0, (cudaStream_t) stream>>>(
            nsys, out.state, report->info, report->siter, report->diter, report->res,
            report->tolsc, report->fact);
        SGB_CUDA_TRY(cudaGetLastError());
    }
    return 0;
}

// ---------------------------------------------------------------------------
// Plan memory: a stream-ordered pool that keeps freed blocks, so that plans
// created and destroyed in turn (a serving loop admitting and retiring cases)
// reuse device memory instead of paying cudaMalloc / cudaFree each time.  A
// plan's blocks return to the pool only after the work it issued completes:
// its frees are ordered after an event recorded at the end of each of its
// calls (per stream), or after a device synchronization when the plan was
// ever recorded into a CUDA graph (a graph may be replayed at any time).
// ---------------------------------------------------------------------------
namespace {
struct PlanPool {
    std::mutex mu;
    cudaMemPool_t pool = nullptr;
    cudaStream_t st = nullptr;
    int dev = -1;
    cudaError_t init()
    {
        int d = 0;
        cudaError_t e = cudaGetDevice(&d);
        if (e != cudaSuccess) return e;
        if (pool && d == dev) return cudaSuccess;
        if (pool) return cudaErrorInvalidDevice;     // one device per process
        cudaMemPoolProps props;
        std::memset(&props, 0, sizeof props);
        props.allocType = cudaMemAllocationTypePinned;
        props.handleTypes = cudaMemHandleTypeNone;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = d;
        e = cudaMemPoolCreate(&pool, &props);
        if (e != cudaSuccess) { pool = nullptr; return e; }
        unsigned long long keep = ~0ull;
        e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        if (e != cudaSuccess) return e;
        dev = d;
        return cudaSuccess;
    }
    cudaError_t alloc(void **p, size_t bytes)
    {
        std::lock_guard<std::mutex> lk(mu);
        cudaError_t e = init();
        if (e != cudaSuccess) return e;
        e = cudaMallocFromPoolAsync(p, bytes, pool, st);
        if (e == cudaErrorMemoryAllocation) {          // give cached blocks back, retry once
            cudaGetLastError();
            cudaStreamSynchronize(st);
            cudaMemPoolTrimTo(pool, 0);
            e = cudaMallocFromPoolAsync(p, bytes, pool, st);
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);   // usable from any stream
        return e;
    }
};
PlanPool g_pool;
}  // namespace

extern "C" int sgb_plan_pool_trim(size_t keep_bytes)
{
    std::lock_guard<std::mutex> lk(g_pool.mu);
    if (!g_pool.pool) return 0;
    SGB_CUDA_TRY(cudaStreamSynchronize(g_pool.st));
    SGB_CUDA_TRY(cudaMemPoolTrimTo(g_pool.pool, keep_bytes));
    return 0;
}

// ---------------------------------------------------------------------------
// Plan: one resident case
// ---------------------------------------------------------------------------
struct sgb_plan {
    sgb_case hc{};            // scalars of the case
    sgb_case dc{};            // device copy
    int nsys = 0, N = 0, KL = 0, KU = 0, nslot64 = 1;
    double *kx = nullptr, *kz = nullptr, *gram = nullptr;
    double *bands = nullptr, *coefs = nullptr;
    float4 *bandf = nullptr;  // (float) M, D1, D2 per band slot
    double2 *b = nullptr, *x = nullptr, *u_stage = nullptr;
    double phi_imp_last = 0;
    // complex128 path
    void *fac64 = nullptr; int *ipiv64 = nullptr, *info64 = nullptr; double2 *y64 = nullptr;
    // mixed path
    void *rws = nullptr; size_t rws_bytes = 0;
    RefineOutputs last{};
    char last_method = 0;
    int *hcount = nullptr;
    size_t dev_bytes = 0;
    PhaseTimer timer;
    std::vector<void *> allocs;
    std::mutex mu;

    std::vector<std::pair<cudaStream_t, cudaEvent_t>> done;   // end of the last call per stream
    bool captured = false;                                     // ever recorded into a graph

    int dalloc(void **p, size_t bytes, const char *what)
    {
        cudaError_t e = g_pool.alloc(p, bytes);
        if (e != cudaSuccess) return sgb_set_error(e, what, __FILE__, __LINE__);
        allocs.push_back(*p);
        dev_bytes += bytes;
        return 0;
    }
    // Marks the end of a call's work on stream st (frees wait for it).
    void note(cudaStream_t st)
    {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) { cudaGetLastError(); captured = true; return; }
        if (cs != cudaStreamCaptureStatusNone) { captured = true; return; }
        for (auto &d : done)
            if (d.first == st) { cudaEventRecord(d.second, st); return; }
        cudaEvent_t ev = nullptr;
        if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            captured = true;       // fall back to a device synchronization at destroy
            return;
        }
        cudaEventRecord(ev, st);
        done.push_back({st, ev});
    }
    ModelSource ms(double phi) const
    {
        ModelSource m;
        m.cs = dc; m.kx = kx; m.kz = kz; m.case_of = nullptr; m.phi = phi; m.mdf = bandf;
        return m;
    }
};

// Gram sums of the bands for the analytic ||A||_F (see k_afrob_model).
static void band_gram(const sgb_case &c, double *G)
{
    const int n = c.n, ld = c.ld;
    std::memset(G, 0, 18 * sizeof(double));
    for (int j = 0; j < n; ++j)
        for (int i = std::max(0, j - c.ku); i <= std::min(n - 1, j + c.kl); ++i) {
            const size_t k = (size_t) j * ld + c.ku + i - j;
            const double m = c.M[k], d1 = c.D1[k], d2 = c.D2[k];
            const double v[6] = {m * m, m * d1, m * d2, d1 * d1, d1 * d2, d2 * d2};
            for (int t = 0; t < 6; ++t) {
                G[t] += v[t];
                if (i == 0) G[6 + t] += v[t];
                if (i == n - 1) G[12 + t] += v[t];
            }
        }
}

extern "C" sgb_plan *sgb_plan_create(const sgb_case *hcase, int nsys, const double *kx,
                                     const double *kz, int max_double_slots)
{
    if (!hcase || nsys < 1 || !kx || !kz) { fail("sgb_plan_create: bad arguments"); return nullptr; }
    const sgb_case &c = *hcase;
    if (c.S < 1 || c.S > 8 || c.n < 2 || c.kl < 0 || c.ku < 0 || c.ld < c.kl + 1 + c.ku) {
        fail("sgb_plan_create: bad case geometry");
        return nullptr;
    }
    sgb_plan *p = new (std::nothrow) sgb_plan;
    if (!p) { fail("sgb_plan_create: out of host memory"); return nullptr; }
    p->hc = c;
    p->nsys = nsys;
    p->N = c.S * c.n;
    p->KL = c.S * (c.kl + 1) - 1;
    p->KU = c.S * (c.ku + 1) - 1;
    if (!geom_ok(p->N, p->KL, p->KU)) { fail("sgb_plan_create: bandwidth too large"); delete p; return nullptr; }
    p->nslot64 = std::max(1, std::min(nsys, max_double_slots > 0 ? max_double_slots : nsys));
    const size_t nb = (size_t) c.ld * c.n, SS = (size_t) c.S * c.S;
    int rc = 0;
    rc |= p->dalloc((void **) &p->bands, 3 * nb * sizeof(double), "cudaMalloc(bands)");
    rc |= p->dalloc((void **) &p->bandf, nb * sizeof(float4), "cudaMalloc(bandf)");
    rc |= p->dalloc((void **) &p->coefs, 4 * SS * sizeof(double), "cudaMalloc(coefs)");
    rc |= p->dalloc((void **) &p->kx, nsys * sizeof(double), "cudaMalloc(kx)");
    rc |= p->dalloc((void **) &p->kz, nsys * sizeof(double), "cudaMalloc(kz)");
    rc |= p->dalloc((void **) &p->gram, 18 * sizeof(double), "cudaMalloc(gram)");
    rc |= p->dalloc((void **) &p->b, (size_t) nsys * p->N * sizeof(double2), "cudaMalloc(b)");
    rc |= p->dalloc((void **) &p->x, (size_t) nsys * p->N * sizeof(double2), "cudaMalloc(x)");
    if (rc) { sgb_plan_destroy(p); return nullptr; }
    cudaError_t e = cudaMallocHost(&p->hcount, sizeof(int));
    if (e != cudaSuccess) { sgb_set_error(e, "cudaMallocHost", __FILE__, __LINE__); sgb_plan_destroy(p); return nullptr; }
    double G[18];
    band_gram(c, G);
    e = cudaMemcpy(p->bands, c.M, nb * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(p->bands + nb, c.D1, nb * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(p->bands + 2 * nb, c.D2, nb * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        std::vector<float4> bf(nb);
        for (size_t k = 0; k < nb; ++k)
            bf[k] = make_float4((float) c.M[k], (float) c.D1[k], (float) c.D2[k], 0.0f);
        e = cudaMemcpy(p->bandf, bf.data(), nb * sizeof(float4), cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) e = cudaMemcpy(p->coefs, c.a, SS * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(p->coefs + SS, c.b, SS * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(p->coefs + 2 * SS, c.c, SS * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(p->coefs + 3 * SS, c.g, SS * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(p->kx, kx, nsys * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(p->kz, kz, nsys * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(p->gram, G, sizeof G, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) { sgb_set_error(e, "cudaMemcpy(plan)", __FILE__, __LINE__); sgb_plan_destroy(p); return nullptr; }
    p->dc = c;
    p->dc.M = p->bands; p->dc.D1 = p->bands + nb; p->dc.D2 = p->bands + 2 * nb;
    p->dc.a = p->coefs; p->dc.b = p->coefs + SS; p->dc.c = p->coefs + 2 * SS; p->dc.g = p->coefs + 3 * SS;
    return p;
}

extern "C" int sgb_plan_destroy(sgb_plan *p)
{
    if (!p) return 0;
    if (!p->allocs.empty()) {
        std::lock_guard<std::mutex> lk(g_pool.mu);
        if (p->captured) cudaDeviceSynchronize();
        for (auto &d : p->done) cudaStreamWaitEvent(g_pool.st, d.second, 0);
        for (void *a : p->allocs) cudaFreeAsync(a, g_pool.st);
    }
    for (auto &d : p->done) cudaEventDestroy(d.second);
    if (p->hcount) cudaFreeHost(p->hcount);
    delete p;
    return 0;
}

extern "C" size_t sgb_plan_device_bytes(const sgb_plan *p) { return p ? p->dev_bytes : 0; }

// Device bytes a plan holds once it has run the given method ('M', 'Z' or 0
// for both): the allocations of sgb_plan_create plus those of the first
// substep, so that a caller can admit work against a memory budget before
// creating the plan.  Each allocation is rounded up to 256 bytes.
extern "C" size_t sgb_plan_estimate_bytes(const sgb_case *c, int nsys, int max_double_slots,
                                          char method)
{
    if (!c || nsys < 1 || c->S < 1 || c->n < 2) return 0;
    auto up = [](size_t b) { return (b + 255) & ~size_t(255); };
    const int N = c->S * c->n, KL = c->S * (c->kl + 1) - 1, KU = c->S * (c->ku + 1) - 1;
    const size_t nb = (size_t) c->ld * c->n, SS = (size_t) c->S * c->S;
    FactorGeom g{N, KL, KU};
    size_t b = up(3 * nb * sizeof(double)) + up(nb * sizeof(float4)) + up(4 * SS * sizeof(double))
             + 2 * up(nsys * sizeof(double)) + up(18 * sizeof(double))
             + 2 * up((size_t) nsys * N * sizeof(double2));
    method = (char) toupper(method);
    if (method == 'Z' || method == 0)
        b += up((size_t) nsys * g.fac_elems() * sizeof(double2)) + up((size_t) nsys * N * sizeof(int))
           + up(nsys * sizeof(int)) + up((size_t) nsys * N * sizeof(double2));
    if (method == 'M' || method == 0) {
        RefineProblem P;
        P.nsys = nsys; P.g = g;
        P.nslot64 = std::max(1, std::min(nsys, max_double_slots > 0 ? max_double_slots : nsys));
        b += up(refine_workspace_bytes(P));
    }
    return b;
}

static int plan_alloc_z(sgb_plan *p)
{
    const int nsys = p->nsys, N = p->N;
    FactorGeom g{N, p->KL, p->KU};
    int rc = p->dalloc(&p->fac64, (size_t) nsys * g.fac_elems() * sizeof(double2), "cudaMalloc(fac64)");
    rc |= p->dalloc((void **) &p->ipiv64, (size_t) nsys * N * sizeof(int), "cudaMalloc(ipiv64)");
    rc |= p->dalloc((void **) &p->info64, (size_t) nsys * sizeof(int), "cudaMalloc(info64)");
    rc |= p->dalloc((void **) &p->y64, (size_t) nsys * N * sizeof(double2), "cudaMalloc(y64)");
    return rc;
}

// The refinement workspace depends only on (nsys, geometry, fallback slots).
static int plan_alloc_m(sgb_plan *p)
{
    RefineProblem P;
    P.nsys = p->nsys; P.g = {p->N, p->KL, p->KU}; P.nslot64 = p->nslot64;
    const size_t need = refine_workspace_bytes(P);
    if (need <= p->rws_bytes) return 0;
    int rc = p->dalloc(&p->rws, need, "cudaMalloc(refine workspace)");
    if (rc) return rc;
    p->rws_bytes = need;
    return 0;
}

// The refinement problem of the mixed method's capturable or host-driven
// substep of plan p at phi_imp.
static RefineProblem plan_refine_problem(sgb_plan *p, double phi_imp, const sgb_refine_spec *spec,
                                         bool capturable);

// capturable: no host synchronization, no allocation, no host-to-device copy
// (the refinement runs its device-counted form), so the call can be
// recorded into a CUDA graph after one ordinary call of the same method.
// stage 1 / 2: the two halves of the capturable mixed substep around an
// external complex64 factor (sgb_plan_substep_stage).

static int plan_substep(sgb_plan *p, char method, double phi_exp, double phi_imp,
                        const void *u_in, void *u_out, const sgb_refine_spec *spec,
                        cudaStream_t st, bool capturable = false, int stage = 0)
{
    const int nsys = p->nsys, N = p->N, S = p->hc.S, n = p->hc.n;
    const long long tot = (long long) nsys * N;
    const unsigned EB = (unsigned) ((tot + 255) / 256);
    PhaseTimer nop;
    PhaseTimer &tm = capturable ? nop : p->timer;
    if (stage == 2) goto refine;      // stage 1 ran the explicit operator and the init
    // 1. explicit operator (or plain permutation) into b
    tm.begin(phi_exp != 0.0 ? "explicit_apply_f64" : "permute_in", st);
    count_launch(1);
    if (phi_exp != 0.0) {
        ApplyArgs aa;
        aa.nsys = nsys; aa.ms = p->ms(phi_exp);
        aa.u = reinterpret_cast<const double2 *>(u_in); aa.u_stride = N;
        aa.y = p->b; aa.y_stride = N;
        SGB_CUDA_TRY(launch_model_apply(aa, st));
    } else {
        k_permute<<<EB, 256, 0, st>>>(nsys, S, n, reinterpret_cast<const double2 *>(u_in), p->b, 0);
        SGB_CUDA_TRY(cudaGetLastError());
    }
    tm.end(st);
refine:
    {
    FactorGeom g{N, p->KL, p->KU};
    p->phi_imp_last = phi_imp;
    if (method == 'Z') {
        if (!p->fac64 && capturable)
            return fail("sgb_plan_substep_capturable: run sgb_plan_substep with method 'Z' first");
        if (!p->fac64) {
            int rc = plan_alloc_z(p);
            if (rc) return rc;
        }
        GbtrfArgs fa;
        fa.prec = 'Z'; fa.g = g; fa.nsys = nsys; fa.model = true; fa.ms = p->ms(phi_imp);
        fa.fac = p->fac64; fa.fac_stride = g.fac_elems(); fa.ipiv = p->ipiv64; fa.info = p->info64;
        fa.rhs = p->b; fa.rhs_stride = N; fa.y = p->y64; fa.y_stride = N;
        tm.begin("factor_c128", st);
        count_launch(1);
        SGB_CUDA_TRY(launch_gbtrf(fa, st));
        tm.end(st);
        GbtrsArgs sa;
        sa.prec = 'Z'; sa.trans = 'N'; sa.g = g; sa.nsys = nsys; sa.fac = p->fac64;
        sa.fac_stride = g.fac_elems(); sa.ipiv = p->ipiv64; sa.fwd_done = true; sa.yin = p->y64;
        sa.ywork = p->y64;
        sa.b_stride = N; sa.x = p->x; sa.x_stride = N;
        tm.begin("backsolve_c128", st);
        count_launch(1);
        SGB_CUDA_TRY(launch_gbtrs(sa, st));
        tm.end(st);
    } else if (method == 'M') {
        RefineProblem P = plan_refine_problem(p, phi_imp, spec, capturable);
        P.stage = stage;
        const size_t need = refine_workspace_bytes(P);
        if (need > p->rws_bytes && capturable)
            return fail("sgb_plan_substep_capturable: run sgb_plan_substep or sgb_plan_prepare "
                        "with method 'M' first");
        if (need > p->rws_bytes) {
            int rc = plan_alloc_m(p);
            if (rc) return rc;
        }
        int rc = refine_batched(P, p->rws, p->rws_bytes, p->last, st);
        if (rc) return sgb_set_error((cudaError_t) rc, "refine_batched", __FILE__, __LINE__);
        if (stage == 1) return 0;
    } else {
        return fail("sgb_plan_substep: method must be 'Z' or 'M'");
    }
    }
    p->last_method = method;
    tm.begin("permute_out", st);
    count_launch(1);
    k_permute<<<EB, 256, 0, st>>>(nsys, S, n, p->x, reinterpret_cast<double2 *>(u_out), 1);
    SGB_CUDA_TRY(cudaGetLastError());
    tm.end(st);
    return 0;
}

extern "C" int sgb_plan_set_timing(sgb_plan *p, int on)
{
    if (!p) return fail("sgb_plan_set_timing: null plan");
    std::lock_guard<std::mutex> lk(p->mu);
    p->timer.collect();
    p->timer.acc.clear();
    p->timer.on = on != 0;
    return 0;
}

extern "C" int sgb_plan_timings(sgb_plan *p, char *buf, int buflen)
{
    if (!p || !buf || buflen < 1) return fail("sgb_plan_timings: bad arguments");
    std::lock_guard<std::mutex> lk(p->mu);
    p->timer.collect();
    std::string s;
    for (auto &kv : p->timer.acc) {
        char line[256];
        std::snprintf(line, sizeof line, "%s %.6f %lld\n", kv.first.c_str(), kv.second.first,
                      kv.second.second);
        s += line;
    }
    std::snprintf(buf, buflen, "%s", s.c_str());
    return (int) s.size() < buflen ? 0 : fail("sgb_plan_timings: buffer too small", -2);
}

extern "C" int sgb_plan_substep(sgb_plan *p, char method, double phi_exp, double phi_imp,
                                const void *u_in, void *u_out, const sgb_refine_spec *spec,
                                void *stream)
{
    if (!p || !u_in || !u_out) return fail("sgb_plan_substep: null argument");
    std::lock_guard<std::mutex> lk(p->mu);
    const int rc = plan_substep(p, (char) toupper(method), phi_exp, phi_imp, u_in, u_out, spec,
                                (cudaStream_t) stream);
    p->note((cudaStream_t) stream);
    return rc;
}

extern "C" int sgb_plan_substep_capturable(sgb_plan *p, char method, double phi_exp,
                                           double phi_imp, const void *u_in, void *u_out,
                                           const sgb_refine_spec *spec, void *stream)
{
    if (!p || !u_in || !u_out) return fail("sgb_plan_substep_capturable: null argument");
    std::lock_guard<std::mutex> lk(p->mu);
    const int rc = plan_substep(p, (char) toupper(method), phi_exp, phi_imp, u_in, u_out, spec,
                                (cudaStream_t) stream, true);
    p->note((cudaStream_t) stream);
    return rc;
}

static RefineProblem plan_refine_problem(sgb_plan *p, double phi_imp, const sgb_refine_spec *spec,
                                         bool capturable)
{
    RefineProblem P;
    const int N = p->N;
    P.nsys = p->nsys; P.g = FactorGeom{N, p->KL, p->KU}; P.trans = 'N'; P.resid_trans = 'N';
    P.model = true;
    P.ms = p->ms(phi_imp); P.gram = p->gram; P.b = p->b; P.b_stride = N;
    P.x = p->x; P.x_stride = N;
    P.aiter = spec ? spec->aiter : 5; P.siter = spec ? spec->siter : 25;
    P.diter = spec ? spec->diter : 5; P.tolsc = spec ? spec->tolsc : 1.0;
    P.nslot64 = p->nslot64; P.host_count = p->hcount;
    P.timer = capturable ? nullptr : &p->timer;
    if (capturable) {
        P.graph = true;
        P.graph_siter = P.siter < 0 ? 0 : P.siter + 1;
        P.graph_diter = P.diter + 2;
    }
    return P;
}

// The capturable mixed substep in two stages around an external complex64
// factor (a ragged batch over many plans): stage 1 runs the explicit operator
// and the refinement's initial state, stage 2 everything from the factor's
// results on.  Stage 1, the ragged factor, then stage 2 give the results of
// sgb_plan_substep_capturable bit for bit.
extern "C" int sgb_plan_substep_stage(sgb_plan *p, int stage, char method, double phi_exp,
                                      double phi_imp, const void *u_in, void *u_out,
                                      const sgb_refine_spec *spec, void *stream)
{
    if (!p || !u_in || !u_out) return fail("sgb_plan_substep_stage: null argument");
    if (stage != 1 && stage != 2) return fail("sgb_plan_substep_stage: stage must be 1 or 2");
    if (toupper(method) != 'M') return fail("sgb_plan_substep_stage: method must be 'M'");
    if (spec && spec->siter < 0) return fail("sgb_plan_substep_stage: needs siter >= 0");
    std::lock_guard<std::mutex> lk(p->mu);
    const int rc = plan_substep(p, 'M', phi_exp, phi_imp, u_in, u_out, spec, (cudaStream_t) stream,
                                true, stage);
    p->note((cudaStream_t) stream);
    return rc;
}

// A ragged batch: the complex64 factors of many plans' substeps (each at its
// own phi_imp) as one launch per kernel kind (the compile-time bandwidth
// instances, else the generic ones for KL <= 40 and KL <= 56), one CTA per
// system position, the largest plans' systems first.
struct sgb_ragged {
    struct Class {
        int kind = 0;             // ragged_kind of its plans' geometry
        RaggedDesc *descs = nullptr;
        int2 *items = nullptr;
        int nitems = 0;
        size_t smem = 0;
    };
    std::vector<Class> cls;
    std::vector<sgb_plan *> plans;
    std::vector<void *> rws;      // each plan's workspace when the batch was made
};

extern "C" void sgb_ragged_destroy(sgb_ragged *r);

extern "C" sgb_ragged *sgb_ragged_create(sgb_plan *const *plans, int nplans, const double *phi_imp,
                                         const sgb_refine_spec *spec)
{
    if (!plans || nplans <= 0 || !phi_imp) { fail("sgb_ragged_create: bad arguments"); return nullptr; }
    if (spec && spec->siter < 0) { fail("sgb_ragged_create: needs siter >= 0"); return nullptr; }
    auto *r = new (std::nothrow) sgb_ragged;
    if (!r) { fail("sgb_ragged_create: out of memory"); return nullptr; }
    struct Acc {
        std::vector<RaggedDesc> descs;
        std::vector<std::pair<long long, int>> order;   // (cost, plan)
        size_t smem = 0;
    };
    std::map<int, Acc> acc;
    std::vector<int> where(nplans);
    for (int i = 0; i < nplans; ++i) {
        sgb_plan *p = plans[i];
        if (!p || p->KL > 56 || p->hc.S > 8) {
            sgb_ragged_destroy(r);
            fail("sgb_ragged_create: a plan is null or has KL > 56 or S > 8");
            return nullptr;
        }
        std::lock_guard<std::mutex> lk(p->mu);
        RefineProblem P = plan_refine_problem(p, phi_imp[i], spec, true);
        if (refine_workspace_bytes(P) > p->rws_bytes) {
            sgb_ragged_destroy(r);
            fail("sgb_ragged_create: run a mixed substep (or sgb_plan_prepare 'M') of every plan first");
            return nullptr;
        }
        RaggedDesc d;
        refine_ragged_desc(P, p->rws, d);
        Acc &a = acc[ragged_kind(d.g)];
        where[i] = (int) a.descs.size();
        a.descs.push_back(d);
        a.order.push_back({(long long) p->N * p->KL * (p->KL + p->KU), i});
        a.smem = std::max(a.smem, gbtrf_blk_smem_bytes(sizeof(float), d.g, p->hc.S, 4, 2));
        r->plans.push_back(p);
        r->rws.push_back(p->rws);
    }
    cudaError_t e = cudaSuccess;
    for (auto &kv : acc) {
        Acc &a = kv.second;
        r->cls.emplace_back();
        sgb_ragged::Class &k = r->cls.back();
        k.kind = kv.first;
        k.smem = a.smem;
        std::sort(a.order.begin(), a.order.end(),
                  [](const std::pair<long long, int> &x, const std::pair<long long, int> &y) {
                      return x.first > y.first;
                  });
        std::vector<int2> it;
        for (auto &o : a.order)
            for (int k2 = 0; k2 < plans[o.second]->nsys; ++k2) it.push_back(make_int2(where[o.second], k2));
        k.nitems = (int) it.size();
        if ((e = cudaMalloc(&k.descs, a.descs.size() * sizeof(RaggedDesc))) != cudaSuccess) break;
        if ((e = cudaMemcpy(k.descs, a.descs.data(), a.descs.size() * sizeof(RaggedDesc),
                            cudaMemcpyHostToDevice)) != cudaSuccess) break;
        if ((e = cudaMalloc(&k.items, it.size() * sizeof(int2))) != cudaSuccess) break;
        if ((e = cudaMemcpy(k.items, it.data(), it.size() * sizeof(int2), cudaMemcpyHostToDevice)) != cudaSuccess)
            break;
    }
    if (e != cudaSuccess) {
        sgb_ragged_destroy(r);
        sgb_set_error(e, "sgb_ragged_create", __FILE__, __LINE__);
        return nullptr;
    }
    return r;
}

extern "C" void sgb_ragged_destroy(sgb_ragged *r)
{
    if (!r) return;
    for (auto &k : r->cls) { cudaFree(k.descs); cudaFree(k.items); }
    delete r;
}

// The ragged factor launches, after every plan's stage 1 and before its
// stage 2 (on the stream given, capturable).
extern "C" int sgb_ragged_factor(sgb_ragged *r, void *stream)
{
    if (!r) return fail("sgb_ragged_factor: null batch");
    cudaStream_t st = (cudaStream_t) stream;
    for (size_t i = 0; i < r->plans.size(); ++i)
        if (r->plans[i]->rws != r->rws[i])
            return fail("sgb_ragged_factor: a plan's workspace moved since the batch was made");
    for (const auto &k : r->cls) {
        if (k.nitems == 0) continue;
        count_launch(1);
        SGB_CUDA_TRY(launch_gbtrf_ragged(k.descs, k.items, k.nitems, k.kind, k.smem, st));
    }
    for (sgb_plan *p : r->plans) p->note(st);
    return 0;
}

// Compile-time bandwidth instances of the complex64 factor on (1, the
// default) or off; both give the same bits.
extern "C" int sgb_gbtrf_set_specialized(int on)
{
    gbtrf_set_specialized(on);
    return 0;
}

extern "C" int sgb_plan_prepare(sgb_plan *p, char method)
{
    if (!p) return fail("sgb_plan_prepare: null plan");
    std::lock_guard<std::mutex> lk(p->mu);
    method = (char) toupper(method);
    if (method != 'M' && method != 'Z' && method != 0)
        return fail("sgb_plan_prepare: method must be 'M', 'Z' or 0");
    if ((method == 'Z' || method == 0) && !p->fac64) {
        int rc = plan_alloc_z(p);
        if (rc) return rc;
    }
    if (method == 'M' || method == 0) return plan_alloc_m(p);
    return 0;
}

extern "C" int sgb_plan_unserved(sgb_plan *p, int *count)
{
    if (!p || !count) return fail("sgb_plan_unserved: null argument");
    std::lock_guard<std::mutex> lk(p->mu);
    *count = 0;
    if (p->last_method != 'M' || !p->last.d_unserved) return 0;
    SGB_CUDA_TRY(cudaMemcpy(count, p->last.d_unserved, sizeof(int), cudaMemcpyDeviceToHost));
    return 0;
}

extern "C" int sgb_plan_substep_host(sgb_plan *p, char method, double phi_exp, double phi_imp,
                                     const void *u_in_host, void *u_out_host,
                                     const sgb_refine_spec *spec, void *stream)
{
    if (!p || !u_in_host || !u_out_host) return fail("sgb_plan_substep_host: null argument");
    std::lock_guard<std::mutex> lk(p->mu);
    cudaStream_t st = (cudaStream_t) stream;
    const size_t bytes = (size_t) p->nsys * p->N * sizeof(double2);
    if (!p->u_stage) {
        int rc = p->dalloc((void **) &p->u_stage, bytes, "cudaMalloc(u_stage)");
        if (rc) return rc;
    }
    SGB_CUDA_TRY(cudaMemcpyAsync(p->u_stage, u_in_host, bytes, cudaMemcpyHostToDevice, st));
    int rc = plan_substep(p, (char) toupper(method), phi_exp, phi_imp, p->u_stage, p->u_stage,
                          spec, st);
    if (rc) return rc;
    SGB_CUDA_TRY(cudaMemcpyAsync(u_out_host, p->u_stage, bytes, cudaMemcpyDeviceToHost, st));
    SGB_CUDA_TRY(cudaStreamSynchronize(st));
    return 0;
}

extern "C" int sgb_plan_report(const sgb_plan *p, int *info, int *siter, int *diter,
                               double *res, double *tolsc, char *fact)
{
    if (!p) return fail("sgb_plan_report: null plan");
    const int nsys = p->nsys;
    SGB_CUDA_TRY(cudaDeviceSynchronize());
    if (p->last_method == 'Z') {
        if (info) SGB_CUDA_TRY(cudaMemcpy(info, p->info64, nsys * sizeof(int), cudaMemcpyDeviceToHost));
        if (siter) std::fill(siter, siter + nsys, 0);
        if (diter) std::fill(diter, diter + nsys, 0);
        if (res) std::fill(res, res + nsys, 0.0);
        if (tolsc) std::fill(tolsc, tolsc + nsys, 0.0);
        if (fact) std::fill(fact, fact + nsys, 'F');
        return 0;
    }
    if (p->last_method != 'M') return fail("sgb_plan_report: no substep has run");
    const RefineState &st = p->last.state;
    if (info) SGB_CUDA_TRY(cudaMemcpy(info, st.info, nsys * sizeof(int), cudaMemcpyDeviceToHost));
    if (siter) SGB_CUDA_TRY(cudaMemcpy(siter, st.siter, nsys * sizeof(int), cudaMemcpyDeviceToHost));
    if (diter) SGB_CUDA_TRY(cudaMemcpy(diter, st.diter, nsys * sizeof(int), cudaMemcpyDeviceToHost));
    if (res) SGB_CUDA_TRY(cudaMemcpy(res, st.res, nsys * sizeof(double), cudaMemcpyDeviceToHost));
    if (tolsc) SGB_CUDA_TRY(cudaMemcpy(tolsc, st.tolsc, nsys * sizeof(double), cudaMemcpyDeviceToHost));
    if (fact) SGB_CUDA_TRY(cudaMemcpy(fact, st.fact, nsys, cudaMemcpyDeviceToHost));
    return 0;
}

// Normwise backward error per system: one warp per system, lanes over rows;
// the S x S block coefficients of the system in shared memory (3 S^2 <= 192).
__global__ void k_backward_error(int nsys, ModelSource ms, const double2 *__restrict__ b,
                                 const double2 *__restrict__ x, double *__restrict__ out)
{
    const int s = blockIdx.x;
    if (s >= nsys) return;
    const sgb_case &cs = ms.cs;
    const int S = cs.S, n = cs.n, N = S * n;
    const double2 *xs = x + (long long) s * N, *bs = b + (long long) s * N;
    double anorm = 0, rmax = 0, xmax = 0, bmax = 0;
    __shared__ sgb_coef cf[3][64];
    for (int ef = threadIdx.x; ef < S * S; ef += 32)
        sgb_block_coefs(&cs, ef / S, ef % S, ms.phi, ms.kx[s], ms.kz[s], &cf[0][ef], &cf[1][ef],
                        &cf[2][ef]);
    __syncwarp();
    for (int I = threadIdx.x; I < N; I += 32) {
        const int p = I / S, e = I % S;
        double2 ax = make_double2(0, 0);
        double rowsum = 0;
        if (((cs.dirichlet_mask >> e) & 1u) && (p == 0 || p == n - 1)) {
            ax = xs[I];
            rowsum = 1;
        } else {
            for (int q = imax(0, p - cs.kl); q <= imin(n - 1, p + cs.ku); ++q) {
                const int k = cs.ku + p - q + q * cs.ld;
                for (int f = 0; f < S; ++f) {
                    double re, im;
                    sgb_block_entry(cf[0][e * S + f], cf[1][e * S + f], cf[2][e * S + f],
                                    cs.M[k], cs.D1[k], cs.D2[k], &re, &im);
                    const double2 a = make_double2(re, im);
                    ax = cfma(a, xs[q * S + f], ax);
                    rowsum += fabs(re) + fabs(im);
                }
            }
        }
        const double2 r = csub(bs[I], ax);
        rmax = fmax(rmax, fmax(fabs(r.x), fabs(r.y)));
        anorm = fmax(anorm, rowsum);
        xmax = fmax(xmax, fmax(fabs(xs[I].x), fabs(xs[I].y)));
        bmax = fmax(bmax, fmax(fabs(bs[I].x), fabs(bs[I].y)));
    }
    for (int off = 16; off; off >>= 1) {
        rmax = fmax(rmax, __shfl_xor_sync(0xffffffffu, rmax, off));
        anorm = fmax(anorm, __shfl_xor_sync(0xffffffffu, anorm, off));
        xmax = fmax(xmax, __shfl_xor_sync(0xffffffffu, xmax, off));
        bmax = fmax(bmax, __shfl_xor_sync(0xffffffffu, bmax, off));
    }
    if (threadIdx.x == 0) out[s] = rmax / (anorm * xmax + bmax);
}

extern "C" int sgb_plan_backward_error(sgb_plan *p, double *berr_host, void *stream)
{
    if (!p || !berr_host) return fail("sgb_plan_backward_error: null argument");
    if (p->hc.S * p->hc.S > 64) return fail("sgb_plan_backward_error: S too large");
    std::lock_guard<std::mutex> lk(p->mu);
    cudaStream_t st = (cudaStream_t) stream;
    double *d = nullptr;
    SGB_CUDA_TRY(cudaMallocAsync((void **) &d, p->nsys * sizeof(double), st));
    k_backward_error<<<p->nsys, 32, 0, st>>>(p->nsys, p->ms(p->phi_imp_last), p->b, p->x, d);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(berr_host, d, p->nsys * sizeof(double), cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(d, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return sgb_set_error(e, "backward error", __FILE__, __LINE__);
    return 0;
}

// ---------------------------------------------------------------------------
// Batch: one case's systems split into resident parts, each a plan on its
// own stream.  The parts' substeps overlap on the device (one part's FP64
// kernels beside another's complex64 factor), and the host-buffer form
// pipelines each part's copy in, substep and copy out on the part's stream,
// so that only the first part's copy in and the last part's copy out are
// not hidden behind computation.
// ---------------------------------------------------------------------------
struct sgb_batch {
    std::vector<sgb_plan *> plans;
    std::vector<int> bounds;                 // parts + 1 row offsets
    std::vector<cudaStream_t> streams;
    std::vector<cudaEvent_t> joins;
    std::vector<cudaEvent_t> copied_in;      // host form: part i's copy in is done
    std::vector<double2 *> stage;            // host form: per-part device staging
    cudaEvent_t fork = nullptr;
    int nsys = 0, N = 0;
    std::mutex mu;
};

extern "C" int sgb_batch_bounds(int nsys, int parts, int *bounds)
{
    if (nsys < 1 || parts < 1 || !bounds) return fail("sgb_batch_bounds: bad arguments");
    parts = std::min(parts, nsys);
    for (int i = 0; i <= parts; ++i) bounds[i] = (int) ((long long) i * nsys / parts);
    return parts;
}

extern "C" int sgb_batch_destroy(sgb_batch *b)
{
    if (!b) return 0;
    for (cudaStream_t s : b->streams) cudaStreamSynchronize(s);
    for (sgb_plan *p : b->plans) sgb_plan_destroy(p);
    if (!b->stage.empty()) {
        std::lock_guard<std::mutex> lk(g_pool.mu);
        for (double2 *s : b->stage) if (s) cudaFreeAsync(s, g_pool.st);
    }
    for (cudaEvent_t e : b->joins) cudaEventDestroy(e);
    for (cudaEvent_t e : b->copied_in) cudaEventDestroy(e);
    if (b->fork) cudaEventDestroy(b->fork);
    for (cudaStream_t s : b->streams) cudaStreamDestroy(s);
    delete b;
    return 0;
}

extern "C" sgb_batch *sgb_batch_create(const sgb_case *hcase, int nsys, const double *kx,
                                       const double *kz, int parts, int max_double_slots,
                                       char method)
{
    if (!hcase || nsys < 1 || !kx || !kz || parts < 1) {
        fail("sgb_batch_create: bad arguments");
        return nullptr;
    }
    method = (char) toupper(method);
    if (method != 'M' && method != 'Z' && method != 0) {
        fail("sgb_batch_create: method must be 'M', 'Z' or 0");
        return nullptr;
    }
    sgb_batch *b = new (std::nothrow) sgb_batch;
    if (!b) { fail("sgb_batch_create: out of host memory"); return nullptr; }
    b->nsys = nsys;
    b->N = hcase->S * hcase->n;
    b->bounds.resize((size_t) std::min(parts, nsys) + 1);
    parts = sgb_batch_bounds(nsys, parts, b->bounds.data());
    const int slots = max_double_slots > 0 ? (max_double_slots + parts - 1) / parts : 0;
    for (int i = 0; i < parts; ++i) {
        const int lo = b->bounds[i], cnt = b->bounds[i + 1] - lo;
        sgb_plan *p = sgb_plan_create(hcase, cnt, kx + lo, kz + lo, slots);
        if (!p) { sgb_batch_destroy(b); return nullptr; }
        b->plans.push_back(p);
        if (sgb_plan_prepare(p, method) != 0) { sgb_batch_destroy(b); return nullptr; }
        cudaStream_t s = nullptr;
        cudaEvent_t e = nullptr;
        cudaEvent_t c = nullptr;
        cudaError_t err = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        if (err == cudaSuccess) b->streams.push_back(s);
        if (err == cudaSuccess) err = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
        if (err == cudaSuccess) b->joins.push_back(e);
        if (err == cudaSuccess) err = cudaEventCreateWithFlags(&c, cudaEventDisableTiming);
        if (err == cudaSuccess) b->copied_in.push_back(c);
        if (err != cudaSuccess) {
            sgb_set_error(err, "sgb_batch_create(stream)", __FILE__, __LINE__);
            sgb_batch_destroy(b);
            return nullptr;
        }
    }
    cudaError_t err = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
    if (err != cudaSuccess) {
        sgb_set_error(err, "sgb_batch_create(event)", __FILE__, __LINE__);
        sgb_batch_destroy(b);
        return nullptr;
    }
    return b;
}

extern "C" int sgb_batch_parts(const sgb_batch *b) { return b ? (int) b->plans.size() : 0; }

extern "C" sgb_plan *sgb_batch_plan(sgb_batch *b, int part)
{
    if (!b || part < 0 || part >= (int) b->plans.size()) return nullptr;
    return b->plans[part];
}

extern "C" size_t sgb_batch_device_bytes(const sgb_batch *b)
{
    if (!b) return 0;
    size_t t = 0;
    for (const sgb_plan *p : b->plans) t += p->dev_bytes;
    for (size_t i = 0; i < b->stage.size(); ++i)
        if (b->stage[i]) t += (size_t) (b->bounds[i + 1] - b->bounds[i]) * b->N * sizeof(double2);
    return t;
}

// Fork every part's stream from st, run body(part, part stream) on each, join
// them back into st.  The same call sequence records correctly into a CUDA
// graph being captured on st.
template <typename Body>
static int batch_fork_join(sgb_batch *b, cudaStream_t st, Body &&body)
{
    SGB_CUDA_TRY(cudaEventRecord(b->fork, st));
    int rc = 0;
    const int parts = (int) b->plans.size();
    for (int i = 0; i < parts; ++i) {
        cudaStream_t ps = b->streams[i];
        SGB_CUDA_TRY(cudaStreamWaitEvent(ps, b->fork, 0));
        if (!rc) rc = body(i, ps);
        SGB_CUDA_TRY(cudaEventRecord(b->joins[i], ps));
        SGB_CUDA_TRY(cudaStreamWaitEvent(st, b->joins[i], 0));
    }
    return rc;
}

extern "C" int sgb_batch_substep(sgb_batch *b, char method, double phi_exp, double phi_imp,
                                 const void *u_in, void *u_out, const sgb_refine_spec *spec,
                                 void *stream)
{
    if (!b || !u_in || !u_out) return fail("sgb_batch_substep: null argument");
    std::lock_guard<std::mutex> lk(b->mu);
    const char m = (char) toupper(method);
    return batch_fork_join(b, (cudaStream_t) stream, [&](int i, cudaStream_t ps) {
        sgb_plan *p = b->plans[i];
        const size_t off = (size_t) b->bounds[i] * b->N;
        std::lock_guard<std::mutex> pk(p->mu);
        const int rc = plan_substep(p, m, phi_exp, phi_imp,
                                    reinterpret_cast<const double2 *>(u_in) + off,
                                    reinterpret_cast<double2 *>(u_out) + off, spec, ps, true);
        p->note(ps);
        return rc;
    });
}

extern "C" int sgb_batch_substep_host(sgb_batch *b, char method, double phi_exp, double phi_imp,
                                      const void *u_in_host, void *u_out_host,
                                      const sgb_refine_spec *spec, void *stream)
{
    if (!b || !u_in_host || !u_out_host) return fail("sgb_batch_substep_host: null argument");
    std::lock_guard<std::mutex> lk(b->mu);
    const int parts = (int) b->plans.size();
    if (b->stage.empty()) {
        b->stage.assign(parts, nullptr);
        for (int i = 0; i < parts; ++i) {
            const size_t bytes = (size_t) (b->bounds[i + 1] - b->bounds[i]) * b->N * sizeof(double2);
            cudaError_t e = g_pool.alloc((void **) &b->stage[i], bytes);
            if (e != cudaSuccess) return sgb_set_error(e, "sgb_batch_substep_host(staging)", __FILE__, __LINE__);
        }
    }
    const char m = (char) toupper(method);
    cudaStream_t st = (cudaStream_t) stream;
    int rc = batch_fork_join(b, st, [&](int i, cudaStream_t ps) {
        sgb_plan *p = b->plans[i];
        const size_t off = (size_t) b->bounds[i] * b->N;
        const size_t bytes = (size_t) (b->bounds[i + 1] - b->bounds[i]) * b->N * sizeof(double2);
        // The copies in follow one another (part i's after part i-1's):
        // issued together they would share the link and every part's data
        // would arrive only when all of it has; in order, part 0 starts
        // computing after a quarter of the transfer and the parts finish
        // staggered, so the early parts' copies out overlap the later work.
        cudaError_t e = i ? cudaStreamWaitEvent(ps, b->copied_in[i - 1], 0) : cudaSuccess;
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(b->stage[i], reinterpret_cast<const double2 *>(u_in_host) + off,
                                bytes, cudaMemcpyHostToDevice, ps);
        if (e == cudaSuccess) e = cudaEventRecord(b->copied_in[i], ps);
        if (e != cudaSuccess) return sgb_set_error(e, "sgb_batch_substep_host(copy in)", __FILE__, __LINE__);
        std::lock_guard<std::mutex> pk(p->mu);
        int r = plan_substep(p, m, phi_exp, phi_imp, b->stage[i], b->stage[i], spec, ps, true);
        p->note(ps);
        if (r) return r;
        e = cudaMemcpyAsync(reinterpret_cast<double2 *>(u_out_host) + off, b->stage[i], bytes,
                            cudaMemcpyDeviceToHost, ps);
        if (e != cudaSuccess) return sgb_set_error(e, "sgb_batch_substep_host(copy out)", __FILE__, __LINE__);
        return 0;
    });
    if (rc) return rc;
    SGB_CUDA_TRY(cudaStreamSynchronize(st));
    return 0;
}

extern "C" int sgb_batch_report(const sgb_batch *b, int *info, int *siter, int *diter,
                                double *res, double *tolsc, char *fact)
{
    if (!b) return fail("sgb_batch_report: null batch");
    for (size_t i = 0; i < b->plans.size(); ++i) {
        const int o = b->bounds[i];
        int rc = sgb_plan_report(b->plans[i], info ? info + o : nullptr, siter ? siter + o : nullptr,
                                 diter ? diter + o : nullptr, res ? res + o : nullptr,
                                 tolsc ? tolsc + o : nullptr, fact ? fact + o : nullptr);
        if (rc) return rc;
    }
    return 0;
}

extern "C" int sgb_batch_backward_error(sgb_batch *b, double *berr_host, void *stream)
{
    if (!b || !berr_host) return fail("sgb_batch_backward_error: null argument");
    for (size_t i = 0; i < b->plans.size(); ++i) {
        int rc = sgb_plan_backward_error(b->plans[i], berr_host + b->bounds[i], stream);
        if (rc) return rc;
    }
    return 0;
}

extern "C" int sgb_batch_unserved(sgb_batch *b, int *count)
{
    if (!b || !count) return fail("sgb_batch_unserved: null argument");
    *count = 0;
    for (sgb_plan *p : b->plans) {
        int c = 0;
        int rc = sgb_plan_unserved(p, &c);
        if (rc) return rc;
        *count += c;
    }
    return 0;
}

// ---------------------------------------------------------------------------
// Packed bands of a plan's operator (the caller-packed form of the solve)
// ---------------------------------------------------------------------------
// One thread per band element: column c = t / ldab, band row i = t % ldab;
// rows off .. off + KL + KU hold A(r, c), r = c + i - off - KU, the others
// and every position outside the matrix are zero (what suzerain_bsmbsm_zpack
// leaves around the band, suzerain/bsmbsm_pack.def:66-119).
// Packed band of every system (ldab x N per system, band rows off ..
// off + KL + KU).  Block (x, s): columns 4x .. 4x+3 of system s, threads
// over (row, column); the system's S x S block coefficients are formed once
// per block in shared memory.
__global__ void k_assemble_packed(int nsys, ModelSource ms, int KL, int KU, double2 *__restrict__ ab,
                                  int ldab, long long ab_stride, int off)
{
    const int s = blockIdx.y;
    const sgb_case &cs = ms.cs;
    const int S = cs.S, N = S * cs.n;
    if (s >= nsys) return;
    __shared__ sgb_coef cf[3][64];
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    for (int ef = tid; ef < S * S; ef += blockDim.x * blockDim.y)
        sgb_block_coefs(&cs, ef / S, ef % S, ms.phi, ms.kx[s], ms.kz[s], &cf[0][ef], &cf[1][ef],
                        &cf[2][ef]);
    __syncthreads();
    const int c = blockIdx.x * blockDim.y + threadIdx.y;
    if (c >= N) return;
    const int q = c / S, f = c - q * S;
    double2 *col = ab + s * ab_stride + (long long) c * ldab;
    for (int i = threadIdx.x; i < ldab; i += blockDim.x) {
        const int r = c + i - off - KU;
        double2 v = make_double2(0.0, 0.0);
        if (i >= off && i <= off + KL + KU && r >= 0 && r < N) {
            const int p = r / S, e = r - p * S;
            if (sgb_is_dirichlet_row(&cs, r)) {
                v.x = (r == c) ? 1.0 : 0.0;
            } else if (p - q <= cs.kl && q - p <= cs.ku) {
                const int k = cs.ku + p - q + q * cs.ld, ef = e * S + f;
                sgb_block_entry(cf[0][ef], cf[1][ef], cf[2][ef], cs.M[k], cs.D1[k], cs.D2[k], &v.x, &v.y);
            }
        }
        col[i] = v;
    }
}

extern "C" int sgb_plan_assemble_packed(sgb_plan *p, double phi, void *ab, int ldab,
                                        long long ab_stride, int off, void *stream)
{
    if (!p || !ab) return fail("sgb_plan_assemble_packed: null argument");
    if (off < 0 || ldab < off + p->KL + p->KU + 1 || ab_stride < (long long) ldab * p->N)
        return fail("sgb_plan_assemble_packed: ldab must be >= off + KL + KU + 1 and "
                    "ab_stride >= ldab * N");
    if (p->hc.S * p->hc.S > 64) return fail("sgb_plan_assemble_packed: S too large");
    std::lock_guard<std::mutex> lk(p->mu);
    dim3 grd((unsigned) ((p->N + 3) / 4), (unsigned) p->nsys);
    count_launch(1);
    k_assemble_packed<<<grd, dim3(64, 4), 0, (cudaStream_t) stream>>>(
        p->nsys, p->ms(phi), p->KL, p->KU, reinterpret_cast<double2 *>(ab), ldab, ab_stride, off);
    SGB_CUDA_TRY(cudaGetLastError());
    p->note((cudaStream_t) stream);
    return 0;
}
