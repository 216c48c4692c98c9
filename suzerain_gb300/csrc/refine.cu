// Batched mixed-precision solve: the control flow of
// suzerain_lapackext_zcgbsvx (suzerain/blas_et_al/dsgbsvx.def:70-313) run for
// thousands of systems at once.  Every system carries its own state
// (fact, siter, diter, res, lastres, tol) and walks the same decisions as the
// reference; systems that converge leave the compacted active list, systems
// whose complex64 refinement stalls (or whose complex64 factor is singular)
// move to the complex128 factor and refine there.
//
// Iterations are launched from the host; every kernel takes the active list
// and a device-resident count, so a launch whose list is empty costs one
// early-returning block.
#include "sgb_internal.h"
#include "sgb_refine.h"
#include "sgb_timer.h"

#include <cmath>
#include <cstring>
#include <vector>

namespace sgb {

enum : int { ST_SINGLE = 1, ST_NEED_D = 2, ST_DOUBLE = 3, ST_DONE = 0, ST_ERROR = -1 };

__global__ void k_refine_init(int nsys, RefineState st, const double *__restrict__ afrob,
                              double tolsc, int N, int smax, int dmax,
                              const double *__restrict__ bnorm, int *__restrict__ listS,
                              int *__restrict__ countS, int *__restrict__ listD,
                              int *__restrict__ countD)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsys) return;
    const double eps = 1.1102230246251565e-16;   // dlamch('E')
    const bool use_eps = (tolsc == 0.0);
    const double res = bnorm[s];
    st.res[s] = res;
    st.lastres[s] = 3.0 * (res + 1.0);           // (resdecay + 1) * (res + 1)
    st.tolconst[s] = use_eps ? 1.0 : afrob[s] * eps * sqrt((double) N) * tolsc;
    st.tol[s] = use_eps ? eps : 0.0;
    st.siter[s] = -1;
    st.diter[s] = -1;
    st.fact[s] = 'N';
    st.info[s] = 0;
    const double tol = st.tol[s];
    if (smax >= 0 && res > tol) {
        st.status[s] = ST_SINGLE;
        st.fact[s] = 'S';
        listS[atomicAdd(countS, 1)] = s;
    } else {
        st.siter[s] = 0;
        if (dmax >= 0 && res > tol) {
            st.status[s] = ST_NEED_D;
            listD[atomicAdd(countD, 1)] = s;
        } else {
            st.status[s] = ST_DONE;
            st.diter[s] = 0;
        }
    }
}

// After the complex64 factorization: a singular factor goes straight to
// complex128 when allowed (dsgbsvx.def:180-186).
__global__ void k_refine_after_sfactor(RefineState st, const int *__restrict__ info32,
                                       const int *__restrict__ list, const int *__restrict__ count,
                                       int dmax, int *__restrict__ listD, int *__restrict__ countD)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= *count) return;
    const int s = list[k];
    if (info32[s] > 0) {
        if (dmax >= 0) {
            st.status[s] = ST_NEED_D;
            listD[atomicAdd(countD, 1)] = s;
        } else {
            st.status[s] = ST_DONE;   // reference keeps refining a singular factor
            st.info[s] = info32[s];
        }
    }
}

// One refinement decision after r = b - A x, ||r||, ||x|| are known.
// phase 0: complex64 loop (siter), phase 1: complex128 loop (diter).
// Mirrors the loop bodies of dsgbsvx.def:189-237 and :254-289.
__global__ void k_refine_decide(RefineState st, int phase, const double *__restrict__ rnorm,
                                const double *__restrict__ xnorm, int aiter, int smax, int dmax,
                                const int *__restrict__ list, const int *__restrict__ count,
                                int *__restrict__ next, int *__restrict__ ncount,
                                int *__restrict__ listD, int *__restrict__ countD)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= *count) return;
    const int s = list[k];
    if (st.status[s] != (phase == 0 ? ST_SINGLE : ST_DOUBLE)) return;
    const double eps = 1.1102230246251565e-16;
    int *it = phase == 0 ? st.siter : st.diter;
    const int imax_ = phase == 0 ? smax : dmax;
    it[s] += 1;
    const double tol = st.use_eps ? eps : xnorm[s] * st.tolconst[s];
    st.tol[s] = tol;
    const double res = rnorm[s];
    st.res[s] = res;
    if (isnan(res)) {             // dsgbsvx.def:204-207 (internal error)
        st.status[s] = ST_ERROR;
        st.info[s] = -1;
        return;
    }
    bool leave = false;
    if (it[s] >= aiter && st.lastres[s] < res * 2.0) {
        leave = true;             // stalled: blame single precision / the problem
    } else {
        st.lastres[s] = res;
        if (!(it[s] < imax_ && res > tol)) leave = true;
    }
    if (!leave) {
        next[atomicAdd(ncount, 1)] = s;
        return;
    }
    if (phase == 0 && dmax >= 0 && res > tol) {
        st.status[s] = ST_NEED_D;
        listD[atomicAdd(countD, 1)] = s;
    } else {
        st.status[s] = ST_DONE;
        if (phase == 0) st.diter[s] = 0;
    }
}

__global__ void k_refine_enter_double(RefineState st, const int *__restrict__ list,
                                      const int *__restrict__ count, const int *__restrict__ info64,
                                      int slot_base, int *__restrict__ next, int *__restrict__ ncount)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= *count) return;
    const int s = list[k];
    st.fact[s] = 'D';
    const int inf = info64[slot_base + k];
    if (inf > 0) {                // dsgbsvx.def:246: singular double factor
        st.status[s] = ST_DONE;
        st.info[s] = inf;
        return;
    }
    st.status[s] = ST_DOUBLE;
    next[atomicAdd(ncount, 1)] = s;
}

// Capturable form: systems still refining in complex64 after the fixed
// number of correction solves leave as if siter were exhausted
// (dsgbsvx.def:223-230): to complex128 when allowed and not converged.
__global__ void k_refine_cap(RefineState st, const int *__restrict__ list,
                             const int *__restrict__ count, int dmax, int *__restrict__ listD,
                             int *__restrict__ countD)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= *count) return;
    const int s = list[k];
    if (st.status[s] != ST_SINGLE) return;
    if (dmax >= 0 && st.res[s] > st.tol[s]) {
        st.status[s] = ST_NEED_D;
        listD[atomicAdd(countD, 1)] = s;
    } else {
        st.status[s] = ST_DONE;
        st.diter[s] = 0;
    }
}

// chunk = min(count, cap); unserved = count - chunk
__global__ void k_chunk_count(const int *__restrict__ count, int cap, int *__restrict__ chunk,
                              int *__restrict__ unserved)
{
    const int c = *count;
    *chunk = c < cap ? c : cap;
    *unserved = c > cap ? c - cap : 0;
}

__global__ void k_refine_finalize(int nsys, RefineState st, double2 *__restrict__ x,
                                  long long x_stride, int N)
{
    const int s = blockIdx.x;
    if (s >= nsys) return;
    const double res = st.res[s];
    if (threadIdx.x == 0) {
        st.tolsc[s] = (res == 0.0) ? 0.0 : res / st.tol[s];
        if (st.siter[s] < 0) st.siter[s] = 0;
        if (st.diter[s] < 0) st.diter[s] = 0;
    }
    if (isnan(res))
        for (int i = threadIdx.x; i < N; i += blockDim.x)
            x[s * x_stride + i] = make_double2(NAN, NAN);
}

__global__ void k_zero_x(int nsys, double2 *__restrict__ x, long long x_stride, int N)
{
    const long long t = (long long) blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long) nsys * N) return;
    const long long s = t / N, i = t - s * N;
    x[s * x_stride + i] = make_double2(0, 0);
}

__global__ void k_bnorm(int nsys, const double2 *__restrict__ b, long long b_stride, int N,
                        double *__restrict__ out)
{
    const int s = blockIdx.x;
    if (s >= nsys) return;
    double acc = 0;
    for (int i = threadIdx.x; i < N; i += 32) {
        const double2 v = b[s * b_stride + i];
        acc = fma(v.x, v.x, fma(v.y, v.y, acc));
    }
    for (int off = 16; off; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    if (threadIdx.x == 0) out[s] = sqrt(acc);
}

// ||A||_F of a packed band (zlangb('F')); one warp per system.
__global__ void k_afrob_packed(int nsys, int N, int KL, int KU, PackedSource src,
                               double *__restrict__ out)
{
    const int s = blockIdx.x;
    if (s >= nsys) return;
    const double2 *ab = src.ab + s * src.stride + src.off;
    double acc = 0;
    for (int j = 0; j < N; ++j) {
        const int i0 = imax(0, j - KU), i1 = imin(N - 1, j + KL);
        for (int i = i0 + (int) threadIdx.x; i <= i1; i += 32) {
            const double2 v = __ldg(ab + KU + i - j + (long long) j * src.ldab);
            acc = fma(v.x, v.x, fma(v.y, v.y, acc));
        }
    }
    for (int off = 16; off; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
    if (threadIdx.x == 0) out[s] = sqrt(acc);
}

// ||A||_F of the synthetic model from the per-case band Gram matrix:
// sum_{e,f} sum_{p,q} |cM M + cD1 D1 + cD2 D2|^2, minus the rows replaced by
// Dirichlet identity rows, plus one per such row.  gram[0..5] are the sums
// over the whole band of MM, MD1, MD2, D1D1, D1D2, D2D2; gram[6..11] and
// gram[12..17] the same over rows p = 0 and p = n-1.
__device__ double quad_form(const double *G, sgb_coef a, sgb_coef b, sgb_coef c)
{
    const double aa = a.re * a.re + a.im * a.im, bb = b.re * b.re + b.im * b.im,
                 cc = c.re * c.re + c.im * c.im;
    const double ab = a.re * b.re + a.im * b.im, ac = a.re * c.re + a.im * c.im,
                 bc = b.re * c.re + b.im * c.im;
    return aa * G[0] + 2 * ab * G[1] + 2 * ac * G[2] + bb * G[3] + 2 * bc * G[4] + cc * G[5];
}

__global__ void k_afrob_model(int nsys, ModelSource ms, const double *__restrict__ gram,
                              double *__restrict__ out)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsys) return;
    const sgb_case &cs = ms.cs;
    const int S = cs.S;
    double acc = 0;
    for (int e = 0; e < S; ++e) {
        const bool dir = (cs.dirichlet_mask >> e) & 1u;
        for (int f = 0; f < S; ++f) {
            sgb_coef cM, cD1, cD2;
            sgb_block_coefs(&cs, e, f, ms.phi, ms.kx[s], ms.kz[s], &cM, &cD1, &cD2);
            acc += quad_form(gram, cM, cD1, cD2);
            if (dir) acc -= quad_form(gram + 6, cM, cD1, cD2) + quad_form(gram + 12, cM, cD1, cD2);
        }
        if (dir) acc += 2.0;
    }
    out[s] = sqrt(fmax(acc, 0.0));
}

static cudaError_t sync_count(const int *d, int *h, cudaStream_t st)
{
    cudaError_t e = cudaMemcpyAsync(h, d, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(st);
}

// Workspace layout (device), carved from one allocation.  The same walk
// sizes the workspace (base == nullptr) and carves it, so they cannot drift.
struct Carve {
    char *p; size_t off = 0;
    template <typename T> T *take(size_t n)
    {
        T *r = p ? reinterpret_cast<T *>(p + off) : nullptr;
        off += (n * sizeof(T) + 255) & ~size_t(255);
        return r;
    }
};

struct RefineLayout {
    float2 *fac32; int *ipiv32, *info32; float2 *y32;
    double2 *fac64; int *ipiv64, *info64; double2 *r;
    RefineState rs;
    double *rnorm, *xnorm, *afrob, *bnorm;
    int *listS, *listS2, *listD, *listD2, *cnt;
};

static size_t carve_layout(const RefineProblem &P, char *base, RefineLayout &Lo)
{
    const int nsys = P.nsys, N = P.g.N;
    Carve cv{base};
    Lo.fac32 = cv.take<float2>((size_t) nsys * P.g.fac_elems());
    Lo.ipiv32 = cv.take<int>((size_t) nsys * N);
    Lo.info32 = cv.take<int>(nsys);
    Lo.y32 = cv.take<float2>((size_t) nsys * N);
    Lo.fac64 = cv.take<double2>((size_t) P.nslot64 * P.g.fac_elems());
    Lo.ipiv64 = cv.take<int>((size_t) P.nslot64 * N);
    Lo.info64 = cv.take<int>(P.nslot64);
    Lo.r = cv.take<double2>((size_t) nsys * N);
    RefineState &rs = Lo.rs;
    rs.res = cv.take<double>(nsys); rs.lastres = cv.take<double>(nsys);
    rs.tolconst = cv.take<double>(nsys); rs.tol = cv.take<double>(nsys);
    rs.tolsc = cv.take<double>(nsys);
    Lo.rnorm = cv.take<double>(nsys); Lo.xnorm = cv.take<double>(nsys);
    Lo.afrob = cv.take<double>(nsys); Lo.bnorm = cv.take<double>(nsys);
    rs.status = cv.take<int>(nsys); rs.siter = cv.take<int>(nsys);
    rs.diter = cv.take<int>(nsys); rs.info = cv.take<int>(nsys);
    rs.fact = cv.take<char>((size_t) nsys);
    Lo.listS = cv.take<int>(nsys); Lo.listS2 = cv.take<int>(nsys);
    Lo.listD = cv.take<int>(nsys); Lo.listD2 = cv.take<int>(nsys);
    Lo.cnt = cv.take<int>(16);   // [0] S  [1] S'  [2] D  [4] chunk  [5,7,8] D lists
    rs.use_eps = (P.tolsc == 0.0);
    return cv.off;
}

size_t refine_workspace_bytes(const RefineProblem &P)
{
    RefineLayout Lo;
    return carve_layout(P, nullptr, Lo);
}

// The complex64 factor of a model problem (trans 'N') as one plan of a
// ragged batch: its outputs and active list in the refinement workspace.
int refine_ragged_desc(const RefineProblem &P, void *workspace, RaggedDesc &d)
{
    if (!P.model || P.trans != 'N' || P.siter < 0) return (int) cudaErrorInvalidValue;
    RefineLayout Lo;
    carve_layout(P, reinterpret_cast<char *>(workspace), Lo);
    d.g = P.g; d.ms = P.ms;
    d.fac = Lo.fac32; d.fac_stride = P.g.fac_elems(); d.ipiv = Lo.ipiv32; d.info = Lo.info32;
    d.rhs = P.b; d.rhs_stride = P.b_stride; d.y = Lo.y32; d.y_stride = P.g.N;
    d.sys_list = Lo.listS; d.d_count = Lo.cnt + 0;
    return 0;
}

__global__ void k_fill(int n, double *__restrict__ p, double v)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

__global__ void k_copy_rows(int nsys, const double2 *__restrict__ src, long long ss,
                            double2 *__restrict__ dst, long long ds, int N)
{
    const long long t = (long long) blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long) nsys * N) return;
    const long long s = t / N, i = t - s * N;
    dst[s * ds + i] = src[s * ss + i];
}

int refine_batched(const RefineProblem &P, void *workspace, size_t workspace_bytes,
                   RefineOutputs &out, cudaStream_t st)
{
    const int nsys = P.nsys, N = P.g.N;
    if (nsys == 0) return 0;
    if (P.nslot64 < 1 || !P.host_count) return (int) cudaErrorInvalidValue;
    if (workspace_bytes < refine_workspace_bytes(P)) return (int) cudaErrorInvalidValue;
    RefineLayout Lo;
    carve_layout(P, reinterpret_cast<char *>(workspace), Lo);
    float2 *fac32 = Lo.fac32; int *ipiv32 = Lo.ipiv32, *info32 = Lo.info32;
    float2 *y32 = Lo.y32; double2 *fac64 = Lo.fac64;
    int *ipiv64 = Lo.ipiv64, *info64 = Lo.info64;
    double2 *r = Lo.r;
    RefineState rs = Lo.rs;
    double *rnorm = Lo.rnorm, *xnorm = Lo.xnorm, *afrob = Lo.afrob, *bnorm = Lo.bnorm;
    int *listS = Lo.listS, *listS2 = Lo.listS2, *listD = Lo.listD, *listD2 = Lo.listD2;
    int *cnt = Lo.cnt;

    int *hcnt = P.host_count;
    PhaseTimer dummy;
    PhaseTimer &tm = P.timer ? *P.timer : dummy;
    const int T = 128, B = (nsys + T - 1) / T;
    const long long tot = (long long) nsys * N;
    const unsigned EB = (unsigned) ((tot + 255) / 256);
    cudaError_t e;
#define TRY(x) do { e = (x); if (e != cudaSuccess) return (int) e; } while (0)
    if (P.stage != 2) {
    TRY(cudaMemsetAsync(cnt, 0, 16 * sizeof(int), st));

    // r = b, x = 0, ||b||, ||A||_F
    tm.begin("refine_init", st);
    count_launch(5);
    k_copy_rows<<<EB, 256, 0, st>>>(nsys, P.b, P.b_stride, r, N, N);
    k_zero_x<<<EB, 256, 0, st>>>(nsys, P.x, P.x_stride, N);
    k_bnorm<<<nsys, 32, 0, st>>>(nsys, P.b, P.b_stride, N, bnorm);
    if (P.tolsc != 0.0) {
        if (P.afrob_in >= 0) k_fill<<<B, T, 0, st>>>(nsys, afrob, P.afrob_in);
        else if (P.model) k_afrob_model<<<B, T, 0, st>>>(nsys, P.ms, P.gram, afrob);
        else k_afrob_packed<<<nsys, 32, 0, st>>>(nsys, N, P.g.KL, P.g.KU, P.src, afrob);
    }
    k_refine_init<<<B, T, 0, st>>>(nsys, rs, afrob, P.tolsc, N, P.siter, P.diter, bnorm,
                                   listS, cnt + 0, listD, cnt + 2);
    TRY(cudaGetLastError());
    tm.end(st);
    }
    if (P.stage == 1) return 0;   // the caller factors (ragged factor), then stage 2

    ResidualArgs ra;
    ra.trans = P.resid_trans; ra.nsys = nsys; ra.N = N; ra.KL = P.g.KL; ra.KU = P.g.KU;
    ra.model = P.model; ra.src = P.src; ra.ms = P.ms;
    ra.b = P.b; ra.b_stride = P.b_stride; ra.x = P.x; ra.x_stride = P.x_stride;
    ra.r = r; ra.r_stride = N; ra.rnorm2 = rnorm; ra.xnorm2 = xnorm;

    // ---- complex64 factor (+ forward elimination of b), first solve, loop --
    int iters = 0;
    if (P.siter >= 0) {
        const bool fuse = (P.trans == 'N');
        GbtrfArgs fa;
        fa.prec = 'C'; fa.g = P.g; fa.nsys = nsys; fa.model = P.model; fa.src = P.src;
        fa.ms = P.ms; fa.fac = fac32; fa.fac_stride = P.g.fac_elems(); fa.ipiv = ipiv32;
        fa.info = info32; fa.sys_list = listS; fa.nlist = nsys; fa.d_count = cnt + 0;
        if (fuse) { fa.rhs = P.b; fa.rhs_stride = P.b_stride; fa.y = y32; fa.y_stride = N; }
        if (P.stage != 2) {
            tm.begin("factor_c64", st);
            count_launch(1);
            TRY(launch_gbtrf(fa, st));
            tm.end(st);
        }
        count_launch(1);
        k_refine_after_sfactor<<<B, T, 0, st>>>(rs, info32, listS, cnt + 0, P.diter, listD, cnt + 2);
        GbtrsArgs sa;
        sa.prec = 'C'; sa.trans = P.trans; sa.g = P.g; sa.nsys = nsys; sa.fac = fac32;
        sa.fac_stride = P.g.fac_elems(); sa.ipiv = ipiv32; sa.x = P.x; sa.x_stride = P.x_stride;
        sa.fwd_done = fuse;
        if (fuse) { sa.yin = y32; sa.b_stride = N; } else { sa.b = P.b; sa.b_stride = P.b_stride; }
        sa.ywork = y32;
        sa.accumulate = false; sa.sys_list = listS; sa.nlist = nsys; sa.d_count = cnt + 0;
        sa.status = rs.status; sa.status_want = ST_SINGLE;
        tm.begin(fuse ? "backsolve_c64" : "solve_c64", st);
        count_launch(1);
        TRY(launch_gbtrs(sa, st));
        tm.end(st);

        int *cur = listS, *nxt = listS2, *ccur = cnt + 0, *cnxt = cnt + 1;
        int ncur = nsys;
        if (P.graph) {
            // capturable: a fixed number of correction solves, grids bounded
            // by the device counts; a final residual + decision, then the cap
            for (int it = 0; it <= P.graph_siter; ++it) {
                ra.sys_list = cur; ra.nlist = nsys; ra.d_count = ccur;
                ra.status = rs.status; ra.status_want = ST_SINGLE;
                count_launch(4);
                TRY(launch_residual(ra, st));
                TRY(cudaMemsetAsync(cnxt, 0, sizeof(int), st));
                k_refine_decide<<<B, T, 0, st>>>(rs, 0, rnorm, xnorm, P.aiter, P.siter, P.diter,
                                                 cur, ccur, nxt, cnxt, listD, cnt + 2);
                TRY(cudaGetLastError());
                if (it == P.graph_siter) {
                    k_refine_cap<<<B, T, 0, st>>>(rs, nxt, cnxt, P.diter, listD, cnt + 2);
                    TRY(cudaGetLastError());
                    break;
                }
                GbtrsArgs ca = sa;
                ca.fwd_done = false; ca.yin = nullptr; ca.b = r; ca.b_stride = N;
                ca.accumulate = true; ca.sys_list = nxt; ca.nlist = nsys; ca.d_count = cnxt;
                TRY(launch_gbtrs(ca, st));
                std::swap(cur, nxt); std::swap(ccur, cnxt);
            }
            iters = P.graph_siter + 1;
        } else {
            for (;;) {
                ra.sys_list = cur; ra.nlist = ncur; ra.d_count = ccur;
                ra.status = rs.status; ra.status_want = ST_SINGLE;
                tm.begin("residual_f64", st);
                count_launch(2);
                TRY(launch_residual(ra, st));
                tm.end(st);
                TRY(cudaMemsetAsync(cnxt, 0, sizeof(int), st));
                k_refine_decide<<<B, T, 0, st>>>(rs, 0, rnorm, xnorm, P.aiter, P.siter, P.diter,
                                                 cur, ccur, nxt, cnxt, listD, cnt + 2);
                TRY(cudaGetLastError());
                TRY(sync_count(cnxt, hcnt, st));
                ++iters;
                if (*hcnt == 0 || iters > P.siter + 1) break;
                ncur = *hcnt;
                GbtrsArgs ca = sa;
                ca.fwd_done = false; ca.yin = nullptr; ca.b = r; ca.b_stride = N;
                ca.accumulate = true; ca.sys_list = nxt; ca.nlist = ncur; ca.d_count = cnxt;
                tm.begin("solve_c64", st);
                count_launch(1);
                TRY(launch_gbtrs(ca, st));
                tm.end(st);
                std::swap(cur, nxt); std::swap(ccur, cnxt);
            }
        }
    }
    out.single_iters = iters;

    // ---- complex128 fallback, in chunks of nslot64 factor slots ------------
    int d_iters = 0;
    auto fallback_chunk = [&](int *clist, int chunk_host, int iters_max, bool host_loop) -> int {
        GbtrfArgs da;
        da.prec = 'Z'; da.g = P.g; da.nsys = nsys; da.model = P.model; da.src = P.src;
        da.ms = P.ms; da.fac = fac64; da.fac_stride = P.g.fac_elems(); da.ipiv = ipiv64;
        da.info = info64; da.sys_list = clist; da.nlist = chunk_host; da.d_count = cnt + 4;
        da.slot_mode = true;
        tm.begin("factor_c128_fallback", st);
        count_launch(2);
        TRY(launch_gbtrf(da, st));
        tm.end(st);
        TRY(cudaMemsetAsync(cnt + 5, 0, sizeof(int), st));
        k_refine_enter_double<<<(chunk_host + T - 1) / T, T, 0, st>>>(rs, clist, cnt + 4, info64, 0,
                                                                      listD2, cnt + 5);
        TRY(cudaGetLastError());
        int active = 1, it = 0;
        if (host_loop) {
            TRY(sync_count(cnt + 5, hcnt, st));
            active = *hcnt;
        }
        while (active > 0 && it < iters_max) {
            GbtrsArgs sa;
            sa.prec = 'Z'; sa.trans = P.trans; sa.g = P.g; sa.nsys = nsys; sa.fac = fac64;
            sa.fac_stride = P.g.fac_elems(); sa.ipiv = ipiv64; sa.b = r; sa.b_stride = N;
            sa.x = P.x; sa.x_stride = P.x_stride; sa.accumulate = true;
            sa.sys_list = clist; sa.nlist = chunk_host; sa.d_count = cnt + 4; sa.slot_mode = true;
            sa.status = rs.status; sa.status_want = ST_DOUBLE;
            tm.begin("solve_c128_fallback", st);
            count_launch(3);
            TRY(launch_gbtrs(sa, st));
            tm.end(st);
            ra.sys_list = clist; ra.nlist = chunk_host; ra.d_count = cnt + 4;
            ra.status = rs.status; ra.status_want = ST_DOUBLE;
            TRY(launch_residual(ra, st));
            TRY(cudaMemsetAsync(cnt + 7, 0, sizeof(int), st));
            k_refine_decide<<<(chunk_host + T - 1) / T, T, 0, st>>>(rs, 1, rnorm, xnorm, P.aiter,
                                                                   P.siter, P.diter, clist, cnt + 4,
                                                                   listD2, cnt + 7, listD2, cnt + 8);
            TRY(cudaGetLastError());
            if (host_loop) {
                TRY(sync_count(cnt + 7, hcnt, st));
                active = *hcnt;
            }
            ++it;
        }
        d_iters = std::max(d_iters, it);
        return 0;
    };
    out.d_unserved = cnt + 9;
    if (P.graph) {
        // capturable: one chunk of at most nslot64 systems, fixed iterations
        count_launch(1);
        k_chunk_count<<<1, 1, 0, st>>>(cnt + 2, P.nslot64, cnt + 4, cnt + 9);
        TRY(cudaGetLastError());
        if (P.diter >= 0) {
            int rc = fallback_chunk(listD, P.nslot64, imax(P.graph_diter, 1), false);
            if (rc) return rc;
        }
        out.n_double = -1;       // on the device: cnt[2]
    } else {
        TRY(cudaMemsetAsync(cnt + 9, 0, sizeof(int), st));
        TRY(sync_count(cnt + 2, hcnt, st));
        const int nd = *hcnt;
        out.n_double = nd;
        for (int base = 0; base < nd; base += P.nslot64) {
            const int chunk = std::min(P.nslot64, nd - base);
            TRY(cudaMemcpyAsync(cnt + 4, &chunk, sizeof(int), cudaMemcpyHostToDevice, st));
            int rc = fallback_chunk(listD + base, chunk, P.diter + 2, true);
            if (rc) return rc;
        }
    }
    out.double_iters = d_iters;
    count_launch(1);
    k_refine_finalize<<<nsys, 32, 0, st>>>(nsys, rs, P.x, P.x_stride, N);
    TRY(cudaGetLastError());
    out.state = rs;
    out.rnorm = rnorm;
    out.xnorm = xnorm;
    out.r = r;
    out.info32 = info32;
    out.afrob = afrob;
    out.fac32 = fac32; out.fac64 = fac64; out.ipiv32 = ipiv32; out.ipiv64 = ipiv64;
#undef TRY
    return 0;
}

}  // namespace sgb
