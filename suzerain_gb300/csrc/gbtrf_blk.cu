// Blocked batched band LU: shared-memory size, supported shapes, the default
// shape choice and the dispatch over (precision, panel width NB, warps per
// system NW).  The kernel template is in gbtrf_blk.cuh; gbtrf_blk_inst.cu,
// compiled once per (precision, NB, warp family), instantiates it.
#include "gbtrf_blk.cuh"

#include <algorithm>
#include <atomic>
#include <mutex>
#include <map>
#include <tuple>

namespace sgb {

// nw > 0: the phased kernel with nw warps (nw > 1 stages the entering
// rows); nw < 0: the lookahead kernel with -nw warps.
size_t gbtrf_blk_smem_bytes(int prec_bytes, const FactorGeom &g, int S, int nb, int nw)
{
    const size_t el = 2 * (size_t) prec_bytes;
    if (nw > 0) {
        const int WR = g.KL + nb, WC = g.KL + g.KU + nb, P = blk_pitch(WC);
        const size_t stage = nw > 1 ? (size_t) nb * WC + nb : 0;
        return ((size_t) (WR + 1) * P + WR + stage + 3 * (size_t) S * S) * el
             + (size_t) nb * sizeof(int) + 4 * sizeof(int) + 12 * 8 + 16;
    }
    // lookahead: panel J-1's rows and columns stay, plus the staged rows
    const int WR = g.KL + 2 * nb, WC = g.KL + g.KU + 2 * nb, P = blk_pitch(WC);
    return ((size_t) (WR + 1) * P + WR + (size_t) nb * WC + nb + 3 * (size_t) S * S) * el
         + (size_t) nb * sizeof(int) + 4 * sizeof(int) + 12 * 8 + 16;
}

// Rows of the trailing update per thread: KL <= 4 NW MAXTR (MAXTR 13, 7, 4
// for NW 1, 2, 4); the panel's rows per lane; row and column indices of the
// model's band assembly below 65536; the window within one CTA's shared
// memory (either kernel).
bool gbtrf_blk_supported(const FactorGeom &g, int nb, int nw)
{
    if (nb != 4 && nb != 8 && nb != 16) return false;
    if (nw == 3) {
        // the three-warp shape of the specialized complex64 instances
        const int kb = gbtrf_spec_band(g);
        return nb == 4 && kb != 0 && spec_has_w3(kb);
    }
    if (nw != 1 && nw != 2 && nw != 4) return false;
    const int maxkl = nw == 1 ? 52 : nw == 2 ? 56 : 64;
    if (g.KL > maxkl || g.N >= 65536) return false;
    return gbtrf_blk_smem_bytes(sizeof(double), g, 8, nb, -(nw > 1 ? nw : 2)) <= 227 * 1024;
}

namespace {
std::mutex g_tune_mu;
std::map<std::tuple<char, int, int, int>, std::pair<int, int>> g_tune;
}  // namespace

void gbtrf_blk_set_choice(char prec, const FactorGeom &g, int nb, int nw)
{
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[std::make_tuple(prec, g.N, g.KL, g.KU)] = {nb, nw};
}

void gbtrf_blk_choice(char prec, const FactorGeom &g, int &nb, int &nw, bool model)
{
    if (nb > 0 && nw != 0) return;          // nw < 0: the lookahead form, given
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune.find(std::make_tuple(prec, g.N, g.KL, g.KU));
        if (it != g_tune.end()) {
            if (nb <= 0) nb = it->second.first;
            if (nw == 0) nw = it->second.second;
            return;
        }
    }
    // Measured on GB300 at N = 960, KL = KU = 34: complex64 is fastest with
    // narrow panels and two warps, complex128 (FP64-throughput bound) with
    // narrow panels and one warp.
    if (nb <= 0) nb = 4;
    if (nw == 0) {
        // complex64 beyond KL = 40: four warps (KL = 48, N = 1344: 18 %
        // faster than two with model rows, 46 % with a packed band)
        nw = g.KL > 56 || (prec == 'C' && g.KL > 40) ? 4 : (prec == 'C' || g.KL > 52) ? 2 : 1;
        // the three-warp shape: every specialized band with a packed
        // source; with model rows at KL = 34 (5 % faster there, N = 960),
        // while KL = 24 measured faster with two
        const int kb = prec == 'C' && nb == 4 ? gbtrf_spec_band(g) : 0;
        if (kb && spec_has_w3(kb) && (!model || kb == 34)) nw = 3;
    }
}

namespace {
template <typename R, int NB>
cudaError_t launch_nb(const GbtrfArgs &a, int nw, cudaStream_t st)
{
    if (a.variant == 2 && nw > 1) return launch_blk_fam<R, NB, 0>(a, nw, st);
    if (nw == 1) return launch_blk_fam<R, NB, 1>(a, nw, st);
    if (nw == 2) return launch_blk_fam<R, NB, 2>(a, nw, st);
    return launch_blk_fam<R, NB, 4>(a, nw, st);
}
}  // namespace

namespace {
std::atomic<int> g_spec{1};
}  // namespace

void gbtrf_set_specialized(int on) { g_spec.store(on ? 1 : 0); }

int gbtrf_spec_band(const FactorGeom &g)
{
    if (!g_spec.load() || g.KL != g.KU || g.N % 4 != 0) return 0;
    for (int kb : kSpecBands)
        if (g.KL == kb) return kb;
    return 0;
}

cudaError_t launch_blk_spec_any(const GbtrfArgs &a, int nw, cudaStream_t st, bool *done)
{
    *done = false;
    if (a.prec != 'C' || (nw != 2 && nw != 3)) return cudaSuccess;
    const int kb = gbtrf_spec_band(a.g);
    if (kb == 0 || (nw == 3 && !spec_has_w3(kb))) return cudaSuccess;
    *done = true;
    if (kb == 24) return launch_blk_spec<24>(a, nw, st);
    return launch_blk_spec<34>(a, nw, st);
}

// Kind of the ragged factor instance for a plan of geometry g: the
// specialized bandwidth instance as KB (two warps: the three-warp form of
// the ragged kernel, whose descriptor adds live registers, still spills at
// 80), else the generic one as -(10 warps + rows per thread): -25 for
// KL <= 40, -43 for KL <= 48, -44 for KL <= 56 (the default shapes of the
// phased kernel).
int ragged_kind(const FactorGeom &g)
{
    const int kb = gbtrf_spec_band(g);
    return kb ? kb : (g.KL <= 40 ? -25 : g.KL <= 48 ? -43 : -44);
}

cudaError_t launch_gbtrf_ragged(const RaggedDesc *descs, const int2 *items, int nitems, int kind,
                                size_t smem, cudaStream_t st)
{
    if (nitems <= 0) return cudaSuccess;
    void (*kern)(const RaggedDesc *, const int2 *) = nullptr;
    int nw = 2;
    switch (kind) {
    case -25: kern = k_gbtrf_ragged<2, 5>; break;
    case -43: kern = k_gbtrf_ragged<4, 3>; nw = 4; break;
    case -44: kern = k_gbtrf_ragged<4, 4>; nw = 4; break;
    case 24: kern = k_gbtrf_ragged<2, spec_maxtr<2>(), 24, 24, true>; break;
    case 34: kern = k_gbtrf_ragged<2, spec_maxtr<2>(), 34, 34, true>; break;
    default: return cudaErrorInvalidValue;
    }
    cudaError_t e = smem_attr((const void *) kern, smem);
    if (e != cudaSuccess) return e;
    kern<<<nitems, 32 * nw, smem, st>>>(descs, items);
    return cudaGetLastError();
}

cudaError_t launch_gbtrf_blk(const GbtrfArgs &a, int nb, int nw, cudaStream_t st)
{
    if (a.prec == 'Z') {
        if (nw == 3) nw = 2;     // three warps exist for complex64 only
        if (nb == 4) return launch_nb<double, 4>(a, nw, st);
        if (nb == 16) return launch_nb<double, 16>(a, nw, st);
        return launch_nb<double, 8>(a, nw, st);
    }
    if (nb == 4 && a.variant != 2 && !a.prof) {
        bool done = false;
        const cudaError_t e = launch_blk_spec_any(a, nw, st, &done);
        if (done) return e;
    }
    if (nw == 3) nw = 2;     // no specialized instance: the generic two-warp kernel
    if (nb == 4) return launch_nb<float, 4>(a, nw, st);
    if (nb == 16) return launch_nb<float, 16>(a, nw, st);
    return launch_nb<float, 8>(a, nw, st);
}

}  // namespace sgb
