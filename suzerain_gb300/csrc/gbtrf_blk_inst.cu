// Blocked band LU kernels of one (precision, panel width, warp family).
// The build compiles this file once per triple with -DSGB_BLK_R=float|double
// -DSGB_BLK_NB=4|8|16 -DSGB_BLK_FAM=0|1|2|4 (24 objects, compiled in
// parallel), and once per specialized bandwidth with -DSGB_BLK_SPEC=KB (the
// complex64 phased kernel with KL = KU = KB fixed at compile time); without
// those definitions it instantiates nothing.
#include "gbtrf_blk.cuh"

namespace sgb {

template <typename R, int NB, int FAM>
cudaError_t launch_blk_fam(const GbtrfArgs &a, int nw, cudaStream_t st)
{
    const int KL = a.g.KL;
    if constexpr (FAM == 0)
        return nw == 2 ? launch_cta_r<R, NB, 2, 1, true>(a, st)
                       : launch_cta_r<R, NB, 4, 1, true>(a, st);
    else if constexpr (FAM == 1)
        return KL <= 36 ? launch_cta_r<R, NB, 1, 9, false>(a, st)
                        : launch_cta_r<R, NB, 1, 13, false>(a, st);
    else if constexpr (FAM == 2)
        return KL <= 40 ? launch_cta_r<R, NB, 2, 5, false>(a, st)
                        : launch_cta_r<R, NB, 2, 7, false>(a, st);
    else
        return KL <= 48 ? launch_cta_r<R, NB, 4, 3, false>(a, st)
                        : launch_cta_r<R, NB, 4, 4, false>(a, st);
}

template <int KB, int W>
cudaError_t launch_blk_spec_w(const GbtrfArgs &a, cudaStream_t st)
{
    constexpr int MT = spec_maxtr<W>();
    const bool fwd = a.rhs != nullptr;
    if (a.model)
        return fwd ? launch_cta_one<float, 4, W, MT, false, true, true, KB, KB, true>(a, st)
                   : launch_cta_one<float, 4, W, MT, false, true, false, KB, KB, true>(a, st);
    return fwd ? launch_cta_one<float, 4, W, MT, false, false, true, KB, KB, true>(a, st)
               : launch_cta_one<float, 4, W, MT, false, false, false, KB, KB, true>(a, st);
}

template <int KB>
cudaError_t launch_blk_spec(const GbtrfArgs &a, int nw, cudaStream_t st)
{
    if constexpr (spec_has_w3(KB))
        if (nw == 3) return launch_blk_spec_w<KB, 3>(a, st);
    return launch_blk_spec_w<KB, 2>(a, st);
}

#if defined(SGB_BLK_SPEC)
template cudaError_t launch_blk_spec<SGB_BLK_SPEC>(const GbtrfArgs &, int, cudaStream_t);
#endif

#if defined(SGB_BLK_R) && defined(SGB_BLK_NB) && defined(SGB_BLK_FAM)
template cudaError_t launch_blk_fam<SGB_BLK_R, SGB_BLK_NB, SGB_BLK_FAM>(
    const GbtrfArgs &, int, cudaStream_t);
#endif

}  // namespace sgb
