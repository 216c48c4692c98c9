// Blocked band LU kernels, complex64, panel width 4.
#include "gbtrf_blk.cuh"

namespace sgb {
SGB_BLK_INSTANTIATE(float, 4, launch_blk_c4)
}  // namespace sgb
