// Blocked band LU kernels, complex64, panel width 8.
#include "gbtrf_blk.cuh"

namespace sgb {
SGB_BLK_INSTANTIATE(float, 8, launch_blk_c8)
}  // namespace sgb
