// Blocked band LU kernels, complex64, panel width 16.
#include "gbtrf_blk.cuh"

namespace sgb {
SGB_BLK_INSTANTIATE(float, 16, launch_blk_c16)
}  // namespace sgb
