// Blocked band LU kernels, complex128, panel width 16.
#include "gbtrf_blk.cuh"

namespace sgb {
SGB_BLK_INSTANTIATE(double, 16, launch_blk_z16)
}  // namespace sgb
