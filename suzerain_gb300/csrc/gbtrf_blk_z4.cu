// Blocked band LU kernels, complex128, panel width 4.
#include "gbtrf_blk.cuh"

namespace sgb {
SGB_BLK_INSTANTIATE(double, 4, launch_blk_z4)
}  // namespace sgb
