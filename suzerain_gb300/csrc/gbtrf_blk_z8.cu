// Blocked band LU kernels, complex128, panel width 8.
#include "gbtrf_blk.cuh"

namespace sgb {
SGB_BLK_INSTANTIATE(double, 8, launch_blk_z8)
}  // namespace sgb
