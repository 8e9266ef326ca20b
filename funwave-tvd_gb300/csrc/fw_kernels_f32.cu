// Mixed-precision instantiation of the kernels (float fields, double
// tridiagonal u/v recovery) and the shared conversion kernels.
#define FW_SHARED_DEFS
#include "fw_kernels.cuh"

namespace fw {
INST(float)
}  // namespace fw
