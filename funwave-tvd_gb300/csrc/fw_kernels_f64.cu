// FP64 instantiation of the kernels.  Compiled with -fmad=false so that
// every multiply and add is rounded separately, in the operation order of
// the reference's statements, like the CPU oracle.
#include "fw_kernels.cuh"

namespace fw {
INST(double)
}  // namespace fw
