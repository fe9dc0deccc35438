// FP32 instantiation of the operator kernels (smoother, residual, transfers of the
// mixed-precision cycle).
#include <type_traits>

#include "ae_kernels.cuh"

#define AE_REAL float
#include "ae_kernels_common.inc"
#undef AE_REAL

namespace ae {
AE_INST_COPY(float, float)
AE_INST_COPY(float, double)
}  // namespace ae
