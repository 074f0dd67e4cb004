// SU(3) instantiations of the kernels (FP32 two-row and FP64 full storage).
#include "tcym_kernels.cuh"

namespace tcym {
template struct Launch<FMT_SU3_F32>;
template struct Launch<FMT_SU3_F64>;
}  // namespace tcym
