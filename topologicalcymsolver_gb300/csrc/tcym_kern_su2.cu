// SU(2) instantiations of the kernels (FP32 and FP64 storage).
#include "tcym_kernels.cuh"

namespace tcym {
template struct Launch<FMT_SU2_F32>;
template struct Launch<FMT_SU2_F64>;
}  // namespace tcym
