// SU(3) instantiations of the kernels (FP32 two-row and FP64 full storage).
#define TCYM_KERNEL_TU
#include "tcym_batch.cuh"

namespace tcym {
template struct Launch<FMT_SU3_F32>;
template struct Launch<FMT_SU3_F64>;
template struct LaunchBatch<FMT_SU3_F32>;
template struct LaunchBatch<FMT_SU3_F64>;
}  // namespace tcym
