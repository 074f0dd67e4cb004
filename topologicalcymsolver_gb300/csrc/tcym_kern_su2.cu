// SU(2) instantiations of the kernels (FP32 and FP64 storage).
#define TCYM_KERNEL_TU
#include "tcym_batch.cuh"

namespace tcym {
template struct Launch<FMT_SU2_F32>;
template struct Launch<FMT_SU2_F64>;
template struct LaunchBatch<FMT_SU2_F32>;
template struct LaunchBatch<FMT_SU2_F64>;
}  // namespace tcym
