// Kernel instantiations, SU(3) FP64: the batched (ensemble) kernels.
// One instantiation set per unit, so that the units compile in parallel.
#define TCYM_KERNEL_TU
#include "tcym_batch.cuh"

namespace tcym {
template struct LaunchBatch<FMT_SU3_F64>;
}  // namespace tcym
