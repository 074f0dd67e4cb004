// Kernel instantiations, SU(2) FP32 (site pairs): single-lattice and batched kernels.
// One instantiation set per unit, so that the units compile in parallel.
#define TCYM_KERNEL_TU
#include "tcym_batch.cuh"

namespace tcym {
template struct Launch<FMT_SU2_F32>;
template struct LaunchBatch<FMT_SU2_F32>;
}  // namespace tcym
