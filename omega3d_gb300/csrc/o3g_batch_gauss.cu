// o3g_batch_gauss.cu -- batched persistent pair kernels, GAUSS core.
#include "o3g_batch_impl.cuh"

namespace o3g {
O3G_DEFINE_BATCH_CORE(CORE_GAUSS)
}  // namespace o3g
