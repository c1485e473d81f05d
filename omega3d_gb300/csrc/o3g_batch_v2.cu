// o3g_batch_v2.cu -- batched persistent pair kernels, V2 core.
#include "o3g_batch_impl.cuh"

namespace o3g {
O3G_DEFINE_BATCH_CORE(CORE_V2)
}  // namespace o3g
