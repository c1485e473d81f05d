// o3g_batch_rm.cu -- batched persistent pair kernels, RM core.
#include "o3g_batch_impl.cuh"

namespace o3g {
O3G_DEFINE_BATCH_CORE(CORE_RM)
}  // namespace o3g
