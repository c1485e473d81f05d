// o3g_batch_wl.cu -- batched persistent pair kernels, WL core.
#include "o3g_batch_impl.cuh"

namespace o3g {
O3G_DEFINE_BATCH_CORE(CORE_WL)
}  // namespace o3g
