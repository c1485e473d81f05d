// o3g_batch_exp.cu -- batched persistent pair kernels, EXP core.
#include "o3g_batch_impl.cuh"

namespace o3g {
O3G_DEFINE_BATCH_CORE(CORE_EXP)
}  // namespace o3g
