// o3g_pair_rm.cu -- instantiates the points_affect_points pipeline for the RM core.
#include "o3g_pair_impl.cuh"
namespace o3g {
O3G_DEFINE_PTPT_CORE(CORE_RM)
}  // namespace o3g
