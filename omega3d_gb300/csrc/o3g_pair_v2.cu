// o3g_pair_v2.cu -- instantiates the points_affect_points pipeline for the V2 core.
#include "o3g_pair_impl.cuh"
namespace o3g {
O3G_DEFINE_PTPT_CORE(CORE_V2)
}  // namespace o3g
