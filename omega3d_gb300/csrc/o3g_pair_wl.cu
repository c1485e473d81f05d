// o3g_pair_wl.cu -- instantiates the points_affect_points pipeline for the WL core.
#include "o3g_pair_impl.cuh"
namespace o3g {
O3G_DEFINE_PTPT_CORE(CORE_WL)
}  // namespace o3g
