// o3g_pair_gauss.cu -- instantiates the points_affect_points pipeline for the GAUSS core.
#include "o3g_pair_impl.cuh"
namespace o3g {
O3G_DEFINE_PTPT_CORE(CORE_GAUSS)
}  // namespace o3g
