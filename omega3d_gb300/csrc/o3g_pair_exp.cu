// o3g_pair_exp.cu -- instantiates the points_affect_points pipeline for the EXP core.
#include "o3g_pair_impl.cuh"
namespace o3g {
O3G_DEFINE_PTPT_CORE(CORE_EXP)
}  // namespace o3g
