// o3g_sort.cuh -- Morton ordering of point sets (see o3g_sort.cu).
#pragma once
#include "o3g_common.cuh"

namespace o3g {
// spread the low 10 bits of v so that bit k lands at bit 3k (one axis of a 30-bit Morton code)
__device__ __forceinline__ uint32_t spread3(uint32_t v) {
  v &= 0x3ffu;
  v = (v | (v << 16)) & 0x030000ffu;
  v = (v | (v << 8)) & 0x0300f00fu;
  v = (v | (v << 4)) & 0x030c30c3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

// workspace bytes needed by morton_sort for n points
size_t morton_sort_bytes(int n);
// perm[k] = index of the k-th point in Z-order (30-bit codes over the set's bounding box)
template <class I>
int32_t morton_sort(const I* x, const I* y, const I* z, int n, uint32_t* perm, char* ws, cudaStream_t st);
}  // namespace o3g
