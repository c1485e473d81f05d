// o3g_sort.cuh -- Morton ordering of point sets (see o3g_sort.cu).
#pragma once
#include "o3g_common.cuh"

namespace o3g {
// workspace bytes needed by morton_sort for n points
size_t morton_sort_bytes(int n);
// perm[k] = index of the k-th point in Z-order (30-bit codes over the set's bounding box)
template <class I>
int32_t morton_sort(const I* x, const I* y, const I* z, int n, uint32_t* perm, char* ws, cudaStream_t st);
}  // namespace o3g
