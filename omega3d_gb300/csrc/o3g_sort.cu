// o3g_sort.cu -- Morton (Z-order) permutation of a point set on the device.
//
// The pair kernels of the cores with distance branches (Gaussian, compact exponential)
// sweep sources and targets in this order, so that a block's targets and a tile's
// sources each occupy a compact box and whole (target block, source tile) pairs can be
// classified as far field by their bounding boxes (no per-pair divergence).
#include "o3g_sort.cuh"

#include <cub/device/device_radix_sort.cuh>

namespace o3g {

// float -> int with the same ordering (for atomicMin/atomicMax on floats)
__device__ __forceinline__ int ord(float f) {
  const int i = __float_as_int(f);
  return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float unord(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

__global__ void k_bbox_init(int* bb) {
  if (threadIdx.x < 3) bb[threadIdx.x] = 0x7fffffff;
  else if (threadIdx.x < 6) bb[threadIdx.x] = (int)0x80000000;
}

template <class I>
__global__ void k_bbox(const I* __restrict__ x, const I* __restrict__ y, const I* __restrict__ z, int n, int* bb) {
  float lo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, hi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float v[3] = {(float)x[i], (float)y[i], (float)z[i]};
#pragma unroll
    for (int d = 0; d < 3; ++d) { lo[d] = fminf(lo[d], v[d]); hi[d] = fmaxf(hi[d], v[d]); }
  }
#pragma unroll
  for (int d = 0; d < 3; ++d)
    for (int o = 16; o > 0; o >>= 1) {
      lo[d] = fminf(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
      hi[d] = fmaxf(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
    }
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int d = 0; d < 3; ++d) { atomicMin(&bb[d], ord(lo[d])); atomicMax(&bb[3 + d], ord(hi[d])); }
  }
}

template <class I>
__global__ void k_morton(const I* __restrict__ x, const I* __restrict__ y, const I* __restrict__ z, int n,
                         const int* __restrict__ bb, uint32_t* code, uint32_t* idx) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t q[3];
  const float v[3] = {(float)x[i], (float)y[i], (float)z[i]};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float lo = unord(bb[d]), hi = unord(bb[3 + d]);
    const float ext = hi - lo;
    float t = ext > 0.f ? (v[d] - lo) / ext : 0.f;
    t = fminf(fmaxf(t, 0.f), 1.f);
    q[d] = (uint32_t)(t * 1023.0f);
  }
  code[i] = spread3(q[0]) | (spread3(q[1]) << 1) | (spread3(q[2]) << 2);
  idx[i] = (uint32_t)i;
}

static size_t cub_bytes(int n) {
  size_t b = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, b, (const uint32_t*)nullptr, (uint32_t*)nullptr,
                                  (const uint32_t*)nullptr, (uint32_t*)nullptr, n, 0, 30);
  return b;
}

size_t morton_sort_bytes(int n) {
  return align_up(6 * sizeof(int)) + 3 * align_up((size_t)n * sizeof(uint32_t)) + align_up(cub_bytes(n));
}

template <class I>
int32_t morton_sort(const I* x, const I* y, const I* z, int n, uint32_t* perm, char* ws, cudaStream_t st) {
  Carve cv(ws);
  int* bb = cv.take<int>(6);
  uint32_t* code_in = cv.take<uint32_t>(n);
  uint32_t* code_out = cv.take<uint32_t>(n);
  uint32_t* idx_in = cv.take<uint32_t>(n);
  size_t tb = cub_bytes(n);
  void* temp = cv.take<char>(tb);
  k_bbox_init<<<1, 32, 0, st>>>(bb);
  int nb = (n + 255) / 256;
  if (nb > 1024) nb = 1024;
  k_bbox<I><<<nb, 256, 0, st>>>(x, y, z, n, bb);
  k_morton<I><<<(n + 255) / 256, 256, 0, st>>>(x, y, z, n, bb, code_in, idx_in);
  note_launch(3);
  O3G_CUDA_TRY(cub::DeviceRadixSort::SortPairs(temp, tb, code_in, code_out, idx_in, perm, n, 0, 30, st));
  O3G_CUDA_TRY(cudaGetLastError());
  return O3G_OK;
}

template int32_t morton_sort<float>(const float*, const float*, const float*, int, uint32_t*, char*, cudaStream_t);
template int32_t morton_sort<double>(const double*, const double*, const double*, int, uint32_t*, char*,
                                     cudaStream_t);

}  // namespace o3g
