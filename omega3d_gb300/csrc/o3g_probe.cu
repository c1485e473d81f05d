// o3g_probe.cu -- FP32 FMA throughput probe: the measured denominator of the pair
// kernels' roofline (their bound is the FP32 pipe, neither HBM nor tensor cores).
#include "o3g_common.cuh"

namespace o3g {

// 8 independent FMA chains per thread, `iters` rounds; every lane of every warp busy.
__global__ void __launch_bounds__(256) k_fma_probe(int iters, float seed, float* out) {
  float a0 = seed + threadIdx.x * 1e-7f, a1 = a0 + 1e-6f, a2 = a0 + 2e-6f, a3 = a0 + 3e-6f;
  float a4 = a0 + 4e-6f, a5 = a0 + 5e-6f, a6 = a0 + 6e-6f, a7 = a0 + 7e-6f;
  const float m = 0.999999f, c = 1e-7f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      a0 = fmaf(a0, m, c); a1 = fmaf(a1, m, c); a2 = fmaf(a2, m, c); a3 = fmaf(a3, m, c);
      a4 = fmaf(a4, m, c); a5 = fmaf(a5, m, c); a6 = fmaf(a6, m, c); a7 = fmaf(a7, m, c);
    }
  }
  const float s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
  if (s == 12345.678f) out[blockIdx.x] = s;  // practically never taken; keeps the chains live
}

}  // namespace o3g

extern "C" int32_t o3g_fp32_peak_probe(int32_t iters, void* stream, double* tflops, float* ms_out) {
  using namespace o3g;
  if (iters <= 0 || !tflops) {
    set_error("o3g_fp32_peak_probe: iters must be > 0 and tflops non-null");
    return O3G_ERR_INVALID_ARG;
  }
  DeviceFacts df;
  O3G_TRY(device_facts(&df));
  cudaStream_t st = (cudaStream_t)stream;
  Workspace* ws = nullptr;
  int nb = 0;
  O3G_TRY(occupancy_blocks((const void*)&k_fma_probe, 256, &nb));
  const int blocks = nb * df.num_sms;
  O3G_TRY(workspace_get(st, (size_t)blocks * sizeof(float), &ws));
  float* out = reinterpret_cast<float*>(ws->base);
  cudaEvent_t e0, e1;
  O3G_CUDA_TRY(cudaEventCreate(&e0));
  O3G_CUDA_TRY(cudaEventCreate(&e1));
  k_fma_probe<<<blocks, 256, 0, st>>>(iters / 4 + 1, 1.0f, out);  // warm-up
  O3G_CUDA_TRY(cudaEventRecord(e0, st));
  k_fma_probe<<<blocks, 256, 0, st>>>(iters, 1.0f, out);
  O3G_CUDA_TRY(cudaEventRecord(e1, st));
  O3G_CUDA_TRY(cudaEventSynchronize(e1));
  float ms = 0.f;
  O3G_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const double flops = 2.0 * 8.0 * 16.0 * (double)iters * 256.0 * (double)blocks;
  *tflops = flops / (ms * 1e-3) / 1e12;
  if (ms_out) *ms_out = ms;
  O3G_CUDA_TRY(cudaGetLastError());
  return O3G_OK;
}

namespace o3g {
__global__ void k_exp_probe(int n, const float* __restrict__ x, float* __restrict__ y) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = exp_tang(x[i]);
}
}  // namespace o3g

extern "C" int32_t o3g_exp_probe(int32_t n, const float* x, float* y, void* stream) {
  using namespace o3g;
  if (n < 0 || (n > 0 && (!x || !y))) {
    set_error("o3g_exp_probe: n must be >= 0 and x, y non-null");
    return O3G_ERR_INVALID_ARG;
  }
  if (n == 0) return O3G_OK;
  DeviceFacts df;
  O3G_TRY(device_facts(&df));
  k_exp_probe<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(n, x, y);
  note_launch();
  O3G_CUDA_TRY(cudaGetLastError());
  return O3G_OK;
}

namespace o3g {
// div3_rn against IEEE division by 3 for the float bit patterns first .. first + count - 1
// (a grid-stride sweep; every mismatch counted)
__global__ void k_div3_check(unsigned long long first, unsigned long long count, unsigned long long* mismatches) {
  unsigned long long bad = 0;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long k = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += stride) {
    const float x = __uint_as_float((unsigned)(first + k));
    if (!isfinite(x)) continue;
    if (__float_as_uint(div3_rn(x)) != __float_as_uint(__fdiv_rn(x, 3.0f))) ++bad;
  }
  if (bad) atomicAdd(mismatches, bad);
}
}  // namespace o3g

extern "C" int32_t o3g_div3_check(uint64_t first, uint64_t count, uint64_t* mismatches, void* stream) {
  using namespace o3g;
  if (!mismatches || first > (1ull << 32) || count > (1ull << 32) - first) {
    set_error("o3g_div3_check: the range must lie within the 2^32 float bit patterns; mismatches non-null");
    return O3G_ERR_INVALID_ARG;
  }
  DeviceFacts df;
  O3G_TRY(device_facts(&df));
  cudaStream_t st = (cudaStream_t)stream;
  Workspace* ws = nullptr;
  O3G_TRY(workspace_get(st, 256, &ws));
  unsigned long long* d = reinterpret_cast<unsigned long long*>(ws->base);
  O3G_CUDA_TRY(cudaMemsetAsync(d, 0, sizeof(unsigned long long), st));
  if (count > 0) {
    k_div3_check<<<8 * df.num_sms, 256, 0, st>>>(first, count, d);
    note_launch();
  }
  unsigned long long h = 0;
  O3G_CUDA_TRY(cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, st));
  O3G_CUDA_TRY(cudaStreamSynchronize(st));
  *mismatches = h;
  return O3G_OK;
}
