// o3g_runtime.cu -- errors, device facts, per-stream workspaces, kernel timing.
#include "o3g_common.cuh"

#include <atomic>

#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <utility>

namespace o3g {

static thread_local char g_last_error[512] = "";

void set_error(const char* what) {
  std::snprintf(g_last_error, sizeof(g_last_error), "%s", what);
}
void set_error_cuda(const char* where, cudaError_t e) {
  std::snprintf(g_last_error, sizeof(g_last_error), "%s: %s (%s)", where, cudaGetErrorString(e),
                cudaGetErrorName(e));
}

int32_t device_facts(DeviceFacts* f) {
  static std::mutex mu;
  static std::map<int, DeviceFacts> cache;
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_error_cuda("cudaGetDevice", e);
    return O3G_ERR_NO_DEVICE;
  }
  std::lock_guard<std::mutex> lk(mu);
  auto it = cache.find(dev);
  if (it == cache.end()) {
    DeviceFacts d;
    d.device = dev;
    O3G_CUDA_TRY(cudaDeviceGetAttribute(&d.num_sms, cudaDevAttrMultiProcessorCount, dev));
    O3G_CUDA_TRY(cudaDeviceGetAttribute(&d.cc_major, cudaDevAttrComputeCapabilityMajor, dev));
    O3G_CUDA_TRY(cudaDeviceGetAttribute(&d.cc_minor, cudaDevAttrComputeCapabilityMinor, dev));
    if (cudaDeviceGetAttribute(&d.clock_khz, cudaDevAttrClockRate, dev) != cudaSuccess) {
      (void)cudaGetLastError();
      d.clock_khz = 0;
    }
    if (d.cc_major != 10 || d.cc_minor != 3) {
      char msg[160];
      std::snprintf(msg, sizeof(msg), "device %d is sm_%d%d; this library is built for sm_103a only", dev,
                    d.cc_major, d.cc_minor);
      set_error(msg);
      return O3G_ERR_NO_DEVICE;
    }
    it = cache.emplace(dev, d).first;
  }
  *f = it->second;
  return O3G_OK;
}

int32_t workspace_get(cudaStream_t stream, size_t bytes, Workspace** out) {
  static std::mutex mu;
  static std::map<std::pair<int, cudaStream_t>, Workspace> spaces;
  int dev = -1;
  O3G_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  Workspace& w = spaces[std::make_pair(dev, stream)];
  if (w.cap < bytes) {
    if (w.base) {
      // earlier work on this stream may still read the old buffer
      O3G_CUDA_TRY(cudaStreamSynchronize(stream));
      O3G_CUDA_TRY(cudaFree(w.base));
      w.base = nullptr;
      w.cap = 0;
    }
    const size_t want = align_up(bytes + bytes / 4, 1 << 20);
    cudaError_t e = dev_alloc((void**)&w.base, want);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      e = dev_alloc((void**)&w.base, align_up(bytes, 1 << 20));
      if (e != cudaSuccess) {
        (void)cudaGetLastError();
        set_error_cuda("cudaMalloc(workspace)", e);
        w.base = nullptr;
        return O3G_ERR_ALLOC;
      }
      w.cap = align_up(bytes, 1 << 20);
    } else {
      w.cap = want;
    }
  }
  *out = &w;
  return O3G_OK;
}

int32_t occupancy_blocks(const void* kernel, int block, int* nb) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, int> cache;
  int dev = -1;
  O3G_CUDA_TRY(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  auto key = std::make_pair(kernel, dev * 4096 + block);
  auto it = cache.find(key);
  if (it == cache.end()) {
    int n = 0;
    O3G_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, block, 0));
    if (n < 1) n = 1;
    it = cache.emplace(key, n).first;
  }
  *nb = it->second;
  return O3G_OK;
}

static thread_local bool g_timing = false;
static thread_local unsigned long long g_launches = 0;
void note_launch(int n) { g_launches += (unsigned long long)n; }

static std::atomic<int> g_wait_test{0};
bool wait_test_on() { return g_wait_test.load() != 0; }

static std::atomic<unsigned long long> g_allocs{0};
cudaError_t dev_alloc(void** p, size_t bytes) {
  const cudaError_t e = cudaMalloc(p, bytes);
  if (e == cudaSuccess) g_allocs.fetch_add(1);
  return e;
}
cudaError_t dev_alloc_async(void** p, size_t bytes, cudaStream_t st) {
  const cudaError_t e = cudaMallocAsync(p, bytes, st);
  if (e == cudaSuccess) g_allocs.fetch_add(1);
  return e;
}
static thread_local KernelTimer g_timer;

KernelTimer& thread_timer() { return g_timer; }

void KernelTimer::begin(cudaStream_t s) {
  active = false;
  if (!g_timing) return;
  if (!start) { cudaEventCreate(&start); cudaEventCreate(&stop); }
  if (cudaEventRecord(start, s) == cudaSuccess) active = true;
}
void KernelTimer::end(cudaStream_t s) {
  if (!active) return;
  if (cudaEventRecord(stop, s) != cudaSuccess) active = false;
}

}  // namespace o3g

extern "C" {

const char* o3g_status_string(int32_t s) {
  switch (s) {
    case O3G_OK: return "ok";
    case O3G_ERR_INVALID_ARG: return "invalid argument";
    case O3G_ERR_CUDA: return "CUDA runtime error";
    case O3G_ERR_NO_DEVICE: return "no usable sm_103 device";
    case O3G_ERR_ALLOC: return "device allocation failed";
    case O3G_ERR_NOT_CONVERGED: return "iterative refinement did not converge";
    case O3G_ERR_TIMEOUT: return "device-side wait timed out";
    case O3G_ERR_SINGULAR: return "singular or non-finite pivot";
    case O3G_ERR_NONFINITE: return "non-finite input";
    case O3G_ERR_STATE: return "call made in the wrong state";
    case O3G_ERR_CAPACITY: return "output arrays too small";
    default: return "unknown status";
  }
}

const char* o3g_last_error(void) { return o3g::g_last_error; }

int32_t o3g_version(void) { return 100; }

int32_t o3g_device_info(int32_t* num_sms, int32_t* sm_clock_khz, int32_t* cc_major, int32_t* cc_minor) {
  o3g::DeviceFacts f;
  O3G_TRY(o3g::device_facts(&f));
  if (num_sms) *num_sms = f.num_sms;
  if (sm_clock_khz) *sm_clock_khz = f.clock_khz;
  if (cc_major) *cc_major = f.cc_major;
  if (cc_minor) *cc_minor = f.cc_minor;
  return O3G_OK;
}

int32_t o3g_flops_per_pair(int32_t core, int32_t grads, int32_t have_tr) {
  // CoreFunc.h flops_t{v,p}{_grads,_nograds} per core, in the order RM, WL, EXP, GAUSS, V2;
  // the Gaussian entries are this library's own tally of its closed-form branch.
  static const int tvg[5] = {9, 16, 14, 15, 13};
  static const int tpg[5] = {7, 14, 11, 13, 10};
  static const int tv[5] = {7, 10, 12, 11, 11};
  static const int tp[5] = {5, 8, 9, 9, 8};
  if (core < 0 || core > 4) return -1;
  if (grads) return 54 + (have_tr ? tvg[core] : tpg[core]);
  return 23 + (have_tr ? tv[core] : tp[core]);
}

int32_t o3g_debug_wait_test(int32_t enable) {
  o3g::g_wait_test.store(enable != 0 ? 1 : 0);
  return O3G_OK;
}

int32_t o3g_alloc_count(uint64_t* n) {
  if (!n) return O3G_ERR_INVALID_ARG;
  *n = (uint64_t)o3g::g_allocs.load();
  return O3G_OK;
}

int32_t o3g_launch_count(uint64_t* n) {
  if (!n) return O3G_ERR_INVALID_ARG;
  *n = (uint64_t)o3g::g_launches;
  return O3G_OK;
}

int32_t o3g_set_timing(int32_t enable) {
  o3g::g_timing = (enable != 0);
  return O3G_OK;
}

int32_t o3g_last_kernel_ms(float* ms) {
  o3g::KernelTimer& t = o3g::g_timer;
  if (!ms) return O3G_ERR_INVALID_ARG;
  if (!t.active) return O3G_ERR_STATE;
  O3G_CUDA_TRY(cudaEventSynchronize(t.stop));
  O3G_CUDA_TRY(cudaEventElapsedTime(ms, t.start, t.stop));
  return O3G_OK;
}

}  // extern "C"
