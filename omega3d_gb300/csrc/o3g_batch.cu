// o3g_batch.cu -- host side of the batched persistent pair sums: packing of many systems
// into one source and one target set (Morton-ordered per system for the cores with
// distance branches), the work-item plan, the autotuner with its per-shape cache, and
// the C-ABI o3g_batch_*.
//
// Plan.  With TB = 128 * TPT targets per block, system i has ceil((np_i + nf_i) / TB)
// target blocks and ceil(np_i / 128) source tiles.  A target block's tiles are cut into
// nsplit contiguous ranges of at most `chunk` tiles, where
//   chunk = max(8, ceil(total block-tiles / (grid * split)))
// so that the largest item is about 1/split of one resident block's share of the work;
// split = 0 never cuts.  Items run longest first.
//
// Autotuner.  Per shape -- (core, precision, grads, SM count, the list of (np, nf)) -- it
// times the persistent kernel for TPT in {1, 2, 4} x split in {0, 4, 16} at full occupancy
// and then the best at half occupancy, on the caller's data with the results redirected
// to scratch, and keeps the fastest.  Choices are cached in the process and in a text file
// ($O3G_TUNE_CACHE, else $XDG_CACHE_HOME/o3dgpu/batch_tune.txt or ~/.cache/o3dgpu/...;
// O3G_TUNE_CACHE set to an empty string keeps the cache in the process only).
// O3G_BATCH_TUNE=0 turns tuning off (cached or default configuration).
#include "o3g_batch.cuh"
#include "o3g_sort.cuh"

#include <cub/device/device_radix_sort.cuh>

#include <sys/stat.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

namespace o3g {

struct BatchCfg {
  int tpt = 0;
  int bps = 0;     // resident blocks per SM in the grid
  int split = 0;   // items per resident block that the longest item may not exceed (0 = never split)
};

struct BatchPlan {
  BatchCfg cfg;
  int grid = 0;
  int chunk = 0;
  int nt_pad = 0;
  long long nslabs = 0;
  std::vector<int> toff;    // nsys + 1
  std::vector<int4> items, tbs;
};

}  // namespace o3g

using namespace o3g;

struct o3g_batch {
  int core = 0, mode = 0;
  bool grads = true;
  int nsys = 0, nbind = 0;
  std::vector<int> np, nf, cp, ct, soff;
  long long totp = 0, tott = 0;
  int ntiles = 0, ns_pad = 0;
  int sms = 0;
  std::string key;
  BatchPlan plan;
  bool tuned = false;
  // device
  char* arena = nullptr;
  BatchSysDev* dsys = nullptr;      // [nbind][nsys]
  int *d_cp = nullptr, *d_ct = nullptr, *d_soff = nullptr, *d_toff = nullptr;
  V4<float>* spos = nullptr;
  V4<float>* sstr = nullptr;
  V4<float>* tpos = nullptr;
  int* tmap = nullptr;
  int4* items = nullptr;
  int4* tbs = nullptr;
  float* partial = nullptr;
  int* arrivals = nullptr;
  int* head = nullptr;
  float4* tile_lo = nullptr;
  float4* tile_hi = nullptr;
  float* bbox = nullptr;
  unsigned long long *kin = nullptr, *kout = nullptr;
  uint32_t *vin = nullptr, *sperm = nullptr, *tperm = nullptr;
  void* cub_tmp = nullptr;
  size_t cub_bytes = 0;
  float* sink = nullptr;
  // capacities of the plan-dependent buffers
  long long cap_tpad = 0, cap_items = 0, cap_tbs = 0, cap_slab_floats = 0;
};

namespace o3g {
namespace {

bool sorted_core(int core) { return core == CORE_GAUSS || core == CORE_EXP; }

std::vector<int> tpt_choices(int mode, bool grads) {
  if (mode == MODE_COMP && grads) return {1, 2};
  return {1, 2, 4};
}
BatchCfg default_cfg(int mode, bool grads) {
  BatchCfg c;
  c.tpt = (mode == MODE_PLAIN) ? (grads ? 2 : 4) : (grads ? 1 : 2);
  c.split = 4;
  return c;
}

const void* kernel_for(int core, int mode, bool grads, int tpt) {
  switch (core) {
    case CORE_RM: return batch_kernel<CORE_RM>(mode, grads, tpt);
    case CORE_WL: return batch_kernel<CORE_WL>(mode, grads, tpt);
    case CORE_EXP: return batch_kernel<CORE_EXP>(mode, grads, tpt);
    case CORE_GAUSS: return batch_kernel<CORE_GAUSS>(mode, grads, tpt);
    default: return batch_kernel<CORE_V2>(mode, grads, tpt);
  }
}
int32_t launch_for(int core, int mode, bool grads, int tpt, int grid, const BatchArgs<float>& a, cudaStream_t st) {
  switch (core) {
    case CORE_RM: return batch_launch<CORE_RM>(mode, grads, tpt, grid, a, st);
    case CORE_WL: return batch_launch<CORE_WL>(mode, grads, tpt, grid, a, st);
    case CORE_EXP: return batch_launch<CORE_EXP>(mode, grads, tpt, grid, a, st);
    case CORE_GAUSS: return batch_launch<CORE_GAUSS>(mode, grads, tpt, grid, a, st);
    default: return batch_launch<CORE_V2>(mode, grads, tpt, grid, a, st);
  }
}

int32_t grid_for(const o3g_batch_t* h, const BatchCfg& c, int* grid) {
  int occ = 0;
  O3G_TRY(occupancy_blocks(kernel_for(h->core, h->mode, h->grads, c.tpt), kBlock, &occ));
  int bps = c.bps > 0 ? std::min(c.bps, occ) : occ;
  if (bps < 1) bps = 1;
  *grid = bps * h->sms;
  return O3G_OK;
}

// np, nf: per system counts; soff: first packed source slot of each system (nsys + 1)
void build_plan_sizes(int nsys, const int* np, const int* nf, const int* soff, const BatchCfg& c, int grid,
                      BatchPlan* p) {
  const int TB = kBlock * c.tpt;
  p->cfg = c;
  p->grid = grid;
  p->toff.assign(nsys + 1, 0);
  long long units = 0;
  std::vector<int> tbl(nsys, 0);
  for (int i = 0; i < nsys; ++i) {
    const int tiles = (np[i] + kBlock - 1) / kBlock;
    tbl[i] = np[i] > 0 ? (np[i] + nf[i] + TB - 1) / TB : 0;
    p->toff[i + 1] = p->toff[i] + tbl[i] * TB;
    units += (long long)tbl[i] * tiles;
  }
  p->nt_pad = p->toff[nsys];
  long long chunk = 1LL << 30;
  if (c.split > 0) {
    const long long per = ((long long)grid * c.split);
    chunk = std::max(8LL, (units + per - 1) / per);
  }
  p->chunk = (int)std::min(chunk, (long long)(1 << 30));
  p->items.clear();
  p->tbs.clear();
  p->nslabs = 0;
  for (int i = 0; i < nsys; ++i) {
    const int tiles = (np[i] + kBlock - 1) / kBlock;
    const int t0 = soff[i] / kBlock;
    for (int b = 0; b < tbl[i]; ++b) {
      int ns = (int)((tiles + chunk - 1) / chunk);
      const int per = (tiles + ns - 1) / ns;
      ns = (tiles + per - 1) / per;
      const int tbi = (int)p->tbs.size();
      p->tbs.push_back(make_int4(i, p->toff[i] + b * TB, ns > 1 ? (int)p->nslabs : -1, ns));
      if (ns > 1) p->nslabs += ns;
      for (int q = 0; q < ns; ++q)
        p->items.push_back(make_int4(tbi, t0 + q * per, std::min(t0 + (q + 1) * per, t0 + tiles), q));
    }
  }
  std::stable_sort(p->items.begin(), p->items.end(),
                   [](const int4& a, const int4& b) { return (a.z - a.y) > (b.z - b.y); });
}

void build_plan(const o3g_batch_t* h, const BatchCfg& c, int grid, BatchPlan* p) {
  build_plan_sizes(h->nsys, h->np.data(), h->nf.data(), h->soff.data(), c, grid, p);
}

long long slab_floats(const o3g_batch_t* h, const BatchPlan& p) {
  const int nc = h->grads ? 12 : 3;
  const int np_ = h->mode == MODE_COMP ? 2 * nc : nc;
  return p.nslabs * np_ * kBlock * p.cfg.tpt;
}

// ---- tuning cache ----------------------------------------------------------------------
std::mutex g_tune_mu;
std::map<std::string, BatchCfg> g_tune;
bool g_tune_loaded = false;

std::string tune_path() {
  const char* e = std::getenv("O3G_TUNE_CACHE");
  if (e) return std::string(e);
  std::string dir;
  const char* x = std::getenv("XDG_CACHE_HOME");
  if (x && *x) dir = x;
  else {
    const char* home = std::getenv("HOME");
    if (!home || !*home) return std::string();
    dir = std::string(home) + "/.cache";
  }
  return dir + "/o3dgpu/batch_tune.txt";
}

void tune_load_locked() {
  if (g_tune_loaded) return;
  g_tune_loaded = true;
  const std::string path = tune_path();
  if (path.empty()) return;
  FILE* f = std::fopen(path.c_str(), "r");
  if (!f) return;
  char key[512];
  int tpt, bps, split;
  while (std::fscanf(f, "%511s %d %d %d%*[^\n]", key, &tpt, &bps, &split) == 4) {
    BatchCfg c;
    c.tpt = tpt; c.bps = bps; c.split = split;
    g_tune[key] = c;
  }
  std::fclose(f);
}

bool tune_lookup(const std::string& key, BatchCfg* c) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  tune_load_locked();
  auto it = g_tune.find(key);
  if (it == g_tune.end()) return false;
  *c = it->second;
  return true;
}

void mkdirs_for(const std::string& path) {
  for (size_t i = 1; i < path.size(); ++i)
    if (path[i] == '/') mkdir(path.substr(0, i).c_str(), 0755);
}

void tune_store(const std::string& key, const BatchCfg& c, float ms) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  tune_load_locked();
  g_tune[key] = c;
  const std::string path = tune_path();
  if (path.empty()) return;
  mkdirs_for(path);
  FILE* f = std::fopen(path.c_str(), "a");
  if (!f) return;
  std::fprintf(f, "%s %d %d %d %.4f\n", key.c_str(), c.tpt, c.bps, c.split, ms);
  std::fclose(f);
}

bool tuning_enabled() {
  const char* e = std::getenv("O3G_BATCH_TUNE");
  return !(e && e[0] == '0');
}

std::string shape_key(const o3g_batch_t* h) {
  uint64_t hsh = 1469598103934665603ULL;
  auto mix = [&](uint64_t v) {
    for (int b = 0; b < 8; ++b) { hsh ^= (v >> (8 * b)) & 0xff; hsh *= 1099511628211ULL; }
  };
  for (int i = 0; i < h->nsys; ++i) { mix((uint64_t)h->np[i]); mix((uint64_t)h->nf[i]); }
  char buf[256];
  std::snprintf(buf, sizeof(buf), "b1:c%d:m%d:g%d:sm%d:n%d:p%lld:t%lld:%016llx", h->core, h->mode, h->grads ? 1 : 0,
                h->sms, h->nsys, h->totp, h->tott, (unsigned long long)hsh);
  return std::string(buf);
}

// ---- device kernels: ordering, packing, tile bounds -------------------------------------------
__device__ __forceinline__ int find_sys(const int* __restrict__ off, int nsys, int j) {
  int lo = 0, hi = nsys;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (off[mid] <= j) lo = mid;
    else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ float core_param_rt(int core, float r) {
  if (core == CORE_EXP) return core_param<CORE_EXP, float>(r);
  if (core == CORE_V2) return core_param<CORE_V2, float>(r);
  return core_param<CORE_RM, float>(r);
}

// per system: bounding box of its particles and field points
__global__ void k_sys_bbox(const BatchSysDev* __restrict__ S, float* bbox) {
  __shared__ float red[8][6];
  const BatchSysDev& s = S[blockIdx.x];
  float v[6] = {3.0e38f, 3.0e38f, 3.0e38f, 3.0e38f, 3.0e38f, 3.0e38f};   // min x,y,z, min -x,-y,-z
  for (int i = threadIdx.x; i < s.np + s.nf; i += blockDim.x) {
    float p[3];
    if (i < s.np) { p[0] = s.p[0][i]; p[1] = s.p[1][i]; p[2] = s.p[2][i]; }
    else { p[0] = s.f[0][i - s.np]; p[1] = s.f[1][i - s.np]; p[2] = s.f[2][i - s.np]; }
#pragma unroll
    for (int d = 0; d < 3; ++d) { v[d] = fminf(v[d], p[d]); v[3 + d] = fminf(v[3 + d], -p[d]); }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int d = 0; d < 6; ++d) v[d] = fminf(v[d], __shfl_xor_sync(0xffffffffu, v[d], o));
  if ((threadIdx.x & 31) == 0)
#pragma unroll
    for (int d = 0; d < 6; ++d) red[threadIdx.x >> 5][d] = v[d];
  __syncthreads();
  if (threadIdx.x < 6) {
    float m = red[0][threadIdx.x];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fminf(m, red[w][threadIdx.x]);
    bbox[blockIdx.x * 6 + threadIdx.x] = threadIdx.x < 3 ? m : -m;
  }
}

// (system << 30 | Morton code within the system's box, concatenated index) for the sources
// (targets == 0) or the targets (particles then field points) of every system
__global__ void k_sys_keys(int n, int nsys, const int* __restrict__ off, const BatchSysDev* __restrict__ S,
                           const float* __restrict__ bbox, int targets, unsigned long long* key, uint32_t* val) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const int i = find_sys(off, nsys, j);
  const BatchSysDev& s = S[i];
  const int q = j - off[i];
  float p[3];
  if (!targets || q < s.np) { p[0] = s.p[0][q]; p[1] = s.p[1][q]; p[2] = s.p[2][q]; }
  else { p[0] = s.f[0][q - s.np]; p[1] = s.f[1][q - s.np]; p[2] = s.f[2][q - s.np]; }
  uint32_t c[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float lo = bbox[i * 6 + d], ext = bbox[i * 6 + 3 + d] - lo;
    float t = ext > 0.f ? (p[d] - lo) / ext : 0.f;
    t = fminf(fmaxf(t, 0.f), 1.f);
    c[d] = (uint32_t)(t * 1023.0f);
  }
  key[j] = ((unsigned long long)i << 30) | (spread3(c[0]) | (spread3(c[1]) << 1) | (spread3(c[2]) << 2));
  val[j] = (uint32_t)j;
}

__global__ void k_bpack_src(int total, int nsys, const int* __restrict__ soff, const BatchSysDev* __restrict__ S,
                            const uint32_t* __restrict__ sperm, int core, V4<float>* spos, V4<float>* sstr) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= total) return;
  const int i = find_sys(soff, nsys, j);
  const BatchSysDev& s = S[i];
  const int q = j - soff[i];
  V4<float> p, w;
  if (q < s.np) {
    const int g = sperm ? (int)sperm[s.cp + q] - s.cp : q;
    const float r = s.p[3][g];
    p.x = s.p[0][g]; p.y = s.p[1][g]; p.z = s.p[2][g]; p.w = core_param_rt(core, r);
    w.x = s.p[4][g]; w.y = s.p[5][g]; w.z = s.p[6][g]; w.w = r;
  } else {
    p.x = 1e9f; p.y = 1e9f; p.z = 1e9f; p.w = 1.f;   // zero strength, finite cores: adds exactly 0
    w.x = 0.f; w.y = 0.f; w.z = 0.f; w.w = 0.f;
  }
  spos[j] = p;
  sstr[j] = w;
}

__global__ void k_bpack_tgt(int total, int nsys, const int* __restrict__ toff, const BatchSysDev* __restrict__ S,
                            const uint32_t* __restrict__ tperm, int core, V4<float>* tpos, int* tmap) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= total) return;
  const int i = find_sys(toff, nsys, j);
  const BatchSysDev& s = S[i];
  const int q = j - toff[i];
  V4<float> p;
  int g = -1;
  if (q < s.np + s.nf) {
    g = tperm ? (int)tperm[s.ct + q] - s.ct : q;
    if (g < s.np) {
      p.x = s.p[0][g]; p.y = s.p[1][g]; p.z = s.p[2][g]; p.w = core_param_rt(core, s.p[3][g]);
    } else {
      const int k = g - s.np;
      p.x = s.f[0][k]; p.y = s.f[1][k]; p.z = s.f[2][k]; p.w = 0.f;
    }
  } else {
    p.x = 0.f; p.y = 0.f; p.z = 0.f; p.w = 0.f;
  }
  tpos[j] = p;
  tmap[j] = g;
}

// per half tile: bounds of its real sources (as k_tile_bounds, tiles of many systems)
__global__ void __launch_bounds__(kBlock) k_btile_bounds(int nsys, const int* __restrict__ soff,
                                                         const BatchSysDev* __restrict__ S,
                                                         const V4<float>* __restrict__ spos, float4* tlo,
                                                         float4* thi) {
  __shared__ float red[kBlock / 32][7];
  const int tile = blockIdx.x;
  const int j0 = tile * kBlock;
  const int i = find_sys(soff, nsys, j0);
  const int nreal = min(kBlock, S[i].np - (j0 - soff[i]));
  float v[7];
  if ((int)threadIdx.x < nreal) {
    const V4<float> p = spos[j0 + threadIdx.x];
    v[0] = p.x; v[1] = p.y; v[2] = p.z;
    v[3] = -p.x; v[4] = -p.y; v[5] = -p.z;
    v[6] = -p.w;
  } else {
#pragma unroll
    for (int d = 0; d < 7; ++d) v[d] = 3.0e38f;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int d = 0; d < 7; ++d) v[d] = fminf(v[d], __shfl_xor_sync(0xffffffffu, v[d], o));
  if ((threadIdx.x & 31) == 0)
#pragma unroll
    for (int d = 0; d < 7; ++d) red[threadIdx.x >> 5][d] = v[d];
  __syncthreads();
  // one box per half tile (kHalf sources, reduced from its two warps); a half without real
  // sources gets an empty box, which every far-field test accepts
  if (threadIdx.x < kBlock / kHalf) {
    const int hf = threadIdx.x;
    constexpr int W = kHalf / 32;
    float m[7];
    for (int d = 0; d < 7; ++d) {
      m[d] = red[hf * W][d];
      for (int wq = 1; wq < W; ++wq) m[d] = fminf(m[d], red[hf * W + wq][d]);
    }
    const float pad = 1e-6f * (fabsf(m[0]) + fabsf(m[1]) + fabsf(m[2]) + fabsf(m[3]) + fabsf(m[4]) + fabsf(m[5]));
    const int u = tile * (kBlock / kHalf) + hf;
    tlo[u] = make_float4(m[0] - pad, m[1] - pad, m[2] - pad, -m[6] * 1.000001f);
    thi[u] = make_float4(-m[3] + pad, -m[4] + pad, -m[5] + pad, 0.f);
  }
}

size_t cub_sort_bytes(long long n) {
  size_t b = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, b, (const unsigned long long*)nullptr, (unsigned long long*)nullptr,
                                  (const uint32_t*)nullptr, (uint32_t*)nullptr, (int)n, 0, 64);
  return b;
}

int bits_for(int n) {
  int b = 0;
  while ((1LL << b) < n) ++b;
  return b;
}

int32_t upload_plan(o3g_batch_t* h, const BatchPlan& p) {
  if ((long long)p.items.size() > h->cap_items || (long long)p.tbs.size() > h->cap_tbs || p.nt_pad > h->cap_tpad ||
      slab_floats(h, p) > h->cap_slab_floats) {
    set_error("batched pair sums: plan exceeds the allocated capacity");
    return O3G_ERR_STATE;
  }
  if (!p.items.empty())
    O3G_CUDA_TRY(cudaMemcpy(h->items, p.items.data(), p.items.size() * sizeof(int4), cudaMemcpyHostToDevice));
  if (!p.tbs.empty())
    O3G_CUDA_TRY(cudaMemcpy(h->tbs, p.tbs.data(), p.tbs.size() * sizeof(int4), cudaMemcpyHostToDevice));
  O3G_CUDA_TRY(cudaMemcpy(h->d_toff, p.toff.data(), p.toff.size() * sizeof(int), cudaMemcpyHostToDevice));
  return O3G_OK;
}

int32_t set_plan(o3g_batch_t* h, const BatchCfg& c) {
  BatchPlan p;
  int grid = 0;
  O3G_TRY(grid_for(h, c, &grid));
  build_plan(h, c, grid, &p);
  O3G_TRY(upload_plan(h, p));
  h->plan = std::move(p);
  return O3G_OK;
}

// sort (when the core classifies tiles), pack sources, tile bounds: independent of the plan
int32_t prep_sources(o3g_batch_t* h, int bind, cudaStream_t st) {
  const BatchSysDev* S = h->dsys + (size_t)bind * h->nsys;
  const uint32_t* sperm = nullptr;
  if (sorted_core(h->core)) {
    const int eb = 30 + bits_for(h->nsys);
    k_sys_bbox<<<h->nsys, 256, 0, st>>>(S, h->bbox);
    note_launch();
    if (h->totp > 0) {
      k_sys_keys<<<(int)((h->totp + 255) / 256), 256, 0, st>>>((int)h->totp, h->nsys, h->d_cp, S, h->bbox, 0, h->kin,
                                                               h->vin);
      note_launch();
      size_t tb = h->cub_bytes;
      O3G_CUDA_TRY(cub::DeviceRadixSort::SortPairs(h->cub_tmp, tb, h->kin, h->kout, h->vin, h->sperm, (int)h->totp, 0,
                                                   eb, st));
    }
    if (h->tott > 0) {
      k_sys_keys<<<(int)((h->tott + 255) / 256), 256, 0, st>>>((int)h->tott, h->nsys, h->d_ct, S, h->bbox, 1,
                                                               h->kin, h->vin);
      note_launch();
      size_t tb = h->cub_bytes;
      O3G_CUDA_TRY(cub::DeviceRadixSort::SortPairs(h->cub_tmp, tb, h->kin, h->kout, h->vin, h->tperm, (int)h->tott,
                                                   0, eb, st));
    }
    sperm = h->sperm;
  }
  if (h->ns_pad > 0) {
    k_bpack_src<<<(h->ns_pad + 255) / 256, 256, 0, st>>>(h->ns_pad, h->nsys, h->d_soff, S, sperm, h->core, h->spos,
                                                         h->sstr);
    note_launch();
    if (sorted_core(h->core)) {
      k_btile_bounds<<<h->ntiles, kBlock, 0, st>>>(h->nsys, h->d_soff, S, h->spos, h->tile_lo, h->tile_hi);
      note_launch();
    }
  }
  O3G_CUDA_TRY(cudaGetLastError());
  return O3G_OK;
}

int32_t prep_targets(o3g_batch_t* h, int bind, const BatchPlan& p, cudaStream_t st) {
  if (p.nt_pad == 0) return O3G_OK;
  const BatchSysDev* S = h->dsys + (size_t)bind * h->nsys;
  k_bpack_tgt<<<(p.nt_pad + 255) / 256, 256, 0, st>>>(p.nt_pad, h->nsys, h->d_toff, S,
                                                      sorted_core(h->core) ? h->tperm : nullptr, h->core, h->tpos,
                                                      h->tmap);
  note_launch();
  O3G_CUDA_TRY(cudaGetLastError());
  return O3G_OK;
}

int32_t sweep(o3g_batch_t* h, int bind, const BatchPlan& p, float* sink, cudaStream_t st) {
  if (p.items.empty()) return O3G_OK;
  BatchArgs<float> a;
  a.spos = h->spos; a.sstr = h->sstr; a.tpos = h->tpos; a.tmap = h->tmap;
  a.items = h->items; a.nitems = (int)p.items.size(); a.tbs = h->tbs;
  a.sys = h->dsys + (size_t)bind * h->nsys;
  a.tile_lo = h->tile_lo; a.tile_hi = h->tile_hi;
  a.partial = h->partial; a.arrivals = h->arrivals; a.head = h->head;
  a.sink = sink; a.sink_ld = h->cap_tpad;
  O3G_CUDA_TRY(cudaMemsetAsync(h->head, 0, sizeof(int), st));
  KernelTimer& tm = thread_timer();
  tm.begin(st);
  O3G_TRY(launch_for(h->core, h->mode, h->grads, p.cfg.tpt, p.grid, a, st));
  tm.end(st);
  return O3G_OK;
}

bool stream_capturing(cudaStream_t st) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) { (void)cudaGetLastError(); return true; }
  return cs != cudaStreamCaptureStatusNone;
}

}  // namespace

int32_t batch_tune(o3g_batch_t* h, cudaStream_t st, bool force) {
  if (h->tuned && !force) return O3G_OK;
  if (stream_capturing(st)) {
    set_error("o3g_batch_tune: the stream is capturing a graph");
    return O3G_ERR_STATE;
  }
  O3G_CUDA_TRY(cudaStreamSynchronize(st));
  cudaEvent_t e0, e1;
  O3G_CUDA_TRY(cudaEventCreate(&e0));
  O3G_CUDA_TRY(cudaEventCreate(&e1));
  int32_t rc = O3G_OK;
  BatchCfg best = h->plan.cfg;
  float best_ms = 3.0e38f;
  auto trial = [&](const BatchCfg& c, float* ms) -> int32_t {
    BatchPlan p;
    int grid = 0;
    O3G_TRY(grid_for(h, c, &grid));
    build_plan(h, c, grid, &p);
    O3G_TRY(upload_plan(h, p));
    O3G_TRY(prep_targets(h, 0, p, st));
    O3G_CUDA_TRY(cudaEventRecord(e0, st));
    O3G_TRY(sweep(h, 0, p, h->sink, st));
    O3G_CUDA_TRY(cudaEventRecord(e1, st));
    O3G_CUDA_TRY(cudaEventSynchronize(e1));
    O3G_CUDA_TRY(cudaEventElapsedTime(ms, e0, e1));
    return O3G_OK;
  };
  do {
    rc = prep_sources(h, 0, st);
    if (rc != O3G_OK) break;
    // warm-up with the current configuration (first launches carry one-time costs)
    float ms = 0.f;
    rc = trial(h->plan.cfg, &ms);
    if (rc != O3G_OK) break;
    for (int tpt : tpt_choices(h->mode, h->grads)) {
      for (int split : {0, 4, 16}) {
        BatchCfg c;
        c.tpt = tpt; c.split = split; c.bps = 0;
        rc = trial(c, &ms);
        if (rc != O3G_OK) break;
        if (ms < best_ms) { best_ms = ms; best = c; }
      }
      if (rc != O3G_OK) break;
    }
    if (rc != O3G_OK) break;
    int occ = 0;
    rc = occupancy_blocks(kernel_for(h->core, h->mode, h->grads, best.tpt), kBlock, &occ);
    if (rc != O3G_OK) break;
    best.bps = occ;
    if (occ >= 2) {
      BatchCfg c = best;
      c.bps = occ / 2;
      rc = trial(c, &ms);
      if (rc != O3G_OK) break;
      if (ms < best_ms) { best_ms = ms; best = c; }
    }
  } while (false);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != O3G_OK) return rc;
  O3G_TRY(set_plan(h, best));
  h->tuned = true;
  tune_store(h->key, best, best_ms);
  return O3G_OK;
}

int32_t batch_run(o3g_batch_t* h, int bind, cudaStream_t st) {
  if (!h || bind < 0 || bind >= h->nbind) {
    set_error("batched pair sums: bad handle or binding");
    return O3G_ERR_INVALID_ARG;
  }
  if (!h->tuned && tuning_enabled() && !stream_capturing(st)) O3G_TRY(batch_tune(h, st, false));
  O3G_TRY(prep_sources(h, bind, st));
  O3G_TRY(prep_targets(h, bind, h->plan, st));
  return sweep(h, bind, h->plan, nullptr, st);
}

int32_t batch_create(int core, int prec, bool grads, int nsys, const BatchSysDev* const* binds, int nbind,
                     o3g_batch_t** out) {
  if (!out || core < 0 || core > 4 || nsys < 1 || nbind < 1 || !binds ||
      (prec != O3G_PREC_PLAIN && prec != O3G_PREC_COMPENSATED)) {
    set_error("batched pair sums: bad arguments (core 0..4, precision PLAIN or COMPENSATED, nsys >= 1)");
    return O3G_ERR_INVALID_ARG;
  }
  DeviceFacts df;
  O3G_TRY(device_facts(&df));
  o3g_batch_t* h = new o3g_batch_t();
  h->core = core;
  h->mode = prec == O3G_PREC_COMPENSATED ? MODE_COMP : MODE_PLAIN;
  h->grads = grads;
  h->nsys = nsys;
  h->nbind = nbind;
  h->sms = df.num_sms;
  h->np.resize(nsys);
  h->nf.resize(nsys);
  h->cp.assign(nsys + 1, 0);
  h->ct.assign(nsys + 1, 0);
  h->soff.assign(nsys + 1, 0);
  const BatchSysDev* b0 = binds[0];
  long long soff = 0;
  for (int i = 0; i < nsys; ++i) {
    h->np[i] = b0[i].np;
    h->nf[i] = b0[i].nf;
    h->cp[i + 1] = h->cp[i] + b0[i].np;
    h->ct[i + 1] = h->ct[i] + b0[i].np + b0[i].nf;
    soff += (long long)((b0[i].np + kBlock - 1) / kBlock) * kBlock;
    h->soff[i + 1] = (int)std::min(soff, (long long)INT32_MAX);
  }
  h->totp = h->cp[nsys];
  h->tott = h->ct[nsys];
  h->ns_pad = h->soff[nsys];
  h->ntiles = h->ns_pad / kBlock;
  // every padded count must fit an int
  if (soff + 16 * kBlock * (long long)nsys >= (1LL << 30) ||
      h->tott + 4LL * kBlock * nsys >= (1LL << 30)) {
    delete h;
    set_error("batched pair sums: too many particles and field points (limit ~1e9 in total)");
    return O3G_ERR_INVALID_ARG;
  }
  h->key = shape_key(h);

  // candidate plans bound the plan-dependent buffers
  std::vector<BatchCfg> cands;
  for (int tpt : tpt_choices(h->mode, h->grads))
    for (int split : {0, 4, 16}) {
      BatchCfg c;
      c.tpt = tpt; c.split = split;
      cands.push_back(c);
    }
  BatchCfg chosen = default_cfg(h->mode, h->grads);
  h->tuned = tune_lookup(h->key, &chosen);
  bool chosen_listed = false;
  for (const BatchCfg& c : cands) chosen_listed |= (c.tpt == chosen.tpt && c.split == chosen.split);
  if (!chosen_listed) cands.push_back(chosen);
  for (const BatchCfg& c0 : cands) {
    BatchCfg c = c0;
    int occ = 0;
    int32_t rc = occupancy_blocks(kernel_for(core, h->mode, grads, c.tpt), kBlock, &occ);
    if (rc != O3G_OK) { delete h; return rc; }
    // half occupancy gives the most slabs (smaller chunks)
    for (int bps : {occ, std::max(1, occ / 2), std::max(1, c.bps)}) {
      BatchPlan p;
      build_plan(h, c, bps * h->sms, &p);
      h->cap_items = std::max(h->cap_items, (long long)p.items.size());
      h->cap_tbs = std::max(h->cap_tbs, (long long)p.tbs.size());
      h->cap_tpad = std::max(h->cap_tpad, (long long)p.nt_pad);
      h->cap_slab_floats = std::max(h->cap_slab_floats, slab_floats(h, p));
    }
  }
  const long long nkeys = std::max(h->totp, h->tott);
  const bool sorted = sorted_core(core);
  h->cub_bytes = sorted ? cub_sort_bytes(std::max(nkeys, 1LL)) : 0;
  size_t bytes = 0;
  auto add = [&](size_t b) { bytes += align_up(b); };
  add((size_t)nbind * nsys * sizeof(BatchSysDev));
  add(4 * (size_t)(nsys + 1) * sizeof(int));
  add((size_t)std::max(h->ns_pad, 1) * sizeof(V4<float>) * 2);
  add((size_t)std::max(h->cap_tpad, 1LL) * (sizeof(V4<float>) + sizeof(int)));
  add((size_t)std::max(h->cap_items, 1LL) * sizeof(int4));
  add((size_t)std::max(h->cap_tbs, 1LL) * (sizeof(int4) + sizeof(int)));
  add((size_t)std::max(h->cap_slab_floats, 1LL) * sizeof(float));
  add(sizeof(int));
  add((size_t)std::max(h->ntiles, 1) * sizeof(float4) * 4);
  add((size_t)nsys * 6 * sizeof(float));
  if (sorted) {
    add((size_t)nkeys * sizeof(unsigned long long) * 2);
    add((size_t)nkeys * sizeof(uint32_t));
    add((size_t)std::max(h->totp, 1LL) * sizeof(uint32_t));
    add((size_t)std::max(h->tott, 1LL) * sizeof(uint32_t));
    add(h->cub_bytes);
  }
  add((size_t)12 * std::max(h->cap_tpad, 1LL) * sizeof(float));   // tuning sink
  cudaError_t e = o3g::dev_alloc((void**)&h->arena, bytes);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    set_error_cuda("batched pair sums: cudaMalloc", e);
    delete h;
    return O3G_ERR_ALLOC;
  }
  Carve cv(h->arena);
  h->dsys = cv.take<BatchSysDev>((size_t)nbind * nsys);
  h->d_cp = cv.take<int>(4 * (size_t)(nsys + 1));
  h->d_ct = h->d_cp + (nsys + 1);
  h->d_soff = h->d_ct + (nsys + 1);
  h->d_toff = h->d_soff + (nsys + 1);
  h->spos = cv.take<V4<float>>((size_t)std::max(h->ns_pad, 1) * 2);
  h->sstr = h->spos + std::max(h->ns_pad, 1);
  {
    char* tp = cv.take<char>((size_t)std::max(h->cap_tpad, 1LL) * (sizeof(V4<float>) + sizeof(int)));
    h->tpos = (V4<float>*)tp;
    h->tmap = (int*)(tp + (size_t)std::max(h->cap_tpad, 1LL) * sizeof(V4<float>));
  }
  h->items = cv.take<int4>((size_t)std::max(h->cap_items, 1LL));
  {
    char* tp = cv.take<char>((size_t)std::max(h->cap_tbs, 1LL) * (sizeof(int4) + sizeof(int)));
    h->tbs = (int4*)tp;
    h->arrivals = (int*)(tp + (size_t)std::max(h->cap_tbs, 1LL) * sizeof(int4));
  }
  h->partial = cv.take<float>((size_t)std::max(h->cap_slab_floats, 1LL));
  h->head = cv.take<int>(1);
  h->tile_lo = cv.take<float4>((size_t)std::max(h->ntiles, 1) * 4);     // two halves per tile
  h->tile_hi = h->tile_lo + 2 * (size_t)std::max(h->ntiles, 1);
  h->bbox = cv.take<float>((size_t)nsys * 6);
  if (sorted) {
    h->kin = cv.take<unsigned long long>((size_t)nkeys * 2);
    h->kout = h->kin + nkeys;
    h->vin = cv.take<uint32_t>((size_t)nkeys);
    h->sperm = cv.take<uint32_t>((size_t)std::max(h->totp, 1LL));
    h->tperm = cv.take<uint32_t>((size_t)std::max(h->tott, 1LL));
    h->cub_tmp = cv.take<char>(h->cub_bytes);
  }
  h->sink = cv.take<float>((size_t)12 * std::max(h->cap_tpad, 1LL));

  std::vector<BatchSysDev> tab((size_t)nbind * nsys);
  for (int b = 0; b < nbind; ++b)
    for (int i = 0; i < nsys; ++i) {
      BatchSysDev d = binds[b][i];
      d.np = h->np[i];
      d.nf = h->nf[i];
      d.cp = h->cp[i];
      d.ct = h->ct[i];
      d.soff = h->soff[i];
      d.pad_ = 0;
      tab[(size_t)b * nsys + i] = d;
    }
  int32_t rc = O3G_OK;
  do {
    e = cudaMemcpy(h->dsys, tab.data(), tab.size() * sizeof(BatchSysDev), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(h->d_cp, h->cp.data(), (nsys + 1) * sizeof(int), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(h->d_ct, h->ct.data(), (nsys + 1) * sizeof(int), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(h->d_soff, h->soff.data(), (nsys + 1) * sizeof(int), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(h->arrivals, 0, (size_t)std::max(h->cap_tbs, 1LL) * sizeof(int));
    if (e != cudaSuccess) {
      set_error_cuda("batched pair sums: table upload", e);
      rc = O3G_ERR_CUDA;
      break;
    }
    rc = set_plan(h, chosen);
  } while (false);
  if (rc != O3G_OK) {
    cudaFree(h->arena);
    delete h;
    return rc;
  }
  *out = h;
  return O3G_OK;
}

}  // namespace o3g

// ---- C-ABI -------------------------------------------------------------------------------
namespace {

int32_t systems_to_desc(int32_t nsys, const o3g_system_t* sys, int32_t grads, std::vector<BatchSysDev>* out) {
  if (nsys < 1 || !sys) {
    set_error("o3g_batch: nsys >= 1 and a system array are required");
    return O3G_ERR_INVALID_ARG;
  }
  out->assign(nsys, BatchSysDev{});
  for (int i = 0; i < nsys; ++i) {
    const o3g_system_t& s = sys[i];
    bool ok = s.np >= 0 && s.nf >= 0;
    if (ok && s.np > 0) {
      ok = s.x && s.y && s.z && s.r && s.sx && s.sy && s.sz && s.u && s.v && s.w;
      if (grads) for (int d = 0; d < 9; ++d) ok = ok && s.ug[d];
    }
    if (ok && s.nf > 0) {
      ok = s.fx && s.fy && s.fz && s.fu && s.fv && s.fw;
      if (grads) for (int d = 0; d < 9; ++d) ok = ok && s.fug[d];
    }
    if (!ok) {
      char buf[160];
      std::snprintf(buf, sizeof(buf), "o3g_batch: system %d has a negative count or a missing array", i);
      set_error(buf);
      return O3G_ERR_INVALID_ARG;
    }
    BatchSysDev& d = (*out)[i];
    const float* p[7] = {s.x, s.y, s.z, s.r, s.sx, s.sy, s.sz};
    for (int k = 0; k < 7; ++k) d.p[k] = p[k];
    d.f[0] = s.fx; d.f[1] = s.fy; d.f[2] = s.fz;
    d.out[0] = s.u; d.out[1] = s.v; d.out[2] = s.w;
    d.fout[0] = s.fu; d.fout[1] = s.fv; d.fout[2] = s.fw;
    for (int k = 0; k < 9; ++k) {
      d.out[3 + k] = grads ? s.ug[k] : nullptr;
      d.fout[3 + k] = grads ? s.fug[k] : nullptr;
    }
    d.np = s.np;
    d.nf = s.nf;
  }
  return O3G_OK;
}

}  // namespace

extern "C" int32_t o3g_batch_create(int32_t core, int32_t prec, int32_t grads, int32_t nsys,
                                    const o3g_system_t* systems, o3g_batch_t** h) {
  if (!h) {
    set_error("o3g_batch_create: null handle pointer");
    return O3G_ERR_INVALID_ARG;
  }
  std::vector<BatchSysDev> desc;
  O3G_TRY(systems_to_desc(nsys, systems, grads, &desc));
  const BatchSysDev* b = desc.data();
  return batch_create(core, prec, grads != 0, nsys, &b, 1, h);
}

extern "C" int32_t o3g_batch_run(o3g_batch_t* h, void* stream) { return batch_run(h, 0, (cudaStream_t)stream); }

extern "C" int32_t o3g_batch_tune(o3g_batch_t* h, void* stream) {
  if (!h) return O3G_ERR_INVALID_ARG;
  return batch_tune(h, (cudaStream_t)stream, true);
}

extern "C" int32_t o3g_batch_set_config(o3g_batch_t* h, int32_t tpt, int32_t blocks_per_sm, int32_t split) {
  if (!h || blocks_per_sm < 0 || split < 0) return O3G_ERR_INVALID_ARG;
  bool ok = false;
  for (int t : tpt_choices(h->mode, h->grads)) ok |= (t == tpt);
  if (!ok || (split != 0 && split != 4 && split != 16)) {
    set_error("o3g_batch_set_config: tpt must be one of the compiled choices and split one of 0, 4, 16");
    return O3G_ERR_INVALID_ARG;
  }
  O3G_CUDA_TRY(cudaDeviceSynchronize());
  BatchCfg c;
  c.tpt = tpt; c.bps = blocks_per_sm; c.split = split;
  O3G_TRY(set_plan(h, c));
  h->tuned = true;
  return O3G_OK;
}

extern "C" int32_t o3g_batch_get_config(const o3g_batch_t* h, int32_t* tpt, int32_t* blocks, int32_t* split,
                                        int32_t* chunk, int32_t* nitems, int32_t* tuned) {
  if (!h) return O3G_ERR_INVALID_ARG;
  if (tpt) *tpt = h->plan.cfg.tpt;
  if (blocks) *blocks = h->plan.grid;
  if (split) *split = h->plan.cfg.split;
  if (chunk) *chunk = h->plan.chunk;
  if (nitems) *nitems = (int32_t)h->plan.items.size();
  if (tuned) *tuned = h->tuned ? 1 : 0;
  return O3G_OK;
}

extern "C" int32_t o3g_batch_destroy(o3g_batch_t* h) {
  if (!h) return O3G_OK;
  cudaDeviceSynchronize();
  cudaFree(h->arena);
  delete h;
  return O3G_OK;
}

extern "C" int32_t o3g_batch_velgrad(int32_t core, int32_t prec, int32_t grads, int32_t nsys,
                                     const o3g_system_t* systems, void* stream) {
  o3g_batch_t* h = nullptr;
  O3G_TRY(o3g_batch_create(core, prec, grads, nsys, systems, &h));
  int32_t rc = o3g_batch_run(h, stream);
  const cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
  if (rc == O3G_OK && e != cudaSuccess) {
    set_error_cuda("o3g_batch_velgrad: cudaStreamSynchronize", e);
    rc = O3G_ERR_CUDA;
  }
  o3g_batch_destroy(h);
  return rc;
}

// Host-only: the work-item plan for given counts (no device needed).  items / tbs receive
// 4 ints per entry when not null (call first with nulls for the counts).
extern "C" int32_t o3g_batch_plan(int32_t nsys, const int32_t* np, const int32_t* nf, int32_t tpt, int32_t grid,
                                  int32_t split, int32_t* nitems, int32_t* ntbs, int32_t* chunk, int64_t* nslabs,
                                  int32_t* items, int32_t* tbs) {
  if (nsys < 1 || !np || !nf || (tpt != 1 && tpt != 2 && tpt != 4) || grid < 1 || split < 0) {
    set_error("o3g_batch_plan: bad arguments");
    return O3G_ERR_INVALID_ARG;
  }
  std::vector<int> soff(nsys + 1, 0);
  long long acc = 0;
  for (int i = 0; i < nsys; ++i) {
    if (np[i] < 0 || nf[i] < 0) {
      set_error("o3g_batch_plan: negative count");
      return O3G_ERR_INVALID_ARG;
    }
    acc += (long long)((np[i] + kBlock - 1) / kBlock) * kBlock;
    if (acc >= (1LL << 30)) {
      set_error("o3g_batch_plan: too many particles");
      return O3G_ERR_INVALID_ARG;
    }
    soff[i + 1] = (int)acc;
  }
  BatchCfg c;
  c.tpt = tpt;
  c.split = split;
  BatchPlan p;
  build_plan_sizes(nsys, np, nf, soff.data(), c, grid, &p);
  if (nitems) *nitems = (int32_t)p.items.size();
  if (ntbs) *ntbs = (int32_t)p.tbs.size();
  if (chunk) *chunk = p.chunk;
  if (nslabs) *nslabs = p.nslabs;
  if (items) std::memcpy(items, p.items.data(), p.items.size() * sizeof(int4));
  if (tbs) std::memcpy(tbs, p.tbs.data(), p.tbs.size() * sizeof(int4));
  return O3G_OK;
}
