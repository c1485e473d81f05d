// o3g_splitmerge.cu -- particle split (split_elongated, Split.h:44-270) and merge
// (merge_close_particles, Merge.h:45-218) on the device, bit-identical to the reference's
// sequential loops (float S).
//
// Both operators search neighbours around each particle's position at the start of the
// operator; the reference searches a nanoflann kd-tree over a copy of them
// (Split.h:65-76, Merge.h:76-87).  Here the search runs on a uniform cell list:
//   * cell size = the largest search radius × (1 + 2^-10), so a match is never more than
//     one cell away per axis, even after float rounding of its distance;
//   * cells are keyed by their linear index (or, for grids of more than 16 cells per
//     particle, cx << 42 | cy << 21 | cz) and particles radix-sorted by key, so the 3 cells
//     along z of each (cx, cy) column are one contiguous range: 9 ranges per query, read
//     from a start table (count + exclusive scan) or, for the packed keys, found by binary
//     search; positions are gathered into key order for coalesced candidate reads;
//   * the match test is nanoflann's: d2 = ((q0-p0)^2 + (q1-p1)^2) + (q2-p2)^2 in float
//     (L2_Adaptor::evalMetric, query minus point), d2 < radius strictly
//     (RadiusResultSet::addPoint);
//   * each query's matches are written as (d2 bits << 32 | index) and put in that order,
//     the reference's visiting order (params.sorted): by a rank sort in shared memory for
//     the split (one warp per query, ~113 matches), by a CUB segmented sort for the merge
//     (under one match per query on average); equal d2 go in increasing index, where the
//     reference's order for such ties follows its kd-tree.
//
// Split.  Particle i's result reads, for every neighbour j < i that was itself split, j's
// state after its split (x moved by halfd * axis, strength halved and corrected), and for
// every other neighbour the state before the operator.  That is a dependency chain in
// index order (about 300 deep for 12,000 splits of 64,000 particles, 829 for 189,000 of
// 1,000,000).  A light kernel first gives every split particle its level in that graph
// (one thread per particle, waiting only for lower ranks); the particles are sorted by
// level; then one cooperative kernel walks the chain: warps claim particles in level order
// through an atomic counter and wait (bounded) only for the ready flags of their
// dependencies, which have lower levels, were claimed earlier by running warps, and so
// always progress.  Claiming in level order instead of index order keeps every resident
// warp on work whose dependencies are at most a level away.  Every term that reads no split state (neighbours not split,
// or split later in index order: about 90 %) is computed beforehand by the parallel fill
// kernel; the chain computes only the others, from the published states, and adds the four
// sums (curvature and dVol) in the sorted order, one lane per sum.
//
// Merge.  Particle i's processing reads and writes only i and its matches, so particles
// interact only within connected groups of the match graph.  Groups come from a lock-free
// union-find over the match edges (parent pointers always point to smaller indices, so
// every loop ends); then one thread per group replays the reference's loop over the
// group's particles in increasing index, in place.  The mean strength
// (Merge.h:100-104) is the reference's sequential float sum: one thread adds the terms in
// index order while the rest of its block stages them in shared memory, on a second stream
// so that it overlaps the neighbour search.  The survivors are compacted in order
// (Merge.h:181-204).
//
// Arithmetic follows the reference's expressions operation by operation, with the float /
// double promotions its C++ implies, using _rn intrinsics so nothing is contracted.
#include "o3g_common.cuh"

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_reduce.cuh>
#include <cub/device/device_scan.cuh>
#include <cub/device/device_segmented_sort.cuh>

#include <algorithm>
#include <climits>
#include <cmath>
#include <mutex>
#include <vector>

namespace o3g {
namespace {

constexpr int64_t kMaxCell = (1 << 21) - 1;
constexpr unsigned kFull = 0xffffffffu;
constexpr uint32_t kReadySpin = 1u << 28;
constexpr uint64_t kReadyNs = 10ull * 1000 * 1000 * 1000;   // 10 s
// the wait test's limits (o3g_debug_wait_test): the waits then read a word nothing sets
constexpr uint32_t kTestSpin = 1u << 14;
constexpr uint64_t kTestNs = 20ull * 1000 * 1000;   // 20 ms
// pause between polls of a flag: thousands of waiting threads polling back to back load
// the L2 enough to slow the stores they wait for
constexpr unsigned kPollNs = 128;

struct GridDev {
  double lo[3];
  double inv_h;
  int64_t cmax[3];   // largest cell coordinate per axis
  int dense;         // 1: keys are linear cell indices with a start table, 0: packed keys
};

struct CellList {
  const uint64_t* keys;   // sorted cell keys
  const int* order;       // particle index per sorted slot
  const float4* pos;      // positions in sorted order
  const int* cstart;      // dense grids: first sorted slot of every cell (one past the end last)
  int n;
};

__device__ __forceinline__ int ord(float f) {
  const int i = __float_as_int(f);
  return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float unord(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

__device__ __forceinline__ uint64_t cell_key(const GridDev& g, int64_t cx, int64_t cy, int64_t cz) {
  if (g.dense) return ((uint64_t)cx * (uint64_t)(g.cmax[1] + 1) + (uint64_t)cy) * (uint64_t)(g.cmax[2] + 1) +
                      (uint64_t)cz;
  return ((uint64_t)cx << 42) | ((uint64_t)cy << 21) | (uint64_t)cz;
}

__device__ __forceinline__ void cell_of(const GridDev& g, float px, float py, float pz, int64_t c[3]) {
  const double p[3] = {(double)px, (double)py, (double)pz};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    double u = floor((p[d] - g.lo[d]) * g.inv_h);
    if (!(u >= 0.0)) u = 0.0;
    if (u > (double)g.cmax[d]) u = (double)g.cmax[d];
    c[d] = (int64_t)u;
  }
}

__device__ __forceinline__ int lower_bound_u64(const uint64_t* a, int n, uint64_t v) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (a[mid] < v) lo = mid + 1; else hi = mid;
  }
  return lo;
}
__device__ __forceinline__ int upper_bound_u64(const uint64_t* a, int n, uint64_t v) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (a[mid] <= v) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// nanoflann L2_Adaptor::evalMetric for 3 dimensions (query minus point, float)
__device__ __forceinline__ float nf_dist2(float qx, float qy, float qz, float4 p) {
  const float d0 = __fsub_rn(qx, p.x), d1 = __fsub_rn(qy, p.y), d2 = __fsub_rn(qz, p.z);
  float r = __fmul_rn(d0, d0);
  r = __fadd_rn(r, __fmul_rn(d1, d1));
  r = __fadd_rn(r, __fmul_rn(d2, d2));
  return r;
}

__device__ __forceinline__ uint64_t match_key(float d2, int j) {
  return ((uint64_t)__float_as_uint(d2) << 32) | (uint32_t)j;
}

// every candidate slot t of the 27 cells around q, LANES lanes at a time; f(t, in) is
// called by all lanes in lockstep rounds (in = false past the end of a range)
template <int LANES, class F>
__device__ __forceinline__ void visit_cells(const CellList& cl, const GridDev& g, float qx, float qy, float qz,
                                            int lane, F&& f) {
  int64_t c[3];
  cell_of(g, qx, qy, qz, c);
  const int64_t z0 = c[2] > 0 ? c[2] - 1 : 0, z1 = c[2] < g.cmax[2] ? c[2] + 1 : g.cmax[2];
  const int64_t x0 = c[0] > 0 ? c[0] - 1 : 0, x1 = c[0] < g.cmax[0] ? c[0] + 1 : g.cmax[0];
  const int64_t y0 = c[1] > 0 ? c[1] - 1 : 0, y1 = c[1] < g.cmax[1] ? c[1] + 1 : g.cmax[1];
  for (int64_t cx = x0; cx <= x1; ++cx)
    for (int64_t cy = y0; cy <= y1; ++cy) {
      const uint64_t k0 = cell_key(g, cx, cy, z0), k1 = cell_key(g, cx, cy, z1);
      // the cells (cx, cy, z0..z1) are consecutive keys: one range of sorted slots
      const int b = g.dense ? cl.cstart[k0] : lower_bound_u64(cl.keys, cl.n, k0);
      const int e = g.dense ? cl.cstart[k1 + 1] : upper_bound_u64(cl.keys, cl.n, k1);
      for (int t0 = b; t0 < e; t0 += LANES) {
        const int t = t0 + lane;
        f(t, t < e);
      }
    }
}

// search radius squared of the split (Split.h:125-129) and merge (Merge.h:122-124) queries
__device__ __forceinline__ float split_radius(float r, float overlap) {
  const float nom_sep = __fdiv_rn(r, overlap);
  return __double2float_rn(__dmul_rn(3.0, (double)nom_sep));
}
__device__ __forceinline__ float merge_radius(float r, float overlap) {
  const float nom_sep = __fdiv_rn(r, overlap);
  return __fmul_rn(nom_sep, 0.5f);
}
__device__ __forceinline__ float radius_sq(float rad) {
  return __double2float_rn(__dmul_rn((double)rad, (double)rad));
}

__device__ __forceinline__ float sumsq3(float a, float b, float c) {
  return __fadd_rn(__fadd_rn(__fmul_rn(a, a), __fmul_rn(b, b)), __fmul_rn(c, c));
}

// ---------------------------------------------------------------------------------
// cell list

// bb: ordered-int minimum [0..2] and maximum [3..5] of the positions
__global__ void k_sm_init(int* bb, int* rmax_bits) {
  if (threadIdx.x < 3) bb[threadIdx.x] = 0x7fffffff;
  else if (threadIdx.x < 6) bb[threadIdx.x] = (int)0x80000000;
  if (threadIdx.x == 6) *rmax_bits = 0;
}

__global__ void k_bbox(int n, const float* __restrict__ x, const float* __restrict__ y, const float* __restrict__ z,
                       int* bb) {
  float lo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, hi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float v[3] = {x[i], y[i], z[i]};
#pragma unroll
    for (int d = 0; d < 3; ++d) { lo[d] = fminf(lo[d], v[d]); hi[d] = fmaxf(hi[d], v[d]); }
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    for (int o = 16; o > 0; o >>= 1) {
      lo[d] = fminf(lo[d], __shfl_xor_sync(kFull, lo[d], o));
      hi[d] = fmaxf(hi[d], __shfl_xor_sync(kFull, hi[d], o));
    }
    if ((threadIdx.x & 31) == 0) {
      atomicMin(&bb[d], ord(lo[d]));
      atomicMax(&bb[3 + d], ord(hi[d]));
    }
  }
}

// cell size and origin; a dense start table when the grid has at most `cap` cells
__global__ void k_grid(const int* bb, const int* rmax_bits, long long cap, GridDev* g) {
  const float rmax = __int_as_float(*rmax_bits);
  double h = 1.0;
  if (rmax > 0.0f && rmax <= 3.0e38f) h = (double)rmax * (1.0 + 1.0 / 1024.0);
  const double inv_h = 1.0 / h;
  double ncells = 1.0;
  for (int d = 0; d < 3; ++d) {
    const float lo = unord(bb[d]), hi = unord(bb[3 + d]);
    const bool fin = lo >= -3.0e38f && lo <= 3.0e38f && hi >= -3.0e38f && hi <= 3.0e38f && hi >= lo;
    g->lo[d] = fin ? (double)lo : 0.0;
    double u = fin ? floor(((double)hi - (double)lo) * inv_h) : (double)kMaxCell;
    if (!(u >= 0.0)) u = 0.0;
    if (u > (double)kMaxCell) u = (double)kMaxCell;
    g->cmax[d] = (int64_t)u;
    ncells *= u + 1.0;
  }
  g->inv_h = inv_h;
  g->dense = ncells <= (double)cap ? 1 : 0;
  if (!g->dense)
    for (int d = 0; d < 3; ++d) g->cmax[d] = kMaxCell;
}

__global__ void k_cell_keys(int n, const float* __restrict__ x, const float* __restrict__ y,
                            const float* __restrict__ z, const GridDev* __restrict__ gp, uint64_t* keys, int* idx,
                            int* ccount) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const GridDev g = *gp;
  int64_t c[3];
  cell_of(g, x[i], y[i], z[i], c);
  const uint64_t key = cell_key(g, c[0], c[1], c[2]);
  keys[i] = key;
  idx[i] = i;
  if (g.dense) atomicAdd(&ccount[key], 1);
}

__global__ void k_gather_pos(int n, const int* __restrict__ order, const float* __restrict__ x,
                             const float* __restrict__ y, const float* __restrict__ z, float4* pos) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = order[t];
  pos[t] = make_float4(x[i], y[i], z[i], 0.0f);
}

// ---------------------------------------------------------------------------------
// split

// flag the elongated particles (Split.h:116) and the largest of their search radii
__global__ void k_split_flag(int n, const float* __restrict__ elong, const float* __restrict__ r, float overlap,
                             float threshold, int* flag, int* rmax_bits) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  int f = 0;
  float rad = 0.0f;
  if (i < n && elong[i] > threshold) {
    f = 1;
    rad = split_radius(r[i], overlap);
    if (!(rad >= 0.0f)) rad = 0.0f;
  }
  if (i < n) flag[i] = f;
  for (int o = 16; o > 0; o >>= 1) rad = fmaxf(rad, __shfl_xor_sync(kFull, rad, o));
  if ((threadIdx.x & 31) == 0 && rad > 0.0f) atomicMax(rmax_bits, __float_as_int(rad));
}

// list[k] = index of the k-th flagged particle; pos_of[i] = k or -1
__global__ void k_scatter_flagged(int n, const int* __restrict__ flag, const int* __restrict__ rank, int* list,
                                  int* pos_of) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (flag[i]) {
    list[rank[i]] = i;
    pos_of[i] = rank[i];
  } else {
    pos_of[i] = -1;
  }
}

// one warp per split particle: the number of matches (self included, Split.h:131-132)
__global__ void k_split_count(int m, const int* __restrict__ list, const float* __restrict__ x,
                              const float* __restrict__ y, const float* __restrict__ z, const float* __restrict__ r,
                              float overlap, CellList cl, const GridDev* __restrict__ gp, int* cnt) {
  const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (k >= m) return;
  const GridDev g = *gp;
  const int i = list[k];
  const float qx = x[i], qy = y[i], qz = z[i];
  const float thr = radius_sq(split_radius(r[i], overlap));
  int c = 0;
  visit_cells<32>(cl, g, qx, qy, qz, lane, [&](int t, bool in) {
    if (in && nf_dist2(qx, qy, qz, cl.pos[t]) < thr) ++c;
  });
  c = __reduce_add_sync(kFull, c);
  if (lane == 0) cnt[k] = c;
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// particle i's own part of the split (Split.h:120-129): position, radius and strength axis
struct SplitSelf {
  float x, y, z, r, ax, ay, az;
};

__device__ __forceinline__ SplitSelf split_self(float xi, float yi, float zi, float ri, float sxi, float syi,
                                                float szi) {
  // normalizeVec (MathHelper.h:186-192)
  const float len = __double2float_rn(__ddiv_rn(1.0, (double)__fsqrt_rn(sumsq3(sxi, syi, szi))));
  return SplitSelf{xi, yi, zi, ri, __fmul_rn(sxi, len), __fmul_rn(syi, len), __fmul_rn(szi, len)};
}

// Split.h:146-177: neighbour j's terms (curv x, y, z, dVol) for split particle p; false
// where the reference skips the neighbour (tStr <= 1e-15 or wgt <= 0)
__device__ __forceinline__ bool split_term(const SplitSelf& p, float xj, float yj, float zj, float s0, float s1,
                                           float s2, float rj, float d2, float overlap, float coef, float4& tv) {
  const float dx0 = __fsub_rn(p.x, xj), dx1 = __fsub_rn(p.y, yj), dx2 = __fsub_rn(p.z, zj);
  const float factor = __fmul_rn(__fsqrt_rn(__fdiv_rn(d2, __fmul_rn(rj, p.r))), overlap);
  const double fd = (double)factor;
  const double cube = __dmul_rn(__dmul_rn(fd, fd), fd);
  const float fac2 = __double2float_rn(__dmul_rn((double)coef, exp(-cube)));
  const float tstr = __fsqrt_rn(sumsq3(s0, s1, s2));
  const float wgt = __fadd_rn(__fadd_rn(__fmul_rn(p.ax, s0), __fmul_rn(p.ay, s1)), __fmul_rn(p.az, s2));
  if (!((double)tstr > 1.e-15 && wgt > 0.0f)) return false;
  const float dsx = __fsub_rn(p.ax, __fdiv_rn(s0, tstr));
  const float dsy = __fsub_rn(p.ay, __fdiv_rn(s1, tstr));
  const float dsz = __fsub_rn(p.az, __fdiv_rn(s2, tstr));
  const float thisfac = __fmul_rn(__fmul_rn(wgt, fac2), tstr);
  tv.x = __fmul_rn(thisfac, __fsub_rn(__fmul_rn(dx1, dsz), __fmul_rn(dx2, dsy)));
  tv.y = __fmul_rn(thisfac, __fsub_rn(__fmul_rn(dx2, dsx), __fmul_rn(dx0, dsz)));
  tv.z = __fmul_rn(thisfac, __fsub_rn(__fmul_rn(dx0, dsy), __fmul_rn(dx1, dsx)));
  tv.w = thisfac;
  return true;
}

// codes of a sorted match: its term is precomputed, skipped, or waits for split particle >= 0
constexpr int kCodeTerm = -1;
constexpr int kCodeSkip = -2;

constexpr int kFillWarps = 8;
constexpr int kSortSmem = 256;   // matches of one query sorted in shared memory (more: from global)
constexpr int kOwn = 8;          // matches a lane ranks per pass (kOwn * 32 = kSortSmem)

struct SplitFillArgs {
  int m;
  const int* list;
  const int* pos_of;
  const float *x, *y, *z, *r, *sx, *sy, *sz;
  float overlap, coef;
  CellList cl;
  const GridDev* g;
  const int* off;
  uint64_t* ukeys;   // matches in discovery order (scratch)
  uint64_t* keys;    // matches in the reference's order: (d2, index)
  float4* terms;     // precomputed terms, in that order
  int* code;         // kCodeTerm, kCodeSkip, or the split rank the term waits for
  int* dep;          // the split ranks waited for, compacted at the start of each segment
  int* ndep;         // their number per split particle
  int* err;
};

// one warp per split particle: its matches, ranked into (d2, index) order, and every term
// that does not depend on an earlier split (neighbours that are not split, or split later)
__global__ void __launch_bounds__(kFillWarps * 32) k_split_fill(SplitFillArgs a) {
  __shared__ uint64_t sk[kFillWarps][kSortSmem];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int k = blockIdx.x * kFillWarps + w;
  if (k >= a.m) return;
  const GridDev g = *a.g;
  const int i = a.list[k];
  const float qx = a.x[i], qy = a.y[i], qz = a.z[i], ri = a.r[i];
  const float thr = radius_sq(split_radius(ri, a.overlap));
  const int base = a.off[k], end = a.off[k + 1], c = end - base;
  int run = 0;
  visit_cells<32>(a.cl, g, qx, qy, qz, lane, [&](int t, bool in) {
    float d2 = 0.0f;
    bool hit = false;
    if (in) {
      d2 = nf_dist2(qx, qy, qz, a.cl.pos[t]);
      hit = d2 < thr;
    }
    const unsigned b = __ballot_sync(kFull, hit);
    if (hit) {
      const int slot = base + run + __popc(b & ((1u << lane) - 1u));
      if (slot < end) a.ukeys[slot] = match_key(d2, a.cl.order[t]);
      else atomicCAS(a.err, 0, O3G_ERR_STATE);
    }
    run += __popc(b);
  });
  if (run != c) {
    if (lane == 0) atomicCAS(a.err, 0, O3G_ERR_STATE);
    return;
  }
  __syncwarp();
  const bool in_smem = c <= kSortSmem;
  if (in_smem) {
    for (int q = lane; q < c; q += 32) sk[w][q] = a.ukeys[base + q];
    __syncwarp();
  }
  const SplitSelf p = split_self(qx, qy, qz, ri, a.sx[i], a.sy[i], a.sz[i]);
  int nd = 0;
  for (int cb = 0; cb < c; cb += 32 * kOwn) {
    const int nown = min(kOwn, (c - cb + 31) >> 5);
    uint64_t own[kOwn];
    int rk[kOwn];
#pragma unroll
    for (int r = 0; r < kOwn; ++r) {
      const int q = cb + r * 32 + lane;
      own[r] = (r < nown && q < c) ? (in_smem ? sk[w][q] : a.ukeys[base + q]) : ~0ull;
      rk[r] = 0;
    }
    // keys are distinct (one per neighbour index): rank = number of smaller keys
    for (int q = 0; q < c; ++q) {
      const uint64_t v = in_smem ? sk[w][q] : a.ukeys[base + q];
#pragma unroll
      for (int r = 0; r < kOwn; ++r)
        if (r < nown) rk[r] += v < own[r] ? 1 : 0;
    }
#pragma unroll
    for (int r = 0; r < kOwn; ++r) {
      const int q = cb + r * 32 + lane;
      const bool mine = r < nown && q < c;
      const uint64_t kv = own[r];
      const int j = (int)(uint32_t)kv;
      const int pj = mine ? a.pos_of[j] : -1;
      const bool waits = mine && pj >= 0 && j < i;
      const unsigned wb = __ballot_sync(kFull, waits);
      if (waits) a.dep[base + nd + __popc(wb & ((1u << lane) - 1u))] = pj;
      nd += __popc(wb);
      if (!mine) continue;
      const int dst = base + rk[r];
      a.keys[dst] = kv;
      if (waits) {
        a.code[dst] = pj;
      } else {
        float4 tv = make_float4(0.f, 0.f, 0.f, 0.f);
        const bool ok = split_term(p, a.x[j], a.y[j], a.z[j], a.sx[j], a.sy[j], a.sz[j], a.r[j],
                                   __uint_as_float((uint32_t)(kv >> 32)), a.overlap, a.coef, tv);
        a.code[dst] = ok ? kCodeTerm : kCodeSkip;
        a.terms[dst] = tv;
      }
    }
  }
  if (lane == 0) a.ndep[k] = nd;
}

// level of every split particle in the dependency graph: 0 without dependencies, else one
// more than the deepest particle it waits for.  One thread per particle, claimed 32 at a
// time in index order (dependencies always have lower ranks); a particle publishes level + 1
// with a release store, read with acquire loads by the particles that wait for it.
struct LevelArgs {
  int m;
  const int* off;
  const int* dep;
  const int* ndep;
  int* lvl1;     // level + 1, 0 until published
  int* claim;
  int* err;
  int spread;    // 1: every particle has its own resident thread (no claiming)
  uint32_t spin; // polls before a wait gives up
  uint64_t ns;   // wall time before a wait gives up
  const int* never;   // the wait test: wait on this word (never set) instead
};

__global__ void k_split_levels(LevelArgs a) {
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  for (int round = 0;; ++round) {
    int k;
    if (a.spread) {
      // consecutive ranks (often dependent on each other) land in different warps
      if (round > 0) break;
      k = lane * nwarps + gw;
    } else {
      int k0 = 0;
      if (lane == 0) k0 = atomicAdd(a.claim, 32);
      k0 = __shfl_sync(kFull, k0, 0);
      if (k0 >= a.m) break;
      k = k0 + lane;
    }
    if (k < a.m) {
      const int b = a.off[k], nd = a.ndep[k];
      int lv = 0;
      for (int q = 0; q < nd; ++q) {
        const int pj = a.dep[b + q];
        const int* flag = a.never ? a.never : a.lvl1 + pj;
        const uint64_t t0 = global_ns();
        int v = 0;
        for (uint32_t it = 0; it < a.spin; ++it) {
          asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(flag) : "memory");
          if (v) break;
          if ((it & 1023u) == 1023u && (*(volatile int*)a.err || global_ns() - t0 > a.ns)) break;
          __nanosleep(kPollNs);
        }
        if (!v) {
          atomicCAS(a.err, 0, O3G_ERR_TIMEOUT);
          break;
        }
        lv = max(lv, v);
      }
      asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(a.lvl1 + k), "r"(lv + 1) : "memory");
    }
  }
}

__global__ void k_level_keys(int m, const int* __restrict__ lvl1, uint32_t* key, int* val) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m) return;
  key[k] = (uint32_t)lvl1[k];
  val[k] = k;
}

struct SplitArgs {
  int m;
  const int* order;             // split ranks by level: every dependency comes earlier
  const int* list;
  const int* off;
  const uint64_t* keys;         // sorted matches per split particle
  const float4* terms;          // their precomputed terms
  const int* code;
  const float *x, *y, *z, *r, *elong, *sx, *sy, *sz;   // state before the operator
  float overlap;
  float coef;                   // get_core_coefficient<float>
  float4* post_x;               // x, y, z after the split, w = halved elongation
  float4* post_s;               // strength after the split
  float4* child_x;              // the new particle's position
  float4* child_s;              // the new particle's strength
  int* ready;
  int* claim;
  int* err;
  uint32_t spin;                // polls before a wait gives up
  uint64_t ns;                  // wall time before a wait gives up
  const int* never;             // the wait test: wait on this word (never set) instead
};

// waits for a ready flag; gives up (setting the error word) after `ns` of wall time or
// `spin` polls, or at once when another wait already gave up
__device__ __forceinline__ bool wait_ready(const int* flag, int* err, uint32_t spin, uint64_t ns) {
  const uint64_t t0 = global_ns();
  for (uint32_t it = 0; it < spin; ++it) {
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(flag) : "memory");
    if (v) return true;
    if ((it & 1023u) == 1023u) {
      if (*(volatile int*)err) return false;
      if (global_ns() - t0 > ns) break;
    }
    __nanosleep(kPollNs);
  }
  atomicCAS(err, 0, O3G_ERR_TIMEOUT);
  return false;
}

constexpr int kChainWarps = 4;
constexpr int kPre = 4;   // rounds of 32 matches whose codes and terms are loaded together

// Split.h:116-243 for every elongated particle, in the dependency order described above:
// the precomputed terms are read, the ones that wait for an earlier split are computed from
// its published state, and the sums are added in the sorted order
__global__ void __launch_bounds__(kChainWarps * 32) k_split_chain(SplitArgs a) {
  __shared__ float4 term[kChainWarps][32];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (;;) {
    int c = 0;
    if (lane == 0) c = atomicAdd(a.claim, 1);
    c = __shfl_sync(kFull, c, 0);
    if (c >= a.m) break;
    const int k = a.order[c];
    const int i = a.list[k];
    const float xi = a.x[i], yi = a.y[i], zi = a.z[i], ri = a.r[i], ei = a.elong[i];
    const float sxi = a.sx[i], syi = a.sy[i], szi = a.sz[i];
    const SplitSelf p = split_self(xi, yi, zi, ri, sxi, syi, szi);
    float acc = 0.0f;   // lane 0..2: curv[lane], lane 3: dVol
    const int b = a.off[k], e = a.off[k + 1];
    for (int cb = b; cb < e; cb += 32 * kPre) {
      int cd[kPre];
      float4 tv[kPre];
      uint64_t kv[kPre];
#pragma unroll
      for (int r = 0; r < kPre; ++r) {
        const int t = cb + r * 32 + lane;
        cd[r] = t < e ? a.code[t] : kCodeSkip;
        tv[r] = t < e ? a.terms[t] : make_float4(0.f, 0.f, 0.f, 0.f);
        kv[r] = t < e ? a.keys[t] : 0ull;
      }
      // terms that wait for an earlier split: radii first (never change), then every wait,
      // then all the published states at once
      float rj[kPre];
#pragma unroll
      for (int r = 0; r < kPre; ++r) rj[r] = cd[r] >= 0 ? a.r[(int)(uint32_t)kv[r]] : 0.0f;
#pragma unroll
      for (int r = 0; r < kPre; ++r)
        if (cd[r] >= 0) wait_ready(a.never ? a.never : &a.ready[cd[r]], a.err, a.spin, a.ns);
      float4 px[kPre], ps[kPre];
#pragma unroll
      for (int r = 0; r < kPre; ++r)
        if (cd[r] >= 0) {
          px[r] = __ldcg(&a.post_x[cd[r]]);
          ps[r] = __ldcg(&a.post_s[cd[r]]);
        }
#pragma unroll
      for (int r = 0; r < kPre; ++r)
        if (cd[r] >= 0) {
          tv[r] = make_float4(0.f, 0.f, 0.f, 0.f);
          const bool ok = split_term(p, px[r].x, px[r].y, px[r].z, ps[r].x, ps[r].y, ps[r].z, rj[r],
                                     __uint_as_float((uint32_t)(kv[r] >> 32)), a.overlap, a.coef, tv[r]);
          cd[r] = ok ? kCodeTerm : kCodeSkip;
        }
#pragma unroll
      for (int r = 0; r < kPre; ++r) {
        const int rb = cb + r * 32;
        if (rb >= e) break;
        term[w][lane] = tv[r];
        const unsigned vm = __ballot_sync(kFull, cd[r] == kCodeTerm);
        __syncwarp();
        if (lane < 4) {
          // the 32 values are read first, then added in order (vm is zero past the end)
          const float* tp = reinterpret_cast<const float*>(&term[w][0]) + lane;
          float v[32];
#pragma unroll
          for (int q = 0; q < 32; ++q) v[q] = tp[4 * q];
#pragma unroll
          for (int q = 0; q < 32; ++q)
            if ((vm >> q) & 1u) acc = __fadd_rn(acc, v[q]);
        }
        __syncwarp();
      }
    }
    float curv0 = __shfl_sync(kFull, acc, 0), curv1 = __shfl_sync(kFull, acc, 1);
    float curv2 = __shfl_sync(kFull, acc, 2);
    const float dvol = __shfl_sync(kFull, acc, 3);
    if (lane == 0) {
      const float nom_sep = __fdiv_rn(ri, a.overlap);
      const float halfd = __double2float_rn(__dmul_rn(__dmul_rn(0.25, (double)ei), (double)nom_sep));
      const float he = __double2float_rn(__dmul_rn(0.5, (double)ei));
      const float hx = __double2float_rn(__dmul_rn(0.5, (double)sxi));
      const float hy = __double2float_rn(__dmul_rn(0.5, (double)syi));
      const float hz = __double2float_rn(__dmul_rn(0.5, (double)szi));
      float csx = hx, csy = hy, csz = hz, psx = hx, psy = hy, psz = hz;
      if ((double)dvol > 1e-15) {
        curv0 = __fdiv_rn(curv0, dvol);
        curv1 = __fdiv_rn(curv1, dvol);
        curv2 = __fdiv_rn(curv2, dvol);
        const float f = __double2float_rn(__ddiv_rn(__dmul_rn((double)a.overlap, 0.398967), (double)ri));
        curv0 = __fmul_rn(curv0, f);
        curv1 = __fmul_rn(curv1, f);
        curv2 = __fmul_rn(curv2, f);
        const float dsx = __fsub_rn(__fmul_rn(hy, curv2), __fmul_rn(hz, curv1));
        const float dsy = __fsub_rn(__fmul_rn(hz, curv0), __fmul_rn(hx, curv2));
        const float dsz = __fsub_rn(__fmul_rn(hx, curv1), __fmul_rn(hy, curv0));
        csx = __fadd_rn(csx, dsx); csy = __fadd_rn(csy, dsy); csz = __fadd_rn(csz, dsz);
        psx = __fsub_rn(psx, dsx); psy = __fsub_rn(psy, dsy); psz = __fsub_rn(psz, dsz);
      }
      const float mx = __fmul_rn(halfd, p.ax), my = __fmul_rn(halfd, p.ay), mz = __fmul_rn(halfd, p.az);
      a.child_x[k] = make_float4(__fsub_rn(xi, mx), __fsub_rn(yi, my), __fsub_rn(zi, mz), 0.0f);
      a.child_s[k] = make_float4(csx, csy, csz, 0.0f);
      a.post_x[k] = make_float4(__fadd_rn(xi, mx), __fadd_rn(yi, my), __fadd_rn(zi, mz), he);
      a.post_s[k] = make_float4(psx, psy, psz, 0.0f);
      // the release store orders the four writes above before the flag
      asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(&a.ready[k]), "r"(1) : "memory");
    }
    __syncwarp();
  }
}

// writes the split's results; nothing when a wait of the chain gave up (the error word is
// set), so that a failed call leaves the particles as they were
__global__ void k_split_write(int m, int n, const int* __restrict__ list, const float4* __restrict__ post_x,
                              const float4* __restrict__ post_s, const float4* __restrict__ child_x,
                              const float4* __restrict__ child_s, float* x, float* y, float* z, float* r, float* elong,
                              float* sx, float* sy, float* sz, const int* __restrict__ err) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m || *err) return;
  const int i = list[k], c = n + k;
  const float4 px = post_x[k], ps = post_s[k], cx = child_x[k], cs = child_s[k];
  x[c] = cx.x; y[c] = cx.y; z[c] = cx.z; r[c] = r[i]; elong[c] = px.w;
  sx[c] = cs.x; sy[c] = cs.y; sz[c] = cs.z;
  x[i] = px.x; y[i] = px.y; z[i] = px.z; elong[i] = px.w;
  sx[i] = ps.x; sy[i] = ps.y; sz[i] = ps.z;
}

// ---------------------------------------------------------------------------------
// merge

// per particle: the mean-strength term (Merge.h:102) and the largest search radius
__global__ void k_merge_prep(int n, const float* __restrict__ sx, const float* __restrict__ sy,
                             const float* __restrict__ sz, const float* __restrict__ r, float overlap, float* term,
                             int* rmax_bits) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  float rad = 0.0f;
  if (i < n) {
    term[i] = __fsqrt_rn(sumsq3(sx[i], sy[i], sz[i]));
    rad = merge_radius(r[i], overlap);
    if (!(rad >= 0.0f)) rad = 0.0f;
  }
  for (int o = 16; o > 0; o >>= 1) rad = fmaxf(rad, __shfl_xor_sync(kFull, rad, o));
  if ((threadIdx.x & 31) == 0 && rad > 0.0f) atomicMax(rmax_bits, __float_as_int(rad));
}

constexpr int kMeanThreads = 256;
constexpr int kMeanChunk = 4096;

// meanstr = (sum in index order of the terms) / (float)n, the reference's float loop;
// warps 1.. stage chunk c+1 in shared memory while thread 0 adds chunk c
__global__ void __launch_bounds__(kMeanThreads) k_meanstr(int n, const float* __restrict__ term, float* out) {
  __shared__ __align__(16) float buf[2][kMeanChunk];
  const int nch = (n + kMeanChunk - 1) / kMeanChunk;
  const int loaders = kMeanThreads - 32, lt = threadIdx.x - 32;
  if (threadIdx.x >= 32)
    for (int q = lt; q < kMeanChunk; q += loaders) buf[0][q] = q < n ? term[q] : 0.0f;
  __syncthreads();
  float s = 0.0f;
  for (int c = 0; c < nch; ++c) {
    if (threadIdx.x >= 32 && c + 1 < nch) {
      const int b = (c + 1) * kMeanChunk;
      for (int q = lt; q < kMeanChunk; q += loaders) buf[(c + 1) & 1][q] = b + q < n ? term[b + q] : 0.0f;
    }
    if (threadIdx.x == 0) {
      const int cnt = min(kMeanChunk, n - c * kMeanChunk);
      const float* p = buf[c & 1];
      // the next 8 terms are read while the current 8 are added
      int q = 0;
      float4 v0, v1;
      if (cnt >= 8) {
        v0 = *reinterpret_cast<const float4*>(p);
        v1 = *reinterpret_cast<const float4*>(p + 4);
      }
      for (; q + 8 <= cnt; q += 8) {
        float4 n0 = v0, n1 = v1;
        if (q + 16 <= cnt) {
          n0 = *reinterpret_cast<const float4*>(p + q + 8);
          n1 = *reinterpret_cast<const float4*>(p + q + 12);
        }
        s = __fadd_rn(s, v0.x); s = __fadd_rn(s, v0.y); s = __fadd_rn(s, v0.z); s = __fadd_rn(s, v0.w);
        s = __fadd_rn(s, v1.x); s = __fadd_rn(s, v1.y); s = __fadd_rn(s, v1.z); s = __fadd_rn(s, v1.w);
        v0 = n0;
        v1 = n1;
      }
      for (; q < cnt; ++q) s = __fadd_rn(s, p[q]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = __fdiv_rn(s, __int2float_rn(n));
}

// thread per particle: matches other than itself (Merge.h:127-135)
template <bool FILL>
__global__ void k_merge_search(int n, const float* __restrict__ x, const float* __restrict__ y,
                               const float* __restrict__ z, const float* __restrict__ r, float overlap, CellList cl,
                               const GridDev* __restrict__ gp, int* cnt, const int* __restrict__ off, uint64_t* keys,
                               int* err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const GridDev g = *gp;
  const float qx = x[i], qy = y[i], qz = z[i];
  const float thr = radius_sq(merge_radius(r[i], overlap));
  int c = 0;
  const int base = FILL ? off[i] : 0, end = FILL ? off[i + 1] : 0;
  visit_cells<1>(cl, g, qx, qy, qz, 0, [&](int t, bool in) {
    if (!in) return;
    const float d2 = nf_dist2(qx, qy, qz, cl.pos[t]);
    if (!(d2 < thr)) return;
    const int j = cl.order[t];
    if (j == i) return;
    if (FILL) {
      if (base + c < end) keys[base + c] = match_key(d2, j);
      else atomicCAS(err, 0, O3G_ERR_STATE);
    }
    ++c;
  });
  if (!FILL) cnt[i] = c;
}

__device__ __forceinline__ int vload(const int* p) { return *(const volatile int*)p; }

// root of x; parent[v] <= v everywhere, so the walk ends; path halving stores only
// ancestors into non-roots
__device__ int uf_find(int* parent, int x) {
  int cur = x;
  int next = vload(&parent[cur]);
  while (next != cur) {
    const int nn = vload(&parent[next]);
    if (nn != next) *(volatile int*)&parent[cur] = nn;
    cur = next;
    next = nn;
  }
  return cur;
}

__device__ void uf_unite(int* parent, int a, int b) {
  int ra = uf_find(parent, a), rb = uf_find(parent, b);
  // every failed CAS moves one side to a strictly smaller index: at most n rounds
  while (ra != rb) {
    if (ra < rb) {
      const int old = atomicCAS(&parent[rb], rb, ra);
      if (old == rb) break;
      rb = old;
    } else {
      const int old = atomicCAS(&parent[ra], ra, rb);
      if (old == ra) break;
      ra = old;
    }
  }
}

__global__ void k_uf_init(int n, int* parent, int* act) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) { parent[i] = i; act[i] = 0; }
}

__global__ void k_uf_edges(int n, const int* __restrict__ off, const uint64_t* __restrict__ keys, int* parent,
                           int* act) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int b = off[i], e = off[i + 1];
  if (e > b) act[i] = 1;
  for (int t = b; t < e; ++t) {
    const int j = (int)(uint32_t)keys[t];
    act[j] = 1;
    uf_unite(parent, i, j);
  }
}

// active particles in index order with their group roots
__global__ void k_scatter_active(int n, int* parent, const int* __restrict__ act, const int* __restrict__ rank,
                                 uint32_t* akey, int* aval) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !act[i]) return;
  akey[rank[i]] = (uint32_t)uf_find(parent, i);
  aval[rank[i]] = i;
}

__global__ void k_group_heads(const int* __restrict__ na_p, const uint32_t* __restrict__ key, int* head) {
  const int na = *na_p;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < na) head[t] = (t == 0 || key[t] != key[t - 1]) ? 1 : 0;
  else if (t == na) head[t] = 0;
}

__global__ void k_scatter_heads(const int* __restrict__ na_p, const int* __restrict__ head,
                                const int* __restrict__ rank, int* start) {
  const int na = *na_p;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < na && head[t]) start[rank[t]] = t;
  if (t == na) start[rank[na]] = na;   // one past the last group
}

struct MergeArgs {
  const int* ng;                // number of groups (device)
  const int* start;             // group g = sorted slots [start[g], start[g + 1])
  const int* member;            // particle index per sorted slot
  const int* off;
  const uint64_t* keys;         // sorted matches per particle
  float *x, *y, *z, *sx, *sy, *sz, *r;
  unsigned char* erase;
  const float* meanstr;
  float overlap, threshold;
  int adapt;
};

// Merge.h:107-176 restricted to one group, its particles in increasing index
__global__ void k_merge_resolve(MergeArgs a) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= *a.ng) return;
  const float meanstr = *a.meanstr;
  const float initial_thresh = 0.5f, always_thresh = 0.1f;
  const float eps = 1.1920929e-07f;   // std::numeric_limits<float>::epsilon()
  for (int t = a.start[g]; t < a.start[g + 1]; ++t) {
    const int i = a.member[t];
    if (a.erase[i]) continue;
    for (int q = a.off[i]; q < a.off[i + 1]; ++q) {
      const uint64_t kv = a.keys[q];
      const int j = (int)(uint32_t)kv;
      if (a.erase[j]) continue;
      const float dist = __fsqrt_rn(__uint_as_float((uint32_t)(kv >> 32)));
      const float rj = a.r[j];
      if (!(dist < __fdiv_rn(__fmul_rn(initial_thresh, rj), a.overlap))) continue;
      float ri = a.r[i];
      const float si = __fadd_rn(__fsqrt_rn(sumsq3(a.sx[i], a.sy[i], a.sz[i])), eps);
      const float so = __fadd_rn(__fsqrt_rn(sumsq3(a.sx[j], a.sy[j], a.sz[j])), eps);
      const float frac = __fdiv_rn(so, __fadd_rn(si, so));
      bool do_merge = false;
      const float min_rad = __fdiv_rn(ri < rj ? ri : rj, a.overlap);   // std::min(r[j], r[i])
      if (__fmul_rn(__fmul_rn(dist, frac), si) < __fmul_rn(__fmul_rn(a.threshold, meanstr), min_rad))
        do_merge = true;
      if (dist < __fmul_rn(always_thresh, min_rad)) do_merge = true;
      if (!do_merge) continue;
      const float omfrac = __double2float_rn(__dsub_rn(1.0, (double)frac));
      const float nx = __fadd_rn(__fmul_rn(a.x[i], omfrac), __fmul_rn(a.x[j], frac));
      const float ny = __fadd_rn(__fmul_rn(a.y[i], omfrac), __fmul_rn(a.y[j], frac));
      const float nz = __fadd_rn(__fmul_rn(a.z[i], omfrac), __fmul_rn(a.z[j], frac));
      a.x[i] = nx;
      a.y[i] = ny;
      a.z[i] = nz;
      if (a.adapt) {
        const double di = (double)ri, dj = (double)rj;
        const double ci = __dmul_rn(__dmul_rn(di, di), di), cj = __dmul_rn(__dmul_rn(dj, dj), dj);
        ri = __double2float_rn(cbrt(__dadd_rn(__dmul_rn((double)omfrac, ci), __dmul_rn((double)frac, cj))));
        a.r[i] = ri;
      }
      a.sx[i] = __fadd_rn(a.sx[i], a.sx[j]);
      a.sy[i] = __fadd_rn(a.sy[i], a.sy[j]);
      a.sz[i] = __fadd_rn(a.sz[i], a.sz[j]);
      a.erase[j] = 1;
    }
  }
}

__global__ void k_keep_flags(int n, const unsigned char* __restrict__ erase, int* keep) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) keep[i] = erase[i] ? 0 : 1;
  else if (i == n) keep[i] = 0;
}

struct Arr7 { float* p[7]; };

__global__ void k_compact(int n, const int* __restrict__ keep, const int* __restrict__ dst, Arr7 src, Arr7 out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !keep[i]) return;
  const int d = dst[i];
#pragma unroll
  for (int c = 0; c < 7; ++c) out.p[c][d] = src.p[c][i];
}

// ---------------------------------------------------------------------------------
// host side

// device scratch of one call, released (stream-ordered) when the call returns
struct Scratch {
  cudaStream_t st;
  std::vector<void*> ptrs;
  explicit Scratch(cudaStream_t s) : st(s) {}
  ~Scratch() {
    for (void* p : ptrs) cudaFreeAsync(p, st);
  }
  template <class T>
  int32_t get(T** p, size_t count) {
    if (count == 0) count = 1;
    const cudaError_t e = o3g::dev_alloc_async((void**)p, count * sizeof(T), st);
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      set_error_cuda("o3g::dev_alloc_async(split/merge scratch)", e);
      return O3G_ERR_ALLOC;
    }
    ptrs.push_back(*p);
    return O3G_OK;
  }
};

inline int blocks(long long n, int t = 256) { return (int)((n + t - 1) / t); }

int32_t exclusive_sum(Scratch& sc, const int* in, int* out, int count) {
  size_t tb = 0;
  O3G_CUDA_TRY(cub::DeviceScan::ExclusiveSum(nullptr, tb, in, out, count, sc.st));
  void* tmp = nullptr;
  O3G_TRY(sc.get((char**)&tmp, tb));
  O3G_CUDA_TRY(cub::DeviceScan::ExclusiveSum(tmp, tb, in, out, count, sc.st));
  return O3G_OK;
}

int32_t read_int(const int* dev, int* host, cudaStream_t st) {
  O3G_CUDA_TRY(cudaMemcpyAsync(host, dev, sizeof(int), cudaMemcpyDeviceToHost, st));
  O3G_CUDA_TRY(cudaStreamSynchronize(st));
  return O3G_OK;
}

// the cell list over n positions; lo_ord / rmax_bits already hold the bbox minimum and
// the largest search radius
int32_t build_cells(Scratch& sc, int n, const float* x, const float* y, const float* z, const int* bb,
                    const int* rmax_bits, CellList* cl, GridDev** grid) {
  cudaStream_t st = sc.st;
  GridDev* g = nullptr;
  uint64_t *kin = nullptr, *kout = nullptr;
  int *iin = nullptr, *iout = nullptr, *ccount = nullptr, *cstart = nullptr;
  float4* pos = nullptr;
  // a dense start table for up to 16 cells per particle (at least 2^20, at most 2^28)
  const long long cap = std::min<long long>(std::max<long long>(16ll * n, 1ll << 20), 1ll << 28);
  O3G_TRY(sc.get(&g, 1));
  O3G_TRY(sc.get(&kin, n));
  O3G_TRY(sc.get(&kout, n));
  O3G_TRY(sc.get(&iin, n));
  O3G_TRY(sc.get(&iout, n));
  O3G_TRY(sc.get(&pos, n));
  O3G_TRY(sc.get(&ccount, (size_t)cap + 1));
  O3G_TRY(sc.get(&cstart, (size_t)cap + 1));
  O3G_CUDA_TRY(cudaMemsetAsync(ccount, 0, ((size_t)cap + 1) * sizeof(int), st));
  k_grid<<<1, 1, 0, st>>>(bb, rmax_bits, cap, g);
  k_cell_keys<<<blocks(n), 256, 0, st>>>(n, x, y, z, g, kin, iin, ccount);
  O3G_TRY(exclusive_sum(sc, ccount, cstart, (int)(cap + 1)));
  size_t tb = 0;
  O3G_CUDA_TRY(cub::DeviceRadixSort::SortPairs(nullptr, tb, kin, kout, iin, iout, n, 0, 63, st));
  void* tmp = nullptr;
  O3G_TRY(sc.get((char**)&tmp, tb));
  O3G_CUDA_TRY(cub::DeviceRadixSort::SortPairs(tmp, tb, kin, kout, iin, iout, n, 0, 63, st));
  k_gather_pos<<<blocks(n), 256, 0, st>>>(n, iout, x, y, z, pos);
  note_launch(3);
  O3G_CUDA_TRY(cudaGetLastError());
  cl->keys = kout;
  cl->order = iout;
  cl->pos = pos;
  cl->cstart = cstart;
  cl->n = n;
  *grid = g;
  return O3G_OK;
}

struct Add64 {
  __host__ __device__ long long operator()(long long a, long long b) const { return a + b; }
};

// the number of matches over all queries, summed in 64 bits: the match lists are indexed
// by int offsets (an int exclusive sum of cnt), so a total above INT_MAX is refused before
// anything is allocated or written
int32_t match_total(Scratch& sc, const int* cnt, int count, int* total, const char* what) {
  long long* sum = nullptr;
  O3G_TRY(sc.get(&sum, 1));
  size_t tb = 0;
  O3G_CUDA_TRY(cub::DeviceReduce::Reduce(nullptr, tb, cnt, sum, count, Add64(), 0ll, sc.st));
  void* tmp = nullptr;
  O3G_TRY(sc.get((char**)&tmp, tb));
  O3G_CUDA_TRY(cub::DeviceReduce::Reduce(tmp, tb, cnt, sum, count, Add64(), 0ll, sc.st));
  long long h = 0;
  O3G_CUDA_TRY(cudaMemcpyAsync(&h, sum, sizeof(h), cudaMemcpyDeviceToHost, sc.st));
  O3G_CUDA_TRY(cudaStreamSynchronize(sc.st));
  if (h < 0 || h > (long long)INT_MAX) {
    set_error(what);
    return O3G_ERR_INVALID_ARG;
  }
  *total = (int)h;
  return O3G_OK;
}

int32_t sort_matches(Scratch& sc, uint64_t* keys, uint64_t** sorted, int total, int nseg, const int* off) {
  uint64_t* out = nullptr;
  O3G_TRY(sc.get(&out, total));
  size_t tb = 0;
  O3G_CUDA_TRY(cub::DeviceSegmentedSort::SortKeys(nullptr, tb, keys, out, total, nseg, off, off + 1, sc.st));
  void* tmp = nullptr;
  O3G_TRY(sc.get((char**)&tmp, tb));
  O3G_CUDA_TRY(cub::DeviceSegmentedSort::SortKeys(tmp, tb, keys, out, total, nseg, off, off + 1, sc.st));
  *sorted = out;
  return O3G_OK;
}

int32_t check_err(const int* err, cudaStream_t st, const char* what) {
  int h = 0;
  O3G_TRY(read_int(err, &h, st));
  if (h != 0) {
    set_error(what);
    return h;
  }
  return O3G_OK;
}

int32_t split_run(int n, int cap, float* x, float* y, float* z, float* r, float* elong, float* sx, float* sy,
                  float* sz, int core, float overlap, float threshold, int* nsplit, cudaStream_t st) {
  Scratch sc(st);
  int *lo_ord = nullptr, *rmax = nullptr, *flag = nullptr, *rank = nullptr, *err = nullptr;
  O3G_TRY(sc.get(&lo_ord, 6));
  O3G_TRY(sc.get(&rmax, 1));
  O3G_TRY(sc.get(&err, 4));   // error word, chain and level claim counters, a word never set
  O3G_TRY(sc.get(&flag, (size_t)n + 1));
  O3G_TRY(sc.get(&rank, (size_t)n + 1));
  O3G_CUDA_TRY(cudaMemsetAsync(err, 0, 4 * sizeof(int), st));
  const bool wtest = wait_test_on();
  const uint32_t wspin = wtest ? kTestSpin : kReadySpin;
  const uint64_t wns = wtest ? kTestNs : kReadyNs;
  const int* never = wtest ? err + 3 : nullptr;
  k_sm_init<<<1, 32, 0, st>>>(lo_ord, rmax);
  k_split_flag<<<blocks(n), 256, 0, st>>>(n, elong, r, overlap, threshold, flag, rmax);
  O3G_CUDA_TRY(cudaMemsetAsync(flag + n, 0, sizeof(int), st));
  note_launch(2);
  O3G_TRY(exclusive_sum(sc, flag, rank, n + 1));
  int m = 0;
  O3G_TRY(read_int(rank + n, &m, st));
  *nsplit = m;
  if (m == 0) return O3G_OK;
  if ((long long)n + m > (long long)cap) {
    set_error("o3g_split_elongated: the arrays have room for fewer particles than n + nsplit");
    return O3G_ERR_CAPACITY;
  }
  int *list = nullptr, *pos_of = nullptr, *cnt = nullptr, *off = nullptr, *ready = nullptr;
  O3G_TRY(sc.get(&list, m));
  O3G_TRY(sc.get(&pos_of, n));
  O3G_TRY(sc.get(&cnt, (size_t)m + 1));
  O3G_TRY(sc.get(&off, (size_t)m + 1));
  O3G_TRY(sc.get(&ready, m));
  k_scatter_flagged<<<blocks(n), 256, 0, st>>>(n, flag, rank, list, pos_of);
  k_bbox<<<std::min(blocks(n), 1024), 256, 0, st>>>(n, x, y, z, lo_ord);
  note_launch(2);
  CellList cl{};
  GridDev* g = nullptr;
  O3G_TRY(build_cells(sc, n, x, y, z, lo_ord, rmax, &cl, &g));
  k_split_count<<<blocks((long long)m * 32), 256, 0, st>>>(m, list, x, y, z, r, overlap, cl, g, cnt);
  O3G_CUDA_TRY(cudaMemsetAsync(cnt + m, 0, sizeof(int), st));
  note_launch(1);
  O3G_TRY(exclusive_sum(sc, cnt, off, m + 1));
  int total = 0;
  O3G_TRY(match_total(sc, cnt, m, &total,
                      "o3g_split_elongated: more than 2^31 - 1 neighbour matches in all (coincident particles?)"));
  uint64_t *ukeys = nullptr, *keys = nullptr;
  float4* terms = nullptr;
  int *code = nullptr, *dep = nullptr, *ndep = nullptr;
  O3G_TRY(sc.get(&ukeys, total));
  O3G_TRY(sc.get(&keys, total));
  O3G_TRY(sc.get(&terms, total));
  O3G_TRY(sc.get(&code, total));
  O3G_TRY(sc.get(&dep, total));
  O3G_TRY(sc.get(&ndep, m));
  const double pi = 3.14159265358979323846;
  // get_core_coefficient<float> (Core.h:32-35): gaussian 1/(pi sqrt(pi)) in double, else 0.23873241
  const float coef = core == O3G_DIFFCORE_GAUSSIAN ? (float)(1.0 / (pi * std::sqrt(pi))) : (float)0.23873241;
  SplitFillArgs fa;
  fa.m = m; fa.list = list; fa.pos_of = pos_of;
  fa.x = x; fa.y = y; fa.z = z; fa.r = r; fa.sx = sx; fa.sy = sy; fa.sz = sz;
  fa.overlap = overlap; fa.coef = coef; fa.cl = cl; fa.g = g; fa.off = off;
  fa.ukeys = ukeys; fa.keys = keys; fa.terms = terms; fa.code = code; fa.dep = dep; fa.ndep = ndep;
  fa.err = err;
  k_split_fill<<<(m + kFillWarps - 1) / kFillWarps, kFillWarps * 32, 0, st>>>(fa);
  note_launch(1);

  // levels, and the split ranks sorted by level: the chain's claim order
  DeviceFacts f;
  O3G_TRY(device_facts(&f));
  int *lvl1 = nullptr, *kin = nullptr, *order = nullptr;
  uint32_t *lkey = nullptr, *lkey2 = nullptr;
  O3G_TRY(sc.get(&lvl1, m));
  O3G_TRY(sc.get(&kin, m));
  O3G_TRY(sc.get(&order, m));
  O3G_TRY(sc.get(&lkey, m));
  O3G_TRY(sc.get(&lkey2, m));
  O3G_CUDA_TRY(cudaMemsetAsync(lvl1, 0, (size_t)m * sizeof(int), st));
  {
    int lb = 0;
    O3G_TRY(occupancy_blocks((const void*)k_split_levels, 256, &lb));
    int lgrid = std::max(1, lb) * f.num_sms;
    lgrid = std::min(lgrid, (m + 255) / 256);
    // with a thread for every particle all of them are in flight at once, so any mapping is
    // deadlock-free; otherwise they are claimed in rank order
    const int spread = (long long)lgrid * 256 >= (long long)m ? 1 : 0;
    LevelArgs la{m, off, dep, ndep, lvl1, err + 2, err, spread, wspin, wns, never};
    void* largs[] = {&la};
    O3G_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)k_split_levels, dim3(lgrid), dim3(256), largs, 0, st));
  }
  k_level_keys<<<blocks(m), 256, 0, st>>>(m, lvl1, lkey, kin);
  note_launch(2);
  {
    int lbits = 1;
    while (lbits < 31 && (1ll << lbits) <= (long long)m + 1) ++lbits;
    size_t tb = 0;
    O3G_CUDA_TRY(cub::DeviceRadixSort::SortPairs(nullptr, tb, lkey, lkey2, kin, order, m, 0, lbits, st));
    void* tmp = nullptr;
    O3G_TRY(sc.get((char**)&tmp, tb));
    O3G_CUDA_TRY(cub::DeviceRadixSort::SortPairs(tmp, tb, lkey, lkey2, kin, order, m, 0, lbits, st));
  }

  float4 *post_x = nullptr, *post_s = nullptr, *child_x = nullptr, *child_s = nullptr;
  O3G_TRY(sc.get(&post_x, m));
  O3G_TRY(sc.get(&post_s, m));
  O3G_TRY(sc.get(&child_x, m));
  O3G_TRY(sc.get(&child_s, m));
  O3G_CUDA_TRY(cudaMemsetAsync(ready, 0, (size_t)m * sizeof(int), st));
  SplitArgs a;
  a.m = m; a.order = order; a.list = list; a.off = off; a.keys = keys; a.terms = terms; a.code = code;
  a.x = x; a.y = y; a.z = z; a.r = r; a.elong = elong; a.sx = sx; a.sy = sy; a.sz = sz;
  a.overlap = overlap;
  a.coef = coef;
  a.post_x = post_x; a.post_s = post_s; a.child_x = child_x; a.child_s = child_s;
  a.ready = ready; a.claim = err + 1; a.err = err;
  a.spin = wspin; a.ns = wns; a.never = never;
  int nb = 0;
  O3G_TRY(occupancy_blocks((const void*)k_split_chain, kChainWarps * 32, &nb));
  int grid = std::max(1, nb) * f.num_sms;
  grid = std::min(grid, (m + kChainWarps - 1) / kChainWarps);
  void* args[] = {&a};
  O3G_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)k_split_chain, dim3(grid), dim3(kChainWarps * 32), args, 0,
                                           st));
  k_split_write<<<blocks(m), 256, 0, st>>>(m, n, list, post_x, post_s, child_x, child_s, x, y, z, r, elong, sx, sy,
                                           sz, err);
  note_launch(2);
  O3G_CUDA_TRY(cudaGetLastError());
  return check_err(err, st, "o3g_split_elongated: a device-side check failed (ready-flag wait or match count)");
}

// a second stream per device for the mean-strength sum, which overlaps the neighbour search
int32_t side_stream(cudaStream_t* out) {
  static std::mutex mu;
  static cudaStream_t streams[64] = {};
  int dev = 0;
  O3G_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) {
    set_error("o3g_merge_close_particles: device index out of range");
    return O3G_ERR_INVALID_ARG;
  }
  std::lock_guard<std::mutex> lk(mu);
  if (!streams[dev]) O3G_CUDA_TRY(cudaStreamCreateWithFlags(&streams[dev], cudaStreamNonBlocking));
  *out = streams[dev];
  return O3G_OK;
}

// joins the side stream back into the caller's stream before the scratch it reads is freed
struct Join {
  cudaStream_t st = nullptr;
  cudaEvent_t done = nullptr;
  ~Join() {
    if (done) {
      cudaStreamWaitEvent(st, done, 0);
      cudaEventDestroy(done);
    }
  }
};

int32_t merge_run(int n, float* x, float* y, float* z, float* sx, float* sy, float* sz, float* r, float overlap,
                  float threshold, int adapt, int* nremoved, cudaStream_t st) {
  Scratch sc(st);
  int *lo_ord = nullptr, *rmax = nullptr, *err = nullptr, *cnt = nullptr, *off = nullptr;
  float *term = nullptr, *meanstr = nullptr;
  O3G_TRY(sc.get(&lo_ord, 6));
  O3G_TRY(sc.get(&rmax, 1));
  O3G_TRY(sc.get(&err, 1));
  O3G_TRY(sc.get(&term, n));
  O3G_TRY(sc.get(&meanstr, 1));
  O3G_TRY(sc.get(&cnt, (size_t)n + 1));
  O3G_TRY(sc.get(&off, (size_t)n + 1));
  O3G_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), st));
  k_sm_init<<<1, 32, 0, st>>>(lo_ord, rmax);
  k_merge_prep<<<blocks(n), 256, 0, st>>>(n, sx, sy, sz, r, overlap, term, rmax);
  // the sequential sum runs on the side stream from here until k_merge_resolve needs it
  cudaStream_t side = nullptr;
  O3G_TRY(side_stream(&side));
  Join join;
  cudaEvent_t prepped = nullptr;
  O3G_CUDA_TRY(cudaEventCreateWithFlags(&prepped, cudaEventDisableTiming));
  cudaError_t ev = cudaEventRecord(prepped, st);
  if (ev == cudaSuccess) ev = cudaStreamWaitEvent(side, prepped, 0);
  cudaEventDestroy(prepped);
  if (ev != cudaSuccess) {
    set_error_cuda("o3g_merge_close_particles: stream fork", ev);
    return O3G_ERR_CUDA;
  }
  k_meanstr<<<1, kMeanThreads, 0, side>>>(n, term, meanstr);
  join.st = st;
  O3G_CUDA_TRY(cudaEventCreateWithFlags(&join.done, cudaEventDisableTiming));
  O3G_CUDA_TRY(cudaEventRecord(join.done, side));
  k_bbox<<<std::min(blocks(n), 1024), 256, 0, st>>>(n, x, y, z, lo_ord);
  note_launch(4);
  CellList cl{};
  GridDev* g = nullptr;
  O3G_TRY(build_cells(sc, n, x, y, z, lo_ord, rmax, &cl, &g));
  k_merge_search<false><<<blocks(n), 256, 0, st>>>(n, x, y, z, r, overlap, cl, g, cnt, nullptr, nullptr, err);
  O3G_CUDA_TRY(cudaMemsetAsync(cnt + n, 0, sizeof(int), st));
  note_launch(1);
  O3G_TRY(exclusive_sum(sc, cnt, off, n + 1));
  int total = 0;
  O3G_TRY(match_total(sc, cnt, n, &total,
                      "o3g_merge_close_particles: more than 2^31 - 1 neighbour matches in all (coincident particles?)"));
  *nremoved = 0;
  if (total == 0) return O3G_OK;
  uint64_t *keys = nullptr, *sorted = nullptr;
  O3G_TRY(sc.get(&keys, total));
  k_merge_search<true><<<blocks(n), 256, 0, st>>>(n, x, y, z, r, overlap, cl, g, nullptr, off, keys, err);
  note_launch(1);
  O3G_TRY(sort_matches(sc, keys, &sorted, total, n, off));

  // groups of the match graph
  int *parent = nullptr, *act = nullptr, *arank = nullptr, *aval = nullptr, *aval2 = nullptr, *head = nullptr,
      *hrank = nullptr, *start = nullptr;
  uint32_t *akey = nullptr, *akey2 = nullptr;
  O3G_TRY(sc.get(&parent, n));
  O3G_TRY(sc.get(&act, (size_t)n + 1));
  O3G_TRY(sc.get(&arank, (size_t)n + 1));
  O3G_TRY(sc.get(&akey, n));
  O3G_TRY(sc.get(&aval, n));
  O3G_TRY(sc.get(&akey2, n));
  O3G_TRY(sc.get(&aval2, n));
  O3G_TRY(sc.get(&head, (size_t)n + 1));
  O3G_TRY(sc.get(&hrank, (size_t)n + 1));
  O3G_TRY(sc.get(&start, (size_t)n + 1));
  k_uf_init<<<blocks(n), 256, 0, st>>>(n, parent, act);
  O3G_CUDA_TRY(cudaMemsetAsync(act + n, 0, sizeof(int), st));
  k_uf_edges<<<blocks(n), 256, 0, st>>>(n, off, sorted, parent, act);
  note_launch(2);
  O3G_TRY(exclusive_sum(sc, act, arank, n + 1));
  k_scatter_active<<<blocks(n), 256, 0, st>>>(n, parent, act, arank, akey, aval);
  note_launch(1);
  int na = 0;
  O3G_TRY(read_int(arank + n, &na, st));
  int bits = 1;
  while (bits < 31 && (1ll << bits) < (long long)n) ++bits;
  size_t tb = 0;
  O3G_CUDA_TRY(cub::DeviceRadixSort::SortPairs(nullptr, tb, akey, akey2, aval, aval2, na, 0, bits, st));
  void* tmp = nullptr;
  O3G_TRY(sc.get((char**)&tmp, tb));
  O3G_CUDA_TRY(cub::DeviceRadixSort::SortPairs(tmp, tb, akey, akey2, aval, aval2, na, 0, bits, st));
  k_group_heads<<<blocks((long long)na + 1), 256, 0, st>>>(arank + n, akey2, head);
  O3G_TRY(exclusive_sum(sc, head, hrank, na + 1));
  k_scatter_heads<<<blocks((long long)na + 1), 256, 0, st>>>(arank + n, head, hrank, start);
  note_launch(2);
  int ng = 0;
  O3G_TRY(read_int(hrank + na, &ng, st));

  unsigned char* erase = nullptr;
  O3G_TRY(sc.get(&erase, n));
  O3G_CUDA_TRY(cudaMemsetAsync(erase, 0, (size_t)n, st));
  MergeArgs a;
  a.ng = hrank + na; a.start = start; a.member = aval2; a.off = off; a.keys = sorted;
  a.x = x; a.y = y; a.z = z; a.sx = sx; a.sy = sy; a.sz = sz; a.r = r;
  a.erase = erase; a.meanstr = meanstr; a.overlap = overlap; a.threshold = threshold; a.adapt = adapt;
  if (ng > 0) {
    O3G_CUDA_TRY(cudaStreamWaitEvent(st, join.done, 0));
    k_merge_resolve<<<blocks(ng, 128), 128, 0, st>>>(a);
    note_launch(1);
  }

  // compaction of the survivors, in order
  int *keep = nullptr, *dst = nullptr;
  O3G_TRY(sc.get(&keep, (size_t)n + 1));
  O3G_TRY(sc.get(&dst, (size_t)n + 1));
  k_keep_flags<<<blocks((long long)n + 1), 256, 0, st>>>(n, erase, keep);
  O3G_TRY(exclusive_sum(sc, keep, dst, n + 1));
  int kept = 0;
  O3G_TRY(read_int(dst + n, &kept, st));
  if (kept < n) {
    float* buf = nullptr;
    O3G_TRY(sc.get(&buf, (size_t)7 * kept));
    Arr7 src{{x, y, z, sx, sy, sz, r}};
    Arr7 out;
    for (int c = 0; c < 7; ++c) out.p[c] = buf + (size_t)c * kept;
    k_compact<<<blocks(n), 256, 0, st>>>(n, keep, dst, src, out);
    note_launch(2);
    for (int c = 0; c < 7; ++c)
      O3G_CUDA_TRY(cudaMemcpyAsync(src.p[c], out.p[c], (size_t)kept * sizeof(float), cudaMemcpyDeviceToDevice, st));
  } else {
    note_launch(1);
  }
  O3G_CUDA_TRY(cudaGetLastError());
  O3G_TRY(check_err(err, st, "o3g_merge_close_particles: a device-side check failed (match count)"));
  *nremoved = n - kept;
  return O3G_OK;
}

}  // namespace
}  // namespace o3g

using namespace o3g;

extern "C" int32_t o3g_split_elongated(int32_t n, int32_t capacity, float* x, float* y, float* z, float* r,
                                       float* elong, float* sx, float* sy, float* sz, int32_t core_func,
                                       float particle_overlap, float threshold, int32_t* nsplit, void* stream) {
  if (nsplit) *nsplit = 0;
  if (n < 0 || capacity < n || !nsplit ||
      (n > 0 && (!x || !y || !z || !r || !elong || !sx || !sy || !sz)) ||
      (core_func != O3G_DIFFCORE_GAUSSIAN && core_func != O3G_DIFFCORE_COMPACTG) || !(particle_overlap > 0.0f)) {
    set_error("o3g_split_elongated: bad arguments (need 0 <= n <= capacity, arrays, a core type, overlap > 0)");
    return O3G_ERR_INVALID_ARG;
  }
  if (n == 0) return O3G_OK;
  int m = 0;
  const int32_t rc = split_run(n, capacity, x, y, z, r, elong, sx, sy, sz, core_func, particle_overlap, threshold,
                               &m, (cudaStream_t)stream);
  *nsplit = m;
  return rc;
}

extern "C" int32_t o3g_merge_close_particles(int32_t n, float* x, float* y, float* z, float* sx, float* sy,
                                             float* sz, float* r, float particle_overlap, float threshold,
                                             int32_t adapt_radii, int32_t* nremoved, void* stream) {
  if (nremoved) *nremoved = 0;
  if (n < 0 || !nremoved || (n > 0 && (!x || !y || !z || !sx || !sy || !sz || !r)) || !(particle_overlap > 0.0f)) {
    set_error("o3g_merge_close_particles: bad arguments (need n >= 0, arrays, overlap > 0)");
    return O3G_ERR_INVALID_ARG;
  }
  if (n == 0) return O3G_OK;
  return merge_run(n, x, y, z, sx, sy, sz, r, particle_overlap, threshold, adapt_radii != 0 ? 1 : 0, nremoved,
                   (cudaStream_t)stream);
}
