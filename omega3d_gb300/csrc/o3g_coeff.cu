// o3g_coeff.cu -- BEM influence-matrix block: panels_on_panels_coeff (Coefficients.h:169-447).
//
// Column (j*nunk + k) of the block holds the velocity induced by unit strength k of source
// panel j (k = 0: vortex sheet along x1, 1: along x2, 2: source sheet when nunk == 3),
// projected on target panel i's x1, x2 (and normal when nunk == 3) at rows i*nunk + l
// (Coefficients.h:221,283-289).  The block is written column-major with leading dimension
// `ld`, so it can be written straight into the full BEM matrix.  Self-influence entries of
// a block of a surface on itself are [0, 2pi; -2pi, 0] (+2pi source-source,
// Coefficients.h:414-436) and everything is scaled by 1/(4pi) (:443-447).
//
// Each (target i, source j) pair is one traversal of rkernel_2vs_2p (Kernels.h:1217-1315):
// the two centroids are compared against 4*(sqrt(sa)+sqrt(ta)) with the reference's
// operation order (no FMA) and, when too close, both panels split into 4 children (16
// child pairs, strength/16) down to maxlev.  The kernel is linear in the source strength,
// so the 2 or 3 unit strengths share one traversal: each leaf computes r3 and d once.
#include "o3g_common.cuh"

#include <algorithm>

namespace o3g {

constexpr int kCB = 128;                 // target panels per block == source panels per tile
constexpr int kCoeffMaxLev = 4;
constexpr int kCStack = 15 * kCoeffMaxLev + 1;

struct SrcRec {
  float4 c;   // centroid, sqrt(area)
  float4 s1;  // x1 * area, area
  float4 s2;  // x2 * area, -
};
struct TriG { float x0, y0, z0, x1, y1, z1, x2, y2, z2; };

__device__ __forceinline__ void cen(const TriG& t, float& cx, float& cy, float& cz) {
  cx = div3_rn(__fadd_rn(__fadd_rn(t.x0, t.x1), t.x2));
  cy = div3_rn(__fadd_rn(__fadd_rn(t.y0, t.y1), t.y2));
  cz = div3_rn(__fadd_rn(__fadd_rn(t.z0, t.z1), t.z2));
}
// |a - b| > thr as the reference decides it (the distance rounded to float: the correctly
// rounded square root of the rounded sum of rounded squares), with thr2 = thr * thr rounded.
// The correctly rounded square root is monotone and thr is a float, so the squared
// distance d2 decides whenever it is more than 2^-20 away from thr2 (relative): above,
// sqrt(d2) > thr (1 + 2^-22), more than half of thr's spacing (at most 2^-23 thr) beyond
// thr, so it rounds above thr; below, sqrt(d2) < thr and it rounds to thr at most.  Only
// the few pairs near the threshold take the square root.
__device__ __forceinline__ bool farther_rn(float ax, float ay, float az, float bx, float by, float bz, float thr,
                                           float thr2) {
  const float dx = __fsub_rn(ax, bx), dy = __fsub_rn(ay, by), dz = __fsub_rn(az, bz);
  const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
  if (d2 > __fmul_rn(thr2, 1.00000095367431640625f)) return true;    // 1 + 2^-20
  if (d2 < __fmul_rn(thr2, 0.99999904632568359375f)) return false;   // 1 - 2^-20
  return __fsqrt_rn(d2) > thr;
}

// singular leaf at target point t from a source point c with vortex strengths s1, s2 and
// source strength q (kernel_0vs_0p with sr = 0, Kernels.h:115-133); u[k] += r3 (s_k x d),
// u[2] += r3 q d
template <int NUNK>
__device__ __forceinline__ void leaf3(float tx, float ty, float tz, float cx, float cy, float cz, float s1x, float s1y,
                                      float s1z, float s2x, float s2y, float s2z, float q, float (*u)[3]) {
  const float dx = tx - cx, dy = ty - cy, dz = tz - cz;
  const float rs = rsqrtf(fmaf(dx, dx, fmaf(dy, dy, dz * dz)));
  const float r3 = rs * rs * rs;
  u[0][0] = fmaf(r3, dz * s1y - dy * s1z, u[0][0]);
  u[0][1] = fmaf(r3, dx * s1z - dz * s1x, u[0][1]);
  u[0][2] = fmaf(r3, dy * s1x - dx * s1y, u[0][2]);
  u[1][0] = fmaf(r3, dz * s2y - dy * s2z, u[1][0]);
  u[1][1] = fmaf(r3, dx * s2z - dz * s2x, u[1][1]);
  u[1][2] = fmaf(r3, dy * s2x - dx * s2y, u[1][2]);
  if (NUNK == 3) {
    const float rq = r3 * q;
    u[2][0] = fmaf(rq, dx, u[2][0]);
    u[2][1] = fmaf(rq, dy, u[2][1]);
    u[2][2] = fmaf(rq, dz, u[2][2]);
  }
}

// child c (0..3) of triangle p: corner/midpoint list {v0, m01, v1, m02, m12, v2}, children
// {0,1,3},{1,2,4},{1,4,3},{3,4,5} (Kernels.h:1292)
__device__ __forceinline__ TriG child(const TriG& p, int c) {
  const float m01x = 0.5f * (p.x0 + p.x1), m01y = 0.5f * (p.y0 + p.y1), m01z = 0.5f * (p.z0 + p.z1);
  const float m02x = 0.5f * (p.x0 + p.x2), m02y = 0.5f * (p.y0 + p.y2), m02z = 0.5f * (p.z0 + p.z2);
  const float m12x = 0.5f * (p.x1 + p.x2), m12y = 0.5f * (p.y1 + p.y2), m12z = 0.5f * (p.z1 + p.z2);
  if (c == 0) return TriG{p.x0, p.y0, p.z0, m01x, m01y, m01z, m02x, m02y, m02z};
  if (c == 1) return TriG{m01x, m01y, m01z, p.x1, p.y1, p.z1, m12x, m12y, m12z};
  if (c == 2) return TriG{m01x, m01y, m01z, m12x, m12y, m12z, m02x, m02y, m02z};
  return TriG{m02x, m02y, m02z, m12x, m12y, m12z, p.x2, p.y2, p.z2};
}
// the sub-triangle reached from `root` by the child indices in `path` (2 bits per level)
__device__ __forceinline__ TriG descend(const TriG& root, unsigned path, int lev) {
  TriG t = root;
  for (int l = 0; l < lev; ++l) t = child(t, (path >> (2 * l)) & 3u);
  return t;
}

// Depth-first pair subdivision in the reference's order (source child outer, target child
// inner).  A stack entry is (level, source path, target path) packed in 32 bits; the
// sub-triangles are rebuilt from the roots, which keeps the stack at 61 words.
template <int NUNK>
__device__ __noinline__ void pair_subdivide(const TriG& s0, const TriG& t0, float sa, float ta, float s1x, float s1y,
                                            float s1z, float s2x, float s2y, float s2z, float q, int maxlev,
                                            float (*u)[3]) {
  const float thr0 = __fmul_rn(__fadd_rn(__fsqrt_rn(sa), __fsqrt_rn(ta)), 4.0f);
  unsigned st[kCStack];
  int sp = 0;
  auto push = [&](unsigned code) {
    const unsigned lev = code & 7u, sps = (code >> 3) & 0xffu, tps = (code >> 11) & 0xffu;
    for (int a = 3; a >= 0; --a)
      for (int b = 3; b >= 0; --b)
        st[sp++] = (lev + 1) | ((sps | ((unsigned)a << (2 * lev))) << 3) | ((tps | ((unsigned)b << (2 * lev))) << 11);
  };
  push(0u);
  while (sp > 0) {
    const unsigned code = st[--sp];
    const int lev = (int)(code & 7u);
    const TriG s = descend(s0, (code >> 3) & 0xffu, lev);
    const TriG t = descend(t0, (code >> 11) & 0xffu, lev);
    const float f4 = __int_as_float((127 - 2 * lev) << 23);   // 0.25^lev: the children's area factor
    float scx, scy, scz, tcx, tcy, tcz;
    cen(s, scx, scy, scz);
    cen(t, tcx, tcy, tcz);
    // 4 (sqrt(sa 0.25^lev) + sqrt(ta 0.25^lev)) = thr0 0.5^lev exactly (scaling by powers of
    // two commutes with the correctly rounded sqrt and add)
    const float thr = __fmul_rn(thr0, __int_as_float((127 - lev) << 23));
    if (lev >= maxlev || farther_rn(tcx, tcy, tcz, scx, scy, scz, thr, __fmul_rn(thr, thr))) {
      const float f = f4 * f4;   // 0.0625^lev (Kernels.h:1275-1278)
      leaf3<NUNK>(tcx, tcy, tcz, scx, scy, scz, s1x * f, s1y * f, s1z * f, s2x * f, s2y * f, s2z * f, q * f, u);
    } else if (sp + 16 <= kCStack) {
      push(code);
    }
  }
}

__global__ void k_pack_src_panels(int np, const float* __restrict__ x, const float* __restrict__ y,
                                  const float* __restrict__ z, const uint32_t* __restrict__ idx,
                                  const float* __restrict__ area, const float* __restrict__ x1x,
                                  const float* __restrict__ x1y, const float* __restrict__ x1z,
                                  const float* __restrict__ x2x, const float* __restrict__ x2y,
                                  const float* __restrict__ x2z, int np_pad, SrcRec* rec, TriG* tri) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= np_pad) return;
  SrcRec r;
  TriG t;
  if (j < np) {
    const uint32_t p0 = idx[3 * (size_t)j], p1 = idx[3 * (size_t)j + 1], p2 = idx[3 * (size_t)j + 2];
    t = TriG{x[p0], y[p0], z[p0], x[p1], y[p1], z[p1], x[p2], y[p2], z[p2]};
    float cx, cy, cz;
    cen(t, cx, cy, cz);
    const float sa = area[j];
    r.c = make_float4(cx, cy, cz, __fsqrt_rn(sa));
    r.s1 = make_float4(__fmul_rn(x1x[j], sa), __fmul_rn(x1y[j], sa), __fmul_rn(x1z[j], sa), sa);
    r.s2 = make_float4(__fmul_rn(x2x[j], sa), __fmul_rn(x2y[j], sa), __fmul_rn(x2z[j], sa), 0.f);
  } else {
    t = TriG{0, 0, 0, 0, 0, 0, 0, 0, 0};
    r.c = make_float4(1.0e18f, 1.0e18f, 1.0e18f, 0.f);
    r.s1 = make_float4(0.f, 0.f, 0.f, 0.f);
    r.s2 = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  rec[j] = r;
  tri[j] = t;
}

struct NearList {
  uint2* pairs;        // (target i, source j) of pairs that need subdivision
  unsigned* count;
  unsigned cap;        // 0: subdivide in the thread that found the pair
};

template <int NUNK>
__global__ void __launch_bounds__(kCB) k_coeff(const SrcRec* __restrict__ srec, const TriG* __restrict__ stri, int snp,
                                               const TriG* __restrict__ ttri, const float* __restrict__ tarea,
                                               const float* __restrict__ t1x, const float* __restrict__ t1y,
                                               const float* __restrict__ t1z, const float* __restrict__ t2x,
                                               const float* __restrict__ t2y, const float* __restrict__ t2z,
                                               const float* __restrict__ tnx, const float* __restrict__ tny,
                                               const float* __restrict__ tnz, int tnp, int is_self, int maxlev,
                                               float* __restrict__ coeff, long long ld, int vec2, NearList nl) {
  __shared__ SrcRec sr[kCB];
  // per warp, one column's entries of its 32 targets, for coalesced stores (NUNK == 3)
  __shared__ float ob[NUNK == 3 ? kCB / 32 : 1][NUNK == 3 ? 3 * 3 * 32 : 1];
  const int i = blockIdx.x * kCB + threadIdx.x;
  const int j0 = blockIdx.y * kCB;
  sr[threadIdx.x] = srec[j0 + threadIdx.x];
  __syncthreads();
  // every lane of a warp stays in the loop (the near-pair list is claimed per warp); lanes
  // past the last target compute on a copy of it and write nothing
  const bool valid = i < tnp;
  const int ic = valid ? i : tnp - 1;
  const TriG tt = ttri[ic];
  float tcx, tcy, tcz;
  cen(tt, tcx, tcy, tcz);
  const float ta = tarea[ic];
  const float sqta = __fsqrt_rn(ta);
  const float b[3][3] = {{t1x[ic], t1y[ic], t1z[ic]}, {t2x[ic], t2y[ic], t2z[ic]},
                         {NUNK == 3 ? tnx[ic] : 0.f, NUNK == 3 ? tny[ic] : 0.f, NUNK == 3 ? tnz[ic] : 0.f}};
  const float fac = (float)(1.0 / (4.0 * 3.14159265358979323846));
  const int lane = threadIdx.x & 31;
  const int jend = min(kCB, snp - j0);
  for (int jj = 0; jj < jend; ++jj) {
    const int j = j0 + jj;
    const bool self = is_self && j == i;
    const SrcRec s = sr[jj];
    const float thr = __fmul_rn(__fadd_rn(s.c.w, sqta), 4.0f);
    const bool far = maxlev == 0 || farther_rn(tcx, tcy, tcz, s.c.x, s.c.y, s.c.z, thr, __fmul_rn(thr, thr));
    const bool near = valid && !self && !far;
    bool listed = false;
    if (nl.cap > 0) {
      // one atomic per warp for its near pairs of this source
      const unsigned m = __ballot_sync(0xffffffffu, near);
      if (m) {
        unsigned base = 0;
        if (lane == __ffs(m) - 1) base = atomicAdd(nl.count, (unsigned)__popc(m));
        base = __shfl_sync(0xffffffffu, base, __ffs(m) - 1);
        const unsigned slot = base + (unsigned)__popc(m & ((1u << lane) - 1u));
        if (near && slot < nl.cap) {
          nl.pairs[slot] = make_uint2((unsigned)i, (unsigned)j);
          listed = true;   // written by k_coeff_near
        }
      }
    }
    // the block entries v[k][l] (source unknown k, target unknown l); the listed pairs get
    // 0 here and their values from k_coeff_near, which runs after this kernel
    float v[NUNK][NUNK];
#pragma unroll
    for (int k = 0; k < NUNK; ++k)
#pragma unroll
      for (int l = 0; l < NUNK; ++l) v[k][l] = 0.f;
    if (self) {
      // Coefficients.h:414-436, then the 1/(4 pi) scale of :443-447, both in float
      const float tp = (float)(2.0 * 3.14159265358979323846);
      v[0][0] = 0.f * fac;
      v[0][1] = tp * fac;
      v[1][0] = -tp * fac;
      if (NUNK == 3) v[2][2] = tp * fac;
    } else if (valid && !listed) {
      // two accumulators: the one handed to the out-of-line subdivision lives in local
      // memory, the far pairs' one stays in registers
      auto project = [&](const float (*u)[3]) {
#pragma unroll
        for (int k = 0; k < NUNK; ++k)
#pragma unroll
          for (int l = 0; l < NUNK; ++l)
            v[k][l] = (u[k][0] * b[l][0] + u[k][1] * b[l][1] + u[k][2] * b[l][2]) * fac;
      };
      if (far) {
        float u[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
        leaf3<NUNK>(tcx, tcy, tcz, s.c.x, s.c.y, s.c.z, s.s1.x, s.s1.y, s.s1.z, s.s2.x, s.s2.y, s.s2.z, s.s1.w, u);
        project(u);
      } else {
        float us[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
        pair_subdivide<NUNK>(stri[j], tt, s.s1.w, ta, s.s1.x, s.s1.y, s.s1.z, s.s2.x, s.s2.y, s.s2.z, s.s1.w,
                             maxlev, us);
        project(us);
      }
    }
    // column j NUNK + k holds rows i NUNK + l: a warp's 32 targets are 32 NUNK consecutive
    // floats of each column
    float* col = coeff + (size_t)j * NUNK * (size_t)ld;
    if (NUNK == 2 && vec2) {
      // 8-byte aligned rows: one float2 per column, each warp store 256 contiguous bytes
      if (valid) {
#pragma unroll
        for (int k = 0; k < NUNK; ++k)
          *reinterpret_cast<float2*>(col + (size_t)k * ld + (size_t)i * 2) = make_float2(v[k][0], v[k][1]);
      }
    } else if (NUNK == 3) {
      // through shared memory, so that each warp store covers 128 contiguous bytes
      float* w = ob[threadIdx.x >> 5];
      const int i0 = i - lane;
#pragma unroll
      for (int k = 0; k < NUNK; ++k)
#pragma unroll
        for (int l = 0; l < NUNK; ++l) w[k * 96 + lane * 3 + l] = v[k][l];
      __syncwarp();
      const int rows = min(32, tnp - i0) * 3;
#pragma unroll
      for (int k = 0; k < NUNK; ++k)
#pragma unroll
        for (int e = lane; e < 96; e += 32)
          if (e < rows) col[(size_t)k * ld + (size_t)i0 * 3 + e] = w[k * 96 + e];
      __syncwarp();
    } else if (valid) {
#pragma unroll
      for (int k = 0; k < NUNK; ++k)
#pragma unroll
        for (int l = 0; l < NUNK; ++l) col[(size_t)k * ld + (size_t)i * NUNK + l] = v[k][l];
    }
  }
}

// One warp per listed pair (maxlev <= 3): the subdivision tree is expanded level by level.
// Level 1 has 16 child pairs (source child a outer, target child b inner, one lane each);
// every child pair that is neither well separated nor at maxlev contributes 16 pairs to the
// next level, kept in a per-warp list in shared memory in enumeration order.  Leaves are
// summed per lane and reduced across the warp in a fixed order.
//
// A pair at level L needs only the centroids of one level-L sub-triangle of each panel,
// and every pair of a level shares them: the warp builds the 4^L sub-triangles of both
// panels once per level (each from its stored parent by child(), the same operations as a
// descent from the root) and keeps their centroids in shared memory, indexed by the
// path (2 bits per level, level 1 in the low bits).  A pair then costs six shared loads,
// the distance test and the leaf.
constexpr int kNearWarps = 4;
struct NearShared {
  float tri[2][20][9];   // [source, target][level 1: 0..3, level 2: 4..19] sub-triangles
  float cen[2][84][3];   // [source, target][level 1: 0..3, level 2: 4..19, level 3: 20..83]
};

__device__ __forceinline__ void store_tri(float* d, const TriG& t) {
  d[0] = t.x0; d[1] = t.y0; d[2] = t.z0; d[3] = t.x1; d[4] = t.y1; d[5] = t.z1; d[6] = t.x2; d[7] = t.y2; d[8] = t.z2;
}
__device__ __forceinline__ TriG load_tri(const float* d) {
  return TriG{d[0], d[1], d[2], d[3], d[4], d[5], d[6], d[7], d[8]};
}
__device__ __forceinline__ void store_cen(float* d, const TriG& t) {
  float cx, cy, cz;
  cen(t, cx, cy, cz);
  d[0] = cx; d[1] = cy; d[2] = cz;
}

// the level-lev sub-triangles of both panels (and their centroids) into sh; lev 1..3
__device__ __forceinline__ void build_level(NearShared& sh, const TriG& S0, const TriG& T0, int lev, int lane) {
  if (lev == 1) {
    if (lane < 8) {
      const int side = lane >> 2, c = lane & 3;
      const TriG t = child(side ? T0 : S0, c);
      store_tri(sh.tri[side][c], t);
      store_cen(sh.cen[side][c], t);
    }
  } else if (lev == 2) {
    // path p = (level-2 child << 2) | level-1 child
    const int side = lane >> 4, p = lane & 15;
    const TriG t = child(load_tri(sh.tri[side][p & 3]), p >> 2);
    store_tri(sh.tri[side][4 + p], t);
    store_cen(sh.cen[side][4 + p], t);
  } else {
#pragma unroll 1
    for (int e = lane; e < 128; e += 32) {
      const int side = e >> 6, p = e & 63;
      store_cen(sh.cen[side][20 + p], child(load_tri(sh.tri[side][4 + (p & 15)]), p >> 4));
    }
  }
  __syncwarp();
}

template <int NUNK>
__global__ void __launch_bounds__(32 * kNearWarps) k_coeff_near(const SrcRec* __restrict__ srec,
                                                               const TriG* __restrict__ stri,
                                                               const TriG* __restrict__ ttri,
                                                               const float* __restrict__ tarea,
                                                               const float* __restrict__ t1x,
                                                               const float* __restrict__ t1y,
                                                               const float* __restrict__ t1z,
                                                               const float* __restrict__ t2x,
                                                               const float* __restrict__ t2y,
                                                               const float* __restrict__ t2z,
                                                               const float* __restrict__ tnx,
                                                               const float* __restrict__ tny,
                                                               const float* __restrict__ tnz, int maxlev,
                                                               float* __restrict__ coeff, long long ld, NearList nl) {
  __shared__ unsigned lst[kNearWarps][2][256];
  __shared__ NearShared shw[kNearWarps];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  NearShared& sh = shw[warp];
  const unsigned total = min(*nl.count, nl.cap);
  const float fac = (float)(1.0 / (4.0 * 3.14159265358979323846));
  for (unsigned p = blockIdx.x * kNearWarps + warp; p < total; p += gridDim.x * kNearWarps) {
    const uint2 ij = nl.pairs[p];
    const int i = (int)ij.x, j = (int)ij.y;
    const SrcRec s = srec[j];
    const TriG S0 = stri[j], T0 = ttri[i];
    const float sa = s.s1.w, ta = tarea[i];
    // the level-lev threshold is thr0 0.5^lev exactly (as in pair_subdivide)
    const float thr0 = __fmul_rn(__fadd_rn(__fsqrt_rn(sa), __fsqrt_rn(ta)), 4.0f);
    float u[3][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
    // level L items: (parent index in the level L-1 list, child 0..15); codes keep the
    // source path in bits 0..7 and the target path in bits 8..15 (2 bits per level)
    int nparent = 1;
    for (int lev = 1; lev <= maxlev; ++lev) {
      build_level(sh, S0, T0, lev, lane);
      const int nitems = nparent * 16;
      const int cur = lev & 1, prev = cur ^ 1;
      int nnext = 0;
      const float f4 = __int_as_float((127 - 2 * lev) << 23);
      const float f = f4 * f4;   // 0.0625^lev (Kernels.h:1275-1278)
      const float thr = __fmul_rn(thr0, __int_as_float((127 - lev) << 23));
      const float thr2 = __fmul_rn(thr, thr);
      const int off = lev == 1 ? 0 : (lev == 2 ? 4 : 20);   // first centroid of the level
      for (int base = 0; base < nitems; base += 32) {
        const int k = base + lane;
        bool expand = false;
        unsigned code = 0;
        if (k < nitems) {
          const unsigned pc = lev == 1 ? 0u : lst[warp][prev][k >> 4];
          const unsigned a = (unsigned)((k & 15) >> 2), b = (unsigned)(k & 3);
          const unsigned sp = (pc & 0xffu) | (a << (2 * (lev - 1)));
          const unsigned tp = ((pc >> 8) & 0xffu) | (b << (2 * (lev - 1)));
          code = sp | (tp << 8);
          const float* sc = sh.cen[0][off + sp];
          const float* tc = sh.cen[1][off + tp];
          const float scx = sc[0], scy = sc[1], scz = sc[2];
          const float tcx = tc[0], tcy = tc[1], tcz = tc[2];
          if (lev >= maxlev || farther_rn(tcx, tcy, tcz, scx, scy, scz, thr, thr2)) {
            leaf3<NUNK>(tcx, tcy, tcz, scx, scy, scz, s.s1.x * f, s.s1.y * f, s.s1.z * f, s.s2.x * f, s.s2.y * f,
                        s.s2.z * f, s.s1.w * f, u);
          } else {
            expand = true;
          }
        }
        const unsigned m = __ballot_sync(0xffffffffu, expand);
        if (expand) lst[warp][cur][nnext + __popc(m & ((1u << lane) - 1u))] = code;
        nnext += __popc(m);
      }
      __syncwarp();
      nparent = nnext;
      if (nparent == 0) break;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) u[k][c] += __shfl_xor_sync(0xffffffffu, u[k][c], o);
    if (lane < NUNK * NUNK) {
      const int k = lane / NUNK, l = lane % NUNK;
      float bx, by, bz;
      if (l == 0) { bx = t1x[i]; by = t1y[i]; bz = t1z[i]; }
      else if (l == 1) { bx = t2x[i]; by = t2y[i]; bz = t2z[i]; }
      else { bx = tnx[i]; by = tny[i]; bz = tnz[i]; }
      const float ux = k == 0 ? u[0][0] : (k == 1 ? u[1][0] : u[2][0]);
      const float uy = k == 0 ? u[0][1] : (k == 1 ? u[1][1] : u[2][1]);
      const float uz = k == 0 ? u[0][2] : (k == 1 ? u[1][2] : u[2][2]);
      float* col = coeff + (size_t)j * NUNK * (size_t)ld + (size_t)i * NUNK;
      col[(size_t)k * ld + l] = (ux * bx + uy * by + uz * bz) * fac;
    }
    __syncwarp();
  }
}

__global__ void k_pack_tri(int np, const float* __restrict__ x, const float* __restrict__ y,
                           const float* __restrict__ z, const uint32_t* __restrict__ idx, TriG* tri) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= np) return;
  const uint32_t p0 = idx[3 * (size_t)j], p1 = idx[3 * (size_t)j + 1], p2 = idx[3 * (size_t)j + 2];
  tri[j] = TriG{x[p0], y[p0], z[p0], x[p1], y[p1], z[p1], x[p2], y[p2], z[p2]};
}

}  // namespace o3g

using namespace o3g;

static bool surf_ok(const o3g_surface_t* s, bool need_norm) {
  if (!s || s->nn < 0 || s->np < 0) return false;
  if (s->np == 0) return true;
  if (!s->x || !s->y || !s->z || !s->idx || !s->area || !s->x1x || !s->x1y || !s->x1z || !s->x2x || !s->x2y || !s->x2z)
    return false;
  if (need_norm && (!s->nx || !s->ny || !s->nz)) return false;
  return true;
}

extern "C" int32_t o3g_panels_on_panels_coeff(int32_t maxlev, int32_t nunk, int32_t is_self, const o3g_surface_t* src,
                                              const o3g_surface_t* targ, float* coeffs, int64_t ld, void* stream) {
  if (maxlev < 0 || maxlev > kCoeffMaxLev || (nunk != 2 && nunk != 3) || !surf_ok(src, false) ||
      !surf_ok(targ, nunk == 3) || !coeffs) {
    set_error("panels_on_panels_coeff: bad maxlev (0..4), nunk (2|3), surface or output pointer");
    return O3G_ERR_INVALID_ARG;
  }
  if (ld < (int64_t)targ->np * nunk) {
    set_error("panels_on_panels_coeff: leading dimension smaller than the block's rows");
    return O3G_ERR_INVALID_ARG;
  }
  if (is_self && src->np != targ->np) {
    set_error("panels_on_panels_coeff: is_self needs the same panel count");
    return O3G_ERR_INVALID_ARG;
  }
  if (src->np == 0 || targ->np == 0) return O3G_OK;
  DeviceFacts df;
  O3G_TRY(device_facts(&df));
  cudaStream_t st = (cudaStream_t)stream;
  const int snp = src->np, tnp = targ->np;
  const int sblocks = (snp + kCB - 1) / kCB, snp_pad = sblocks * kCB;
  // near-pair list for the warp-cooperative subdivision (maxlev <= 3; deeper trees stay in-thread)
  const unsigned cap = maxlev <= 3 ? (unsigned)std::min<long long>((long long)snp * tnp, 512LL * (tnp > snp ? tnp : snp))
                                   : 0u;
  size_t bytes = align_up((size_t)snp_pad * sizeof(SrcRec)) + align_up((size_t)snp_pad * sizeof(TriG)) +
                 align_up((size_t)tnp * sizeof(TriG)) + align_up(sizeof(unsigned)) + align_up((size_t)cap * 8);
  Workspace* ws = nullptr;
  O3G_TRY(workspace_get(st, bytes, &ws));
  Carve cv(ws->base);
  SrcRec* srec = cv.take<SrcRec>(snp_pad);
  TriG* stri = cv.take<TriG>(snp_pad);
  TriG* ttri = cv.take<TriG>(tnp);
  NearList nl;
  nl.count = cv.take<unsigned>(1);
  nl.pairs = cv.take<uint2>(cap > 0 ? cap : 1);
  nl.cap = cap;
  O3G_CUDA_TRY(cudaMemsetAsync(nl.count, 0, sizeof(unsigned), st));
  k_pack_src_panels<<<(snp_pad + 255) / 256, 256, 0, st>>>(snp, src->x, src->y, src->z, src->idx, src->area, src->x1x,
                                                          src->x1y, src->x1z, src->x2x, src->x2y, src->x2z, snp_pad,
                                                          srec, stri);
  k_pack_tri<<<(tnp + 255) / 256, 256, 0, st>>>(tnp, targ->x, targ->y, targ->z, targ->idx, ttri);
  note_launch(2);
  dim3 grid((tnp + kCB - 1) / kCB, sblocks);
  KernelTimer& tm = thread_timer();
  tm.begin(st);
  const int nearblocks = 8 * df.num_sms;
  // float2 stores when every row pair (2 i, 2 i + 1) of every column is 8-byte aligned
  const int vec2 = nunk == 2 && ((uintptr_t)coeffs & 7u) == 0 && (ld & 1) == 0;
  if (nunk == 2) {
    k_coeff<2><<<grid, kCB, 0, st>>>(srec, stri, snp, ttri, targ->area, targ->x1x, targ->x1y, targ->x1z, targ->x2x,
                                     targ->x2y, targ->x2z, nullptr, nullptr, nullptr, tnp, is_self, maxlev, coeffs, ld,
                                     vec2, nl);
    if (cap > 0)
      k_coeff_near<2><<<nearblocks, 32 * kNearWarps, 0, st>>>(srec, stri, ttri, targ->area, targ->x1x, targ->x1y,
                                                              targ->x1z, targ->x2x, targ->x2y, targ->x2z, nullptr,
                                                              nullptr, nullptr, maxlev, coeffs, ld, nl);
  } else {
    k_coeff<3><<<grid, kCB, 0, st>>>(srec, stri, snp, ttri, targ->area, targ->x1x, targ->x1y, targ->x1z, targ->x2x,
                                     targ->x2y, targ->x2z, targ->nx, targ->ny, targ->nz, tnp, is_self, maxlev, coeffs,
                                     ld, 0, nl);
    if (cap > 0)
      k_coeff_near<3><<<nearblocks, 32 * kNearWarps, 0, st>>>(srec, stri, ttri, targ->area, targ->x1x, targ->x1y,
                                                              targ->x1z, targ->x2x, targ->x2y, targ->x2z, targ->nx,
                                                              targ->ny, targ->nz, maxlev, coeffs, ld, nl);
  }
  note_launch(cap > 0 ? 2 : 1);
  tm.end(st);
  O3G_CUDA_TRY(cudaGetLastError());
  return O3G_OK;
}
