// o3g_pair_impl.cuh -- particle/field-point Biot-Savart pair sums (points_affect_points).
//
// Data layout in HBM (inside the per-stream workspace):
//   spos[ns_pad] : float4 (x, y, z, core parameter of sr)      16 B / source
//   sstr[ns_pad] : float4 (sx, sy, sz, sr)                     16 B / source
//   tpos[nt_pad] : float4 (x, y, z, core parameter of tr or 0) 16 B / target
//   (double4 for the FP64 mode).  Padding sources have zero strength and core parameter 1
//   (as the reference's Vc padding, Influence.h:232-238) and sit at (1e9, 1e9, 1e9): every
//   core and the singular far-field loop give finite r3 and bbb there (d^4 = 9e36 stays
//   below the float range), so with zero strength they add exactly zero, also to a target
//   at the origin.
//
// Kernel k_pair: a block of kBlock threads owns kBlock*TPT targets; each warp owns a
// contiguous run of 32*TPT of them (lane l holds targets l, l+32, ... so loads and stores
// coalesce) and sweeps a contiguous range of source tiles.  Each tile of kBlock sources is staged in shared memory and read by
// every thread as a broadcast.  When the targets alone cannot fill the GPU, the source
// range is split across blockIdx.y and the per-split partial sums go to scratch,
// reduced afterwards in a fixed order (deterministic, k_reduce).
//
// Cores with distance branches (Gaussian, compact exponential) sweep Morton-ordered
// sources and targets.  For every (warp's targets, half tile of kHalf sources) the
// bounding boxes decide whether all of the pairs lie beyond the core's far-field
// threshold; such halves run the branch-free singular loop (r3 = 1/d^3, bbb = -3/d^5),
// the others the full core.  The decision is uniform over the warp, so its lanes never
// diverge on it.
#pragma once

#include "o3g_common.cuh"
#include "o3g_sort.cuh"

namespace o3g {

constexpr int kBlock = 128;  // threads per block == sources per shared tile
constexpr int kHalf = 64;    // sources per far-field classification unit (two per tile)

enum { MODE_PLAIN = 0, MODE_COMP = 1, MODE_FP64 = 2, MODE_DS = 3 };
enum { CORE_SING = 5 };      // internal: singular far-field kernel (cst ignored)

}  // namespace o3g
#include "o3g_ds.cuh"
namespace o3g {

// compensated (Fast2Sum-folded) sums: the COMPENSATED and the accurate mode
template <int MODE> struct SumComp { static constexpr bool value = (MODE == MODE_COMP || MODE == MODE_DS); };

template <class T, class O> struct PairArgs {
  const V4<T>* spos;
  const V4<T>* sstr;
  int ntiles;                // source tiles of kBlock sources
  int tiles_per_split;       // tiles swept by one block
  const V4<T>* tpos;
  int nt;                    // real targets
  int nt_pad;                // padded targets (multiple of kBlock*TPT)
  T* partial;                // [nsplit][ncomp * (COMP ? 2 : 1)][nt_pad] or nullptr
  OutPtrs<O> out;            // accumulated into when partial == nullptr
  const uint32_t* tperm;     // sorted target k -> caller's index, or nullptr
  const float4* tile_lo;     // per half tile: (min x, min y, min z, max core param)
  const float4* tile_hi;     // per half tile: (max x, max y, max z, -)
};

// one pair, velocity + gradient.  a[0..2] velocity, a[3..11] gradient sums of
// bbb * d (x) (s x d) in the reference order, a[12..14] = sum r3 * s (folded into the
// antisymmetric gradient terms by fold_grads, Kernels.h:184-192).
template <int C, bool ACC, bool HAVE_TR, class T>
__device__ __forceinline__ void pair_g(const V4<T>& t, const V4<T>& s, const V4<T>& w, T* a,
                                       const float* gtab = nullptr) {
  const T dx = t.x - s.x;
  const T dy = t.y - s.y;
  const T dz = t.z - s.z;
  T r3, bbb;
  if (C == CORE_SING) {
    const T r2 = fma(dx, dx, fma(dy, dy, dz * dz));
    const T rs = rsq<ACC>(r2);
    const T rs2 = rs * rs;
    r3 = rs2 * rs;
    bbb = T(-3.0) * r3 * rs2;
  } else {
    const T cst = HAVE_TR ? (s.w + t.w) : s.w;
    core_g<C, ACC, T>(dx, dy, dz, cst, r3, bbb, gtab);
  }
  T cx = dz * w.y - dy * w.z;
  T cy = dx * w.z - dz * w.x;
  T cz = dy * w.x - dx * w.y;
  a[0] = fma(r3, cx, a[0]);
  a[1] = fma(r3, cy, a[1]);
  a[2] = fma(r3, cz, a[2]);
  cx *= bbb;
  cy *= bbb;
  cz *= bbb;
  a[3] = fma(dx, cx, a[3]);
  a[4] = fma(dx, cy, a[4]);
  a[5] = fma(dx, cz, a[5]);
  a[6] = fma(dy, cx, a[6]);
  a[7] = fma(dy, cy, a[7]);
  a[8] = fma(dy, cz, a[8]);
  a[9] = fma(dz, cx, a[9]);
  a[10] = fma(dz, cy, a[10]);
  a[11] = fma(dz, cz, a[11]);
  a[12] = fma(r3, w.x, a[12]);
  a[13] = fma(r3, w.y, a[13]);
  a[14] = fma(r3, w.z, a[14]);
}

// velocity only
template <int C, bool ACC, bool HAVE_TR, class T>
__device__ __forceinline__ void pair_v(const V4<T>& t, const V4<T>& s, const V4<T>& w, T* a,
                                       const float* gtab = nullptr) {
  const T dx = t.x - s.x;
  const T dy = t.y - s.y;
  const T dz = t.z - s.z;
  T r3;
  if (C == CORE_SING) {
    const T rs = rsq<ACC>(fma(dx, dx, fma(dy, dy, dz * dz)));
    r3 = rs * rs * rs;
  } else {
    const T cst = HAVE_TR ? (s.w + t.w) : s.w;
    r3 = core_v<C, ACC, T>(dx, dy, dz, cst, gtab);
  }
  a[0] = fma(r3, dz * w.y - dy * w.z, a[0]);
  a[1] = fma(r3, dx * w.z - dz * w.x, a[1]);
  a[2] = fma(r3, dy * w.x - dx * w.y, a[2]);
}

// The accurate mode's pair (o3g_ds.cuh): separation, d^2, core and cross product in
// double-single; the velocity terms go unrounded into double-single running sums (a[0..2]
// and their low parts a[15..17]); the gradient terms from the core rounded to float.  The
// radii come raw: s.w of the strength record and t.w of the target record.
template <int C, bool HAVE_TR>
__device__ __forceinline__ void pair_g_ds(const V4<float>& t, const V4<float>& s, const V4<float>& w, float* a) {
  const dsf dx = ds_two_sum(t.x, -s.x);
  const dsf dy = ds_two_sum(t.y, -s.y);
  const dsf dz = ds_two_sum(t.z, -s.z);
  const dsf d2 = ds_add(ds_add(ds_sq(dx), ds_sq(dy)), ds_sq(dz));
  dsf r3;
  float bbb;
  core_ds<C, true>(d2, w.w, HAVE_TR ? t.w : 0.f, r3, bbb);
  const dsf cx = ds_cross(dz, w.y, dy, w.z);
  const dsf cy = ds_cross(dx, w.z, dz, w.x);
  const dsf cz = ds_cross(dy, w.x, dx, w.y);
  ds_accum(a[0], a[15], r3, cx);
  ds_accum(a[1], a[16], r3, cy);
  ds_accum(a[2], a[17], r3, cz);
  const float bx = __fmul_rn(__fadd_rn(cx.h, cx.l), bbb);
  const float by = __fmul_rn(__fadd_rn(cy.h, cy.l), bbb);
  const float bz = __fmul_rn(__fadd_rn(cz.h, cz.l), bbb);
  const float ex = dx.h, ey = dy.h, ez = dz.h;
  a[3] = fmaf(ex, bx, a[3]);
  a[4] = fmaf(ex, by, a[4]);
  a[5] = fmaf(ex, bz, a[5]);
  a[6] = fmaf(ey, bx, a[6]);
  a[7] = fmaf(ey, by, a[7]);
  a[8] = fmaf(ey, bz, a[8]);
  a[9] = fmaf(ez, bx, a[9]);
  a[10] = fmaf(ez, by, a[10]);
  a[11] = fmaf(ez, bz, a[11]);
  const float r3f = ds_round(r3);
  a[12] = fmaf(r3f, w.x, a[12]);
  a[13] = fmaf(r3f, w.y, a[13]);
  a[14] = fmaf(r3f, w.z, a[14]);
}
template <int C, bool HAVE_TR>
__device__ __forceinline__ void pair_v_ds(const V4<float>& t, const V4<float>& s, const V4<float>& w, float* a) {
  const dsf dx = ds_two_sum(t.x, -s.x);
  const dsf dy = ds_two_sum(t.y, -s.y);
  const dsf dz = ds_two_sum(t.z, -s.z);
  const dsf d2 = ds_add(ds_add(ds_sq(dx), ds_sq(dy)), ds_sq(dz));
  dsf r3;
  float bbb;
  core_ds<C, false>(d2, w.w, HAVE_TR ? t.w : 0.f, r3, bbb);
  ds_accum(a[0], a[3], r3, ds_cross(dz, w.y, dy, w.z));
  ds_accum(a[1], a[4], r3, ds_cross(dx, w.z, dz, w.x));
  ds_accum(a[2], a[5], r3, ds_cross(dy, w.x, dx, w.y));
}

// a[12..14] -> antisymmetric gradient terms: tvx += sz r3, twx -= sy r3, tuy -= sz r3,
// twy += sx r3, tuz += sy r3, tvz -= sx r3 (Kernels.h:185-191)
template <class T>
__device__ __forceinline__ void fold_grads(T* a) {
  a[4] += a[14];
  a[5] -= a[13];
  a[6] -= a[14];
  a[8] += a[12];
  a[9] += a[13];
  a[10] -= a[12];
}

// Sweep the staged tile (kBlock sources in shared memory) for TPT targets.  In the
// compensated mode the plain partial of every FOLD sources is folded into (hi, lo) with
// Fast2Sum.
template <int C, int MODE, bool GRADS, bool HAVE_TR, int TPT, class T, int NA, int NC, int NH, int NS = kBlock>
__device__ __forceinline__ void sweep_tile(const V4<T>* sp, const V4<T>* sw, const V4<T>* tp, T (*acc)[NA],
                                           float (*hi)[NH], float (*lo)[NH], const float* gtab = nullptr) {
  constexpr bool ACC = (MODE == MODE_COMP);
  constexpr bool SUMC = SumComp<MODE>::value;
  constexpr int FOLD = SUMC ? 16 : NS;
#pragma unroll 1
  for (int j0 = 0; j0 < NS; j0 += FOLD) {
#pragma unroll 4
    for (int j = j0; j < j0 + FOLD; ++j) {
      const V4<T> s = sp[j];
      const V4<T> w = sw[j];
#pragma unroll
      for (int k = 0; k < TPT; ++k) {
        if constexpr (MODE == MODE_DS) {
          if (GRADS) pair_g_ds<C, HAVE_TR>(tp[k], s, w, acc[k]);
          else       pair_v_ds<C, HAVE_TR>(tp[k], s, w, acc[k]);
        } else {
          if (GRADS) pair_g<C, ACC, HAVE_TR, T>(tp[k], s, w, acc[k], gtab);
          else       pair_v<C, ACC, HAVE_TR, T>(tp[k], s, w, acc[k], gtab);
        }
      }
    }
    if (SUMC) {
#pragma unroll
      for (int k = 0; k < TPT; ++k) {
        if (GRADS) fold_grads(acc[k]);
#pragma unroll
        for (int c = 0; c < NC; ++c) {
          float s, e;
          if constexpr (MODE == MODE_DS) {
            // two-sum: exact in any order (a running sum that passes near zero while the
            // partials are large would otherwise lose the partial's rounding)
            const dsf t2 = ds_two_sum(hi[k][c], (float)acc[k][c]);
            s = t2.h;
            e = t2.l;
          } else {
            // Fast2Sum: exact error term when |hi| >= |partial|, the usual case once a few
            // folds have accumulated; otherwise that fold loses at most its own rounding
            s = hi[k][c] + (float)acc[k][c];
            e = (float)acc[k][c] - (s - hi[k][c]);
          }
          hi[k][c] = s;
          lo[k][c] += e;
        }
        if constexpr (MODE == MODE_DS) {
          // the velocity sums' low parts (the last three accumulators)
#pragma unroll
          for (int c = 0; c < 3; ++c) lo[k][c] += (float)acc[k][NA - 3 + c];
        }
#pragma unroll
        for (int c = 0; c < NA; ++c) acc[k][c] = T(0);
      }
    }
  }
}

// ---- packed FP32: two sources per instruction (FFMA2 / FADD2 / FMUL2 on float2) -----------
// The FP32 kernels are bound by instruction issue, not by the FMA pipe: a packed
// instruction does two sources' operation in one issue slot.  Each lane of a packed
// operation rounds exactly like the scalar instruction.  A staged tile is re-laid out in
// shared memory as pairs of sources (2p, 2p+1), component-major so every load yields
// float2 operands directly:
//   Q[0][p] = (-x0, -x1, -y0, -y1)    Q[1][p] = (-z0, -z1, c0, c1)     (c: core parameter)
//   Q[2][p] = (wx0, wx1, wy0, wy1)    Q[3][p] = (wz0, wz1, -wx0, -wx1)
//   Q[4][p] = (-wy0, -wy1, -wz0, -wz1)
// (negated copies turn the separations and the cross products' differences into adds
// and fused multiply-adds).
__device__ __forceinline__ void stage_pair(const V4<float>& s, const V4<float>& w, float4 (*Q)[kBlock / 2], int j) {
  const int p = j >> 1, h = j & 1;
  float* q0 = reinterpret_cast<float*>(&Q[0][p]);
  float* q1 = reinterpret_cast<float*>(&Q[1][p]);
  float* q2 = reinterpret_cast<float*>(&Q[2][p]);
  float* q3 = reinterpret_cast<float*>(&Q[3][p]);
  float* q4 = reinterpret_cast<float*>(&Q[4][p]);
  q0[h] = -s.x; q0[2 + h] = -s.y;
  q1[h] = -s.z; q1[2 + h] = s.w;
  q2[h] = w.x;  q2[2 + h] = w.y;
  q3[h] = w.z;  q3[2 + h] = -w.x;
  q4[h] = -w.y; q4[2 + h] = -w.z;
}

__device__ __forceinline__ float2 f2lo(const float4& q) { return make_float2(q.x, q.y); }
__device__ __forceinline__ float2 f2hi(const float4& q) { return make_float2(q.z, q.w); }

// one target (tt = (x,x), (y,y), (z,z), (c,c)) against the source pair of q0..q4; a[] as in
// pair_g / pair_v, one float2 lane per source.  RM and the singular far-field kernel are
// packed throughout; the other cores evaluate r3 (and bbb) per lane with the scalar core.
template <int C, bool ACC, bool HAVE_TR, bool GRADS>
__device__ __forceinline__ void pair2(const float2* tt, const float4& q0, const float4& q1, const float4& q2,
                                      const float4& q3, const float4& q4, float2* a, const float* gtab) {
  const float2 dx = __fadd2_rn(tt[0], f2lo(q0));
  const float2 dy = __fadd2_rn(tt[1], f2hi(q0));
  const float2 dz = __fadd2_rn(tt[2], f2lo(q1));
  float2 r3, bbb = make_float2(0.f, 0.f);
  if constexpr (C == CORE_SING || C == CORE_RM) {
    float2 r2;
    if constexpr (C == CORE_RM) {
      const float2 cst = HAVE_TR ? __fadd2_rn(f2hi(q1), tt[3]) : f2hi(q1);
      r2 = __ffma2_rn(dz, dz, cst);
    } else {
      r2 = __fmul2_rn(dz, dz);
    }
    r2 = __ffma2_rn(dy, dy, r2);
    r2 = __ffma2_rn(dx, dx, r2);
    float2 rs = make_float2(rsqrtf(r2.x), rsqrtf(r2.y));
    if (ACC) {
      // y' = y + y/2 (1 - x y^2), as rsq<true>: fma(-y/2, x y^2 - 1, y)
      const float2 h = __fmul2_rn(r2, rs);
      const float2 e = __ffma2_rn(h, rs, make_float2(-1.f, -1.f));
      rs = __ffma2_rn(__fmul2_rn(rs, make_float2(-0.5f, -0.5f)), e, rs);
    }
    const float2 rs2 = __fmul2_rn(rs, rs);
    r3 = __fmul2_rn(rs2, rs);
    if (GRADS) bbb = __fmul2_rn(__fmul2_rn(r3, make_float2(-3.f, -3.f)), rs2);
  } else {
    const float2 cst = HAVE_TR ? __fadd2_rn(f2hi(q1), tt[3]) : f2hi(q1);
    if (GRADS) {
      core_g<C, ACC, float>(dx.x, dy.x, dz.x, cst.x, r3.x, bbb.x, gtab);
      core_g<C, ACC, float>(dx.y, dy.y, dz.y, cst.y, r3.y, bbb.y, gtab);
    } else {
      r3.x = core_v<C, ACC, float>(dx.x, dy.x, dz.x, cst.x, gtab);
      r3.y = core_v<C, ACC, float>(dx.y, dy.y, dz.y, cst.y, gtab);
    }
  }
  const float2 wx = f2lo(q2), wy = f2hi(q2), wz = f2lo(q3);
  const float2 nwx = f2hi(q3), nwy = f2lo(q4), nwz = f2hi(q4);
  float2 cx = __ffma2_rn(dz, wy, __fmul2_rn(dy, nwz));   // dz wy - dy wz
  float2 cy = __ffma2_rn(dx, wz, __fmul2_rn(dz, nwx));   // dx wz - dz wx
  float2 cz = __ffma2_rn(dy, wx, __fmul2_rn(dx, nwy));   // dy wx - dx wy
  a[0] = __ffma2_rn(r3, cx, a[0]);
  a[1] = __ffma2_rn(r3, cy, a[1]);
  a[2] = __ffma2_rn(r3, cz, a[2]);
  if (GRADS) {
    cx = __fmul2_rn(cx, bbb);
    cy = __fmul2_rn(cy, bbb);
    cz = __fmul2_rn(cz, bbb);
    a[3] = __ffma2_rn(dx, cx, a[3]);
    a[4] = __ffma2_rn(dx, cy, a[4]);
    a[5] = __ffma2_rn(dx, cz, a[5]);
    a[6] = __ffma2_rn(dy, cx, a[6]);
    a[7] = __ffma2_rn(dy, cy, a[7]);
    a[8] = __ffma2_rn(dy, cz, a[8]);
    a[9] = __ffma2_rn(dz, cx, a[9]);
    a[10] = __ffma2_rn(dz, cy, a[10]);
    a[11] = __ffma2_rn(dz, cz, a[11]);
    a[12] = __ffma2_rn(r3, wx, a[12]);
    a[13] = __ffma2_rn(r3, wy, a[13]);
    a[14] = __ffma2_rn(r3, wz, a[14]);
  }
}

// Sweep NP staged source pairs from pair p0 for TPT targets; in the compensated mode the
// two lanes' partials of every 8 pairs (16 sources) are added and folded into (hi, lo)
// with Fast2Sum, as sweep_tile does.
template <int C, int MODE, bool GRADS, bool HAVE_TR, int TPT, int NA, int NC, int NH, int NP>
__device__ __forceinline__ void sweep_pairs(const float4 (*Q)[kBlock / 2], int p0, const float2 (*tt)[4],
                                            float2 (*acc)[NA], float (*hi)[NH], float (*lo)[NH], const float* gtab) {
  constexpr bool ACC = (MODE == MODE_COMP);
  constexpr int FOLD = ACC ? 8 : NP;
#pragma unroll 1
  for (int j0 = 0; j0 < NP; j0 += FOLD) {
#pragma unroll 2
    for (int j = j0; j < j0 + FOLD; ++j) {
      const int p = p0 + j;
      const float4 q0 = Q[0][p], q1 = Q[1][p], q2 = Q[2][p], q3 = Q[3][p], q4 = Q[4][p];
#pragma unroll
      for (int k = 0; k < TPT; ++k) pair2<C, ACC, HAVE_TR, GRADS>(tt[k], q0, q1, q2, q3, q4, acc[k], gtab);
    }
    if (ACC) {
#pragma unroll
      for (int k = 0; k < TPT; ++k) {
        float a1[NA];
#pragma unroll
        for (int c = 0; c < NA; ++c) a1[c] = acc[k][c].x + acc[k][c].y;
        if (GRADS) fold_grads(a1);
#pragma unroll
        for (int c = 0; c < NC; ++c) {
          const float s = hi[k][c] + a1[c];
          const float e = a1[c] - (s - hi[k][c]);
          hi[k][c] = s;
          lo[k][c] += e;
        }
#pragma unroll
        for (int c = 0; c < NA; ++c) acc[k][c] = make_float2(0.f, 0.f);
      }
    }
  }
}

// far-field threshold on the squared distance, as a multiple of the pair's core parameter
template <int C> struct FarRule {
  __device__ static bool far(float, float) { return false; }
};
template <> struct FarRule<CORE_GAUSS> {
  // q = d^2 / (sr^2 + tr^2) > qfar: the Gaussian core equals the singular kernel
  __device__ static bool far(float d2min, float maxcst) { return d2min > GaussP<float>::qfar * maxcst; }
};
template <> struct FarRule<CORE_EXP> {
  // reld3 = d^3 / (sr^3 + tr^3) > 16 (CoreFunc.h:121): exp_cond returns 1/d^3; the box
  // test asks for 20 to stay clear of the boundary
  __device__ static bool far(float d2min, float maxcst) { return d2min * sqrtf(d2min) > 20.0f * maxcst; }
};

// bounding box and largest core parameter of the real targets of one warp (all lanes get
// the result), widened by a relative 1e-6 so float rounding never makes it too small;
// returns false when the warp holds no real target
template <int TPT, class T, bool RAW_R = false>
__device__ __forceinline__ bool warp_box(const V4<T>* tp, const bool* real, float* blo, float* bhi, float& bw) {
  float lo3[3] = {3.0e38f, 3.0e38f, 3.0e38f}, hi3[3] = {-3.0e38f, -3.0e38f, -3.0e38f}, mw = 0.f;
  bool any = false;
#pragma unroll
  for (int k = 0; k < TPT; ++k) {
    if (real[k]) {
      const float v[3] = {(float)tp[k].x, (float)tp[k].y, (float)tp[k].z};
#pragma unroll
      for (int d = 0; d < 3; ++d) { lo3[d] = fminf(lo3[d], v[d]); hi3[d] = fmaxf(hi3[d], v[d]); }
      // the core parameter r^2; the accurate mode's targets carry r itself
      mw = fmaxf(mw, RAW_R ? (float)tp[k].w * (float)tp[k].w : (float)tp[k].w);
      any = true;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      lo3[d] = fminf(lo3[d], __shfl_xor_sync(0xffffffffu, lo3[d], o));
      hi3[d] = fmaxf(hi3[d], __shfl_xor_sync(0xffffffffu, hi3[d], o));
    }
    mw = fmaxf(mw, __shfl_xor_sync(0xffffffffu, mw, o));
  }
  const float pad = 1e-6f * (fabsf(lo3[0]) + fabsf(lo3[1]) + fabsf(lo3[2]) + fabsf(hi3[0]) + fabsf(hi3[1]) +
                             fabsf(hi3[2]));
#pragma unroll
  for (int d = 0; d < 3; ++d) { blo[d] = lo3[d] - pad; bhi[d] = hi3[d] + pad; }
  bw = mw * 1.000001f;
  return __any_sync(0xffffffffu, any);
}

// far-field test of a warp's box against one half tile's box
template <int C, bool HAVE_TR>
__device__ __forceinline__ bool half_is_far(const float4& slo, const float4& shi, const float* blo, const float* bhi,
                                            float bw) {
  const float gx = fmaxf(0.f, fmaxf(slo.x - bhi[0], blo[0] - shi.x));
  const float gy = fmaxf(0.f, fmaxf(slo.y - bhi[1], blo[1] - shi.y));
  const float gz = fmaxf(0.f, fmaxf(slo.z - bhi[2], blo[2] - shi.z));
  return FarRule<C>::far(gx * gx + gy * gy + gz * gz, HAVE_TR ? slo.w + bw : slo.w);
}

template <int C, int MODE, bool GRADS, bool HAVE_TR, int TPT, class T, class O>
__global__ void __launch_bounds__(kBlock) k_pair(const PairArgs<T, O> a) {
  constexpr bool ACC = SumComp<MODE>::value;
  constexpr bool CLASSIFY = (C == CORE_GAUSS || C == CORE_EXP);
  // accumulators during the sweep (the accurate mode adds the velocity sums' low parts)
  constexpr int NA = (GRADS ? 15 : 3) + (MODE == MODE_DS ? 3 : 0);
  constexpr int NC = GRADS ? 12 : 3;   // output components
  constexpr int NH = ACC ? NC : 1;
  __shared__ V4<T> sp[kBlock];
  __shared__ V4<T> sw[kBlock];

  const int tid = threadIdx.x;
  const int split = blockIdx.y;
  // lane l of warp w holds targets tbase + 32 k (k < TPT): a contiguous run per warp
  const int tbase = blockIdx.x * (kBlock * TPT) + (tid >> 5) * (32 * TPT) + (tid & 31);

  V4<T> tp[TPT];
  bool real[TPT];
#pragma unroll
  for (int k = 0; k < TPT; ++k) {
    tp[k] = a.tpos[tbase + 32 * k];
    real[k] = tbase + 32 * k < a.nt;
  }

  float blo[3] = {0.f, 0.f, 0.f}, bhi[3] = {0.f, 0.f, 0.f}, bw = 0.f;
  bool live = true;
  if (CLASSIFY) live = warp_box<TPT, T, MODE == MODE_DS>(tp, real, blo, bhi, bw);

  T acc[TPT][NA];
#pragma unroll
  for (int k = 0; k < TPT; ++k)
#pragma unroll
    for (int c = 0; c < NA; ++c) acc[k][c] = T(0);
  float hi[TPT][NH], lo[TPT][NH];
#pragma unroll
  for (int k = 0; k < TPT; ++k)
#pragma unroll
    for (int c = 0; c < NH; ++c) { hi[k][c] = 0.f; lo[k][c] = 0.f; }

  const int t_begin = split * a.tiles_per_split;
  const int t_end = min(a.ntiles, t_begin + a.tiles_per_split);
  for (int tile = t_begin; tile < t_end; ++tile) {
    __syncthreads();
    sp[tid] = a.spos[(size_t)tile * kBlock + tid];
    sw[tid] = a.sstr[(size_t)tile * kBlock + tid];
    __syncthreads();
    if constexpr (CLASSIFY) {
      if (!live) continue;
#pragma unroll 1
      for (int hf = 0; hf < kBlock / kHalf; ++hf) {
        const int u = tile * (kBlock / kHalf) + hf;
        if (half_is_far<C, HAVE_TR>(a.tile_lo[u], a.tile_hi[u], blo, bhi, bw))
          sweep_tile<CORE_SING, MODE, GRADS, HAVE_TR, TPT, T, NA, NC, NH, kHalf>(sp + hf * kHalf, sw + hf * kHalf, tp,
                                                                               acc, hi, lo);
        else
          sweep_tile<C, MODE, GRADS, HAVE_TR, TPT, T, NA, NC, NH, kHalf>(sp + hf * kHalf, sw + hf * kHalf, tp, acc,
                                                                       hi, lo);
      }
    } else {
      sweep_tile<C, MODE, GRADS, HAVE_TR, TPT, T, NA, NC, NH>(sp, sw, tp, acc, hi, lo);
    }
  }

  // epilogue
#pragma unroll
  for (int k = 0; k < TPT; ++k) {
    const int idx = tbase + 32 * k;
    if (!ACC && GRADS) fold_grads(acc[k]);
    if (a.partial) {
      if (ACC) {
        T* base = a.partial + (size_t)split * (2 * NC) * a.nt_pad;
#pragma unroll
        for (int c = 0; c < NC; ++c) {
          base[(size_t)c * a.nt_pad + idx] = hi[k][c];
          base[(size_t)(NC + c) * a.nt_pad + idx] = lo[k][c];
        }
      } else {
        T* base = a.partial + (size_t)split * NC * a.nt_pad;
#pragma unroll
        for (int c = 0; c < NC; ++c) base[(size_t)c * a.nt_pad + idx] = acc[k][c];
      }
    } else if (idx < a.nt) {
      const int o = a.tperm ? (int)a.tperm[idx] : idx;
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        O* p = a.out.p[c] + o;
        if (ACC) *p = (O)((double)*p + ((double)hi[k][c] + (double)lo[k][c]));
        else     *p = (O)((T)*p + acc[k][c]);
      }
    }
  }
}

// k_pair for FP32 (PLAIN and COMPENSATED): the same blocks, tiles, far-field classification,
// splits and epilogue, with the sweep in packed FP32 over pairs of sources.  The staged
// tiles are double-buffered: the next tile is loaded into the other buffer before the
// current one is swept, so one barrier per tile orders both (two, without the second
// buffer, and the loads' latency in the open).
template <int C, int MODE, bool GRADS, bool HAVE_TR, int TPT>
__global__ void __launch_bounds__(kBlock) k_pair_f(const PairArgs<float, float> a) {
  constexpr bool ACC = (MODE == MODE_COMP);
  constexpr bool CLASSIFY = (C == CORE_GAUSS || C == CORE_EXP);
  constexpr int NA = GRADS ? 15 : 3;
  constexpr int NC = GRADS ? 12 : 3;
  constexpr int NH = ACC ? NC : 1;
  __shared__ float4 QB[2][5][kBlock / 2];
  // the Gaussian core's polynomial table, read from shared memory by the near-field pairs
  __shared__ __align__(16) float gsh[C == CORE_GAUSS ? kGaussPolyStride * kGaussPolyN : 1];
  const float* gtab = nullptr;
  if constexpr (C == CORE_GAUSS) {
    stage_gauss_table(gsh);   // visible after the first tile's __syncthreads
    gtab = gsh;
  }

  const int tid = threadIdx.x;
  const int split = blockIdx.y;
  const int tbase = blockIdx.x * (kBlock * TPT) + (tid >> 5) * (32 * TPT) + (tid & 31);

  V4<float> tp[TPT];
  bool real[TPT];
  float2 tt[TPT][4];
#pragma unroll
  for (int k = 0; k < TPT; ++k) {
    tp[k] = a.tpos[tbase + 32 * k];
    real[k] = tbase + 32 * k < a.nt;
    tt[k][0] = make_float2(tp[k].x, tp[k].x);
    tt[k][1] = make_float2(tp[k].y, tp[k].y);
    tt[k][2] = make_float2(tp[k].z, tp[k].z);
    tt[k][3] = make_float2(tp[k].w, tp[k].w);
  }

  float blo[3] = {0.f, 0.f, 0.f}, bhi[3] = {0.f, 0.f, 0.f}, bw = 0.f;
  bool live = true;
  if (CLASSIFY) live = warp_box<TPT, float>(tp, real, blo, bhi, bw);

  float2 acc[TPT][NA];
#pragma unroll
  for (int k = 0; k < TPT; ++k)
#pragma unroll
    for (int c = 0; c < NA; ++c) acc[k][c] = make_float2(0.f, 0.f);
  float hi[TPT][NH], lo[TPT][NH];
#pragma unroll
  for (int k = 0; k < TPT; ++k)
#pragma unroll
    for (int c = 0; c < NH; ++c) { hi[k][c] = 0.f; lo[k][c] = 0.f; }

  const int t_begin = split * a.tiles_per_split;
  const int t_end = min(a.ntiles, t_begin + a.tiles_per_split);
  if (t_begin < t_end)
    stage_pair(a.spos[(size_t)t_begin * kBlock + tid], a.sstr[(size_t)t_begin * kBlock + tid], QB[0], tid);
  for (int tile = t_begin; tile < t_end; ++tile) {
    // this tile's buffer is visible after the barrier, which also ends every sweep of the
    // other buffer (the previous tile), so the next tile may be written there
    __syncthreads();
    const int buf = (tile - t_begin) & 1;
    if (tile + 1 < t_end)
      stage_pair(a.spos[(size_t)(tile + 1) * kBlock + tid], a.sstr[(size_t)(tile + 1) * kBlock + tid], QB[buf ^ 1],
                 tid);
    const float4 (*Q)[kBlock / 2] = QB[buf];
    if constexpr (CLASSIFY) {
      if (!live) continue;
#pragma unroll 1
      for (int hf = 0; hf < kBlock / kHalf; ++hf) {
        const int u = tile * (kBlock / kHalf) + hf;
        if (half_is_far<C, HAVE_TR>(a.tile_lo[u], a.tile_hi[u], blo, bhi, bw))
          sweep_pairs<CORE_SING, MODE, GRADS, HAVE_TR, TPT, NA, NC, NH, kHalf / 2>(Q, hf * (kHalf / 2), tt, acc,
                                                                                  hi, lo, gtab);
        else
          sweep_pairs<C, MODE, GRADS, HAVE_TR, TPT, NA, NC, NH, kHalf / 2>(Q, hf * (kHalf / 2), tt, acc, hi, lo,
                                                                          gtab);
      }
    } else {
      sweep_pairs<C, MODE, GRADS, HAVE_TR, TPT, NA, NC, NH, kBlock / 2>(Q, 0, tt, acc, hi, lo, gtab);
    }
  }

  // epilogue: the two lanes of the plain sums are added here, as the last step of the sums
#pragma unroll
  for (int k = 0; k < TPT; ++k) {
    const int idx = tbase + 32 * k;
    float a1[NA];
#pragma unroll
    for (int c = 0; c < NA; ++c) a1[c] = acc[k][c].x + acc[k][c].y;
    if (!ACC && GRADS) fold_grads(a1);
    if (a.partial) {
      if (ACC) {
        float* base = a.partial + (size_t)split * (2 * NC) * a.nt_pad;
#pragma unroll
        for (int c = 0; c < NC; ++c) {
          base[(size_t)c * a.nt_pad + idx] = hi[k][c];
          base[(size_t)(NC + c) * a.nt_pad + idx] = lo[k][c];
        }
      } else {
        float* base = a.partial + (size_t)split * NC * a.nt_pad;
#pragma unroll
        for (int c = 0; c < NC; ++c) base[(size_t)c * a.nt_pad + idx] = a1[c];
      }
    } else if (idx < a.nt) {
      const int o = a.tperm ? (int)a.tperm[idx] : idx;
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        float* p = a.out.p[c] + o;
        if (ACC) *p = (float)((double)*p + ((double)hi[k][c] + (double)lo[k][c]));
        else     *p = *p + a1[c];
      }
    }
  }
}

// Sum the per-split partials in split order and add into the outputs.
template <int NC, bool ACC, class T, class O>
__global__ void k_reduce(const T* __restrict__ partial, int nsplit, int nt, int nt_pad, OutPtrs<O> out,
                         const uint32_t* __restrict__ tperm) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (idx >= nt) return;
  O* p = out.p[c] + (tperm ? (int)tperm[idx] : idx);
  if (ACC) {
    double s = 0.0;
    for (int k = 0; k < nsplit; ++k) {
      const T* base = partial + (size_t)k * (2 * NC) * nt_pad;
      s += (double)base[(size_t)c * nt_pad + idx];
      s += (double)base[(size_t)(NC + c) * nt_pad + idx];
    }
    *p = (O)((double)*p + s);
  } else {
    T s = T(0);
    for (int k = 0; k < nsplit; ++k) s += partial[((size_t)k * NC + c) * nt_pad + idx];
    *p = (O)((T)*p + s);
  }
}

// SoA -> packed float4/double4 sources, optionally gathered through perm
template <int C, class I, class T>
__global__ void k_pack_src(int n, int n_pad, const I* __restrict__ x, const I* __restrict__ y,
                           const I* __restrict__ z, const I* __restrict__ r, const I* __restrict__ sx,
                           const I* __restrict__ sy, const I* __restrict__ sz, const uint32_t* __restrict__ perm,
                           V4<T>* spos, V4<T>* sstr) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_pad) return;
  V4<T> p, w;
  if (i < n) {
    const int j = perm ? (int)perm[i] : i;
    const T ri = (T)r[j];
    p.x = (T)x[j]; p.y = (T)y[j]; p.z = (T)z[j]; p.w = core_param<C, T>(ri);
    w.x = (T)sx[j]; w.y = (T)sy[j]; w.z = (T)sz[j]; w.w = ri;
  } else {
    p.x = T(1e9); p.y = T(1e9); p.z = T(1e9); p.w = T(1);
    w.x = T(0); w.y = T(0); w.z = T(0); w.w = T(0);
  }
  spos[i] = p;
  sstr[i] = w;
}

// SoA -> packed targets; r == nullptr means field points (core parameter 0)
// RAW_R: w = r itself (the accurate mode forms r^2 exactly in the pair), else the core
// parameter
template <int C, class I, class T, bool RAW_R = false>
__global__ void k_pack_tgt(int n, int n_pad, const I* __restrict__ x, const I* __restrict__ y,
                           const I* __restrict__ z, const I* __restrict__ r, const uint32_t* __restrict__ perm,
                           V4<T>* tpos) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_pad) return;
  V4<T> p;
  if (i < n) {
    const int j = perm ? (int)perm[i] : i;
    p.x = (T)x[j]; p.y = (T)y[j]; p.z = (T)z[j];
    p.w = r ? (RAW_R ? (T)r[j] : core_param<C, T>((T)r[j])) : T(0);
  } else {
    p.x = T(0); p.y = T(0); p.z = T(0); p.w = T(0);
  }
  tpos[i] = p;
}

// per half tile (kHalf sources): bounding box of its real sources and their largest core
// parameter, widened by a relative 1e-6 so float rounding never shrinks it.  One block of
// kBlock threads per tile; half h is reduced by warps 2h and 2h+1.  A half without real
// sources gets an empty box (lo > hi), which every far-field test accepts.
template <class T>
__global__ void __launch_bounds__(kBlock) k_tile_bounds(const V4<T>* __restrict__ spos, int ns, float4* tlo,
                                                        float4* thi) {
  __shared__ float red[kBlock / 32][7];
  const int tile = blockIdx.x;
  const int i = tile * kBlock + threadIdx.x;
  float v[7];
  if (i < ns) {
    const V4<T> p = spos[i];
    v[0] = (float)p.x; v[1] = (float)p.y; v[2] = (float)p.z;
    v[3] = -(float)p.x; v[4] = -(float)p.y; v[5] = -(float)p.z;   // max via -min(-x)
    v[6] = -(float)p.w;
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

// ------------------------------------------------------------------------------
// host side
struct PairPlan {
  int tpt = 1;
  int ns_pad = 0, nt_pad = 0, ntiles = 0;
  int nsplit = 1, tiles_per_split = 0;
  int tblocks = 0;
};

template <int C, int MODE, bool GRADS, bool HAVE_TR, int TPT, class T, class O>
struct PairKernel {
  static const void* ptr() {
    if constexpr (std::is_same<T, float>::value && std::is_same<O, float>::value && MODE != MODE_DS)
      return (const void*)&k_pair_f<C, MODE, GRADS, HAVE_TR, TPT>;
    else
      return (const void*)&k_pair<C, MODE, GRADS, HAVE_TR, TPT, T, O>;
  }
};

// Chooses the source split so that the grid covers >= `waves` waves of resident blocks.
// The blocks' work differs (near- and far-field tiles), so the last wave leaves SMs idle;
// more, shorter blocks shrink that tail.  Measured on the 262,144-particle Gaussian cloud
// (compensated kernel, one GB300): 6 waves 116.7 ms, 12 113.2, 24 111.8, 48 110.8, 96
// 110.2 ms, while the per-split partial sums the reduction reads grow with the split
// count (29 splits, 730 MB, at 96 waves).  The allocating entry points use kPairWaves.
constexpr int kPairWaves = 48;
inline void plan_pair(int ns, int nt, int tpt, int slots, PairPlan* p, int waves = 6) {
  p->tpt = tpt;
  p->ntiles = (ns + kBlock - 1) / kBlock;
  p->ns_pad = p->ntiles * kBlock;
  const int tchunk = kBlock * tpt;
  p->tblocks = (nt + tchunk - 1) / tchunk;
  p->nt_pad = p->tblocks * tchunk;
  const long want = (long)waves * (slots > 0 ? slots : 1);
  long nsplit = (want + p->tblocks - 1) / p->tblocks;
  const long max_split = p->ntiles >= 2 ? p->ntiles / 2 : 1;
  if (nsplit > max_split) nsplit = max_split;
  if (nsplit < 1) nsplit = 1;
  p->tiles_per_split = (int)((p->ntiles + nsplit - 1) / nsplit);
  p->nsplit = (p->ntiles + p->tiles_per_split - 1) / p->tiles_per_split;
  if (p->nsplit < 1) p->nsplit = 1;
}

// The pipeline for one (core, mode, grads, target kind): [sort], pack, sweep, reduce.
template <int C, int MODE, bool GRADS, bool HAVE_TR, int TPT, class T, class I, class O>
int32_t run_points_points(int ns, const I* sx, const I* sy, const I* sz, const I* sr,
                          const I* ssx, const I* ssy, const I* ssz,
                          int nt, const I* tx, const I* ty, const I* tz, const I* tr,
                          OutPtrs<O> out, bool same, cudaStream_t st, size_t* ws_bytes_needed, char* ws_base) {
  constexpr int NC = GRADS ? 12 : 3;
  constexpr bool ACC = SumComp<MODE>::value;
  constexpr bool SORT = (C == CORE_GAUSS || C == CORE_EXP);
  // the accurate mode squares the radii itself: targets carry r (the sources' r is in the
  // strength record); same-set calls then pack the targets separately
  if (MODE == MODE_DS && tr) same = false;
  DeviceFacts df;
  O3G_TRY(device_facts(&df));
  int nb = 0;
  O3G_TRY(occupancy_blocks(PairKernel<C, MODE, GRADS, HAVE_TR, TPT, T, O>::ptr(), kBlock, &nb));
  PairPlan pl;
  plan_pair(ns, nt, TPT, nb * df.num_sms, &pl, kPairWaves);
  const int nsp = same ? (pl.ns_pad > pl.nt_pad ? pl.ns_pad : pl.nt_pad) : pl.ns_pad;
  size_t bytes = 2 * align_up((size_t)nsp * sizeof(V4<T>));
  if (!same) bytes += align_up((size_t)pl.nt_pad * sizeof(V4<T>));
  if (pl.nsplit > 1) bytes += align_up((size_t)pl.nsplit * NC * (ACC ? 2 : 1) * pl.nt_pad * sizeof(T));
  size_t sort_bytes = 0;
  if (SORT) {
    bytes += align_up((size_t)ns * sizeof(uint32_t)) + 2 * align_up((size_t)pl.ntiles * 2 * sizeof(float4));
    if (!same) bytes += align_up((size_t)nt * sizeof(uint32_t));
    sort_bytes = morton_sort_bytes(ns > nt ? ns : nt);
    bytes += sort_bytes;
  }
  if (ws_bytes_needed) { *ws_bytes_needed = bytes; return O3G_OK; }

  Carve cv(ws_base);
  V4<T>* spos = cv.take<V4<T>>(nsp);
  V4<T>* sstr = cv.take<V4<T>>(nsp);
  V4<T>* tpos = same ? spos : cv.take<V4<T>>(pl.nt_pad);
  T* partial = pl.nsplit > 1 ? cv.take<T>((size_t)pl.nsplit * NC * (ACC ? 2 : 1) * pl.nt_pad) : nullptr;
  uint32_t* sperm = nullptr;
  uint32_t* tperm = nullptr;
  float4* tile_lo = nullptr;
  float4* tile_hi = nullptr;
  if (SORT) {
    sperm = cv.take<uint32_t>(ns);
    tperm = same ? sperm : cv.take<uint32_t>(nt);
    tile_lo = cv.take<float4>((size_t)pl.ntiles * 2);
    tile_hi = cv.take<float4>((size_t)pl.ntiles * 2);
    char* sort_ws = cv.take<char>(sort_bytes);
    O3G_TRY(morton_sort<I>(sx, sy, sz, ns, sperm, sort_ws, st));
    if (!same) O3G_TRY(morton_sort<I>(tx, ty, tz, nt, tperm, sort_ws, st));
  }

  k_pack_src<C, I, T><<<(nsp + 255) / 256, 256, 0, st>>>(ns, nsp, sx, sy, sz, sr, ssx, ssy, ssz, sperm, spos, sstr);
  note_launch();
  if (!same) {
    k_pack_tgt<C, I, T, MODE == MODE_DS><<<(pl.nt_pad + 255) / 256, 256, 0, st>>>(nt, pl.nt_pad, tx, ty, tz, tr,
                                                                                tperm, tpos);
    note_launch();
  }
  if (SORT) {
    k_tile_bounds<T><<<pl.ntiles, kBlock, 0, st>>>(spos, ns, tile_lo, tile_hi);
    note_launch();
  }

  PairArgs<T, O> a;
  a.spos = spos; a.sstr = sstr; a.ntiles = pl.ntiles; a.tiles_per_split = pl.tiles_per_split;
  a.tpos = tpos; a.nt = nt; a.nt_pad = pl.nt_pad; a.partial = partial; a.out = out;
  a.tperm = tperm; a.tile_lo = tile_lo; a.tile_hi = tile_hi;
  dim3 grid(pl.tblocks, pl.nsplit);
  KernelTimer& tm = thread_timer();
  tm.begin(st);
  if constexpr (std::is_same<T, float>::value && std::is_same<O, float>::value && MODE != MODE_DS)
    k_pair_f<C, MODE, GRADS, HAVE_TR, TPT><<<grid, kBlock, 0, st>>>(a);
  else
    k_pair<C, MODE, GRADS, HAVE_TR, TPT, T, O><<<grid, kBlock, 0, st>>>(a);
  note_launch();
  tm.end(st);
  if (pl.nsplit > 1) {
    dim3 rg((nt + 255) / 256, NC);
    k_reduce<NC, ACC, T, O><<<rg, 256, 0, st>>>(partial, pl.nsplit, nt, pl.nt_pad, out, tperm);
    note_launch();
  }
  O3G_CUDA_TRY(cudaGetLastError());
  return O3G_OK;
}

// Dispatch on (mode, grads, target kind) for one core; declared here, defined per core
// in o3g_pair_<core>.cu so the instantiations compile in parallel.
struct PtPtCall {
  int mode;      // MODE_*
  bool grads;
  int ns, nt;
  bool same;     // sources and targets are the same packed set
  cudaStream_t st;
};
template <int C>
int32_t ptpt_core_f(const PtPtCall& c, const float* sx, const float* sy, const float* sz, const float* sr,
                    const float* ssx, const float* ssy, const float* ssz, const float* tx, const float* ty,
                    const float* tz, const float* tr, OutPtrs<float> out, size_t* need, char* ws);
template <int C>
int32_t ptpt_core_d(const PtPtCall& c, const double* sx, const double* sy, const double* sz, const double* sr,
                    const double* ssx, const double* ssy, const double* ssz, const double* tx, const double* ty,
                    const double* tz, const double* tr, OutPtrs<double> out, size_t* need, char* ws);

#define O3G_PTPT_ARGS c.ns, sx, sy, sz, sr, ssx, ssy, ssz, c.nt, tx, ty, tz, tr, out, c.same, c.st, need, ws
#define O3G_DEFINE_PTPT_CORE(CORE)                                                                           \
  template <>                                                                                                \
  int32_t ptpt_core_f<CORE>(const PtPtCall& c, const float* sx, const float* sy, const float* sz,            \
                            const float* sr, const float* ssx, const float* ssy, const float* ssz,           \
                            const float* tx, const float* ty, const float* tz, const float* tr,              \
                            OutPtrs<float> out, size_t* need, char* ws) {                                    \
    const bool htr = (tr != nullptr);                                                                        \
    if (c.mode == MODE_PLAIN) {                                                                              \
      if (c.grads) {                                                                                         \
        if (htr) return run_points_points<CORE, MODE_PLAIN, true, true, 2, float>(O3G_PTPT_ARGS);            \
        return run_points_points<CORE, MODE_PLAIN, true, false, 2, float>(O3G_PTPT_ARGS);                    \
      }                                                                                                      \
      if (htr) return run_points_points<CORE, MODE_PLAIN, false, true, 4, float>(O3G_PTPT_ARGS);             \
      return run_points_points<CORE, MODE_PLAIN, false, false, 4, float>(O3G_PTPT_ARGS);                     \
    }                                                                                                        \
    if (c.mode == MODE_COMP) {                                                                               \
      if (c.grads) {                                                                                         \
        if (htr) return run_points_points<CORE, MODE_COMP, true, true, 1, float>(O3G_PTPT_ARGS);             \
        return run_points_points<CORE, MODE_COMP, true, false, 1, float>(O3G_PTPT_ARGS);                     \
      }                                                                                                      \
      if (htr) return run_points_points<CORE, MODE_COMP, false, true, 2, float>(O3G_PTPT_ARGS);              \
      return run_points_points<CORE, MODE_COMP, false, false, 2, float>(O3G_PTPT_ARGS);                      \
    }                                                                                                        \
    if (c.mode == MODE_DS) {                                                                                 \
      if constexpr (CORE == CORE_RM || CORE == CORE_GAUSS) {                                                 \
        if (c.grads) {                                                                                       \
          if (htr) return run_points_points<CORE, MODE_DS, true, true, 1, float>(O3G_PTPT_ARGS);             \
          return run_points_points<CORE, MODE_DS, true, false, 1, float>(O3G_PTPT_ARGS);                     \
        }                                                                                                    \
        if (htr) return run_points_points<CORE, MODE_DS, false, true, 1, float>(O3G_PTPT_ARGS);              \
        return run_points_points<CORE, MODE_DS, false, false, 1, float>(O3G_PTPT_ARGS);                      \
      } else {                                                                                               \
        set_error("points_affect_points: precision ACCURATE supports the RM and Gaussian cores");            \
        return O3G_ERR_INVALID_ARG;                                                                          \
      }                                                                                                      \
    }                                                                                                        \
    if (c.grads) {                                                                                           \
      if (htr) return run_points_points<CORE, MODE_FP64, true, true, 1, double>(O3G_PTPT_ARGS);              \
      return run_points_points<CORE, MODE_FP64, true, false, 1, double>(O3G_PTPT_ARGS);                      \
    }                                                                                                        \
    if (htr) return run_points_points<CORE, MODE_FP64, false, true, 1, double>(O3G_PTPT_ARGS);               \
    return run_points_points<CORE, MODE_FP64, false, false, 1, double>(O3G_PTPT_ARGS);                       \
  }                                                                                                          \
  template <>                                                                                                \
  int32_t ptpt_core_d<CORE>(const PtPtCall& c, const double* sx, const double* sy, const double* sz,         \
                            const double* sr, const double* ssx, const double* ssy, const double* ssz,       \
                            const double* tx, const double* ty, const double* tz, const double* tr,          \
                            OutPtrs<double> out, size_t* need, char* ws) {                                   \
    const bool htr = (tr != nullptr);                                                                        \
    if (c.grads) {                                                                                           \
      if (htr) return run_points_points<CORE, MODE_FP64, true, true, 1, double>(O3G_PTPT_ARGS);              \
      return run_points_points<CORE, MODE_FP64, true, false, 1, double>(O3G_PTPT_ARGS);                      \
    }                                                                                                        \
    if (htr) return run_points_points<CORE, MODE_FP64, false, true, 1, double>(O3G_PTPT_ARGS);               \
    return run_points_points<CORE, MODE_FP64, false, false, 1, double>(O3G_PTPT_ARGS);                       \
  }

}  // namespace o3g
