// o3g_ds.cuh -- the accurate precision mode (O3G_PREC_ACCURATE) of the particle pair
// kernels: double-single ("float-float") arithmetic on FP32 instructions.
//
// A value is carried as hi + lo (two floats, |lo| about ulp(hi)/2 or less), about 44
// significant bits.  Per pair the mode forms, in double-single:
//   * the separation d = t - s (exact: a two-sum of the float coordinates);
//   * d^2 and the core parameter sigma^2 = sr^2 + tr^2 from exact products (fma);
//   * the core factor r3 (RM: (d^2 + sigma^2)^(-3/2); Gaussian: G(q) / sigma^3 from the
//     double-single polynomials of o3g_gauss_poly_ds.h; beyond q = 48 and in far tiles the
//     singular d^(-3): reciprocal square roots by one Newton step with the residual in
//     double-single);
//   * the cross product d x s (s, the strength, is a float);
// and adds each velocity term r3 (d x s) unrounded into a double-single running sum (a
// two-sum into the partial, the errors into a second float), folded every 16 sources into
// the (hi, lo) accumulators by a two-sum (exact in any order; COMPENSATED's Fast2Sum is
// not when the running sum is smaller than the partial).  The outputs are floats, so what
// remains of the velocity error is their final rounding.  Gradient terms use the double-
// single core rounded to float and the float separation, as in COMPENSATED.  Every operation is an explicitly rounded
// intrinsic (__fadd_rn, __fmul_rn, __fmaf_rn), so the compiler neither contracts nor
// reorders the error-free transformations.
//
// Error-free transformations: two-sum (Knuth), fast two-sum (Dekker, |a| >= |b|), and the
// product error fma(a, b, -a b) -- the standard float-float toolkit (Dekker 1971; Hida, Li
// and Bailey 2001).
#pragma once

#include "o3g_common.cuh"
#include "o3g_gauss_poly_ds.h"

namespace o3g {

struct dsf {
  float h, l;
};

__device__ __forceinline__ dsf ds_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
// |a| >= |b| (or a == 0)
__device__ __forceinline__ dsf ds_fast(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ dsf ds_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return {p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ dsf ds_add(dsf x, dsf y) {
  const dsf s = ds_two_sum(x.h, y.h);
  return ds_fast(s.h, __fadd_rn(s.l, __fadd_rn(x.l, y.l)));
}
__device__ __forceinline__ dsf ds_add_f(dsf x, float y) {
  const dsf s = ds_two_sum(x.h, y);
  return ds_fast(s.h, __fadd_rn(s.l, x.l));
}
__device__ __forceinline__ dsf ds_mul(dsf x, dsf y) {
  const float p = __fmul_rn(x.h, y.h);
  float e = __fmaf_rn(x.h, y.h, -p);
  e = __fmaf_rn(x.h, y.l, e);
  e = __fmaf_rn(x.l, y.h, e);
  return ds_fast(p, e);
}
__device__ __forceinline__ dsf ds_mul_f(dsf x, float y) {
  const float p = __fmul_rn(x.h, y);
  float e = __fmaf_rn(x.h, y, -p);
  e = __fmaf_rn(x.l, y, e);
  return ds_fast(p, e);
}
// d^2 with d = d.h + d.l (d.l^2, below 2^-48 relative, dropped)
__device__ __forceinline__ dsf ds_sq(dsf d) {
  const float p = __fmul_rn(d.h, d.h);
  float e = __fmaf_rn(d.h, d.h, -p);
  e = __fmaf_rn(__fmul_rn(2.0f, d.h), d.l, e);
  return ds_fast(p, e);
}
// x^(-1/2): the hardware estimate y, then y + y (1 - x y^2) / 2 with the residual formed from
// exact products (it is below 2^-21, so its own rounding is below 2^-45 relative)
__device__ __forceinline__ dsf ds_rsqrt(dsf x) {
  const float y = rsqrtf(x.h);
  const dsf y2 = ds_prod(y, y);
  float r = __fmaf_rn(-x.h, y2.h, 1.0f);
  r = __fmaf_rn(-x.h, y2.l, r);
  r = __fmaf_rn(-x.l, y2.h, r);
  return ds_fast(y, __fmul_rn(__fmul_rn(0.5f, y), r));
}
// p u - q v (p, q double-single, u, v float), unnormalised: the sum hi + lo is the value
// to about 2^-46 of |p u| + |q v|
__device__ __forceinline__ dsf ds_cross(dsf p, float u, dsf q, float v) {
  dsf a = ds_prod(p.h, u);
  a.l = __fmaf_rn(p.l, u, a.l);
  dsf b = ds_prod(q.h, v);
  b.l = __fmaf_rn(q.l, v, b.l);
  const dsf s = ds_two_sum(a.h, -b.h);
  return {s.h, __fadd_rn(s.l, __fsub_rn(a.l, b.l))};
}
// (x * c) rounded once to float, x and c double-single (c may be unnormalised)
__device__ __forceinline__ float ds_term(dsf x, dsf c) {
  const float th = __fmul_rn(x.h, c.h);
  float tl = __fmaf_rn(x.h, c.h, -th);
  tl = __fmaf_rn(x.h, c.l, tl);
  tl = __fmaf_rn(x.l, c.h, tl);
  return __fadd_rn(th, tl);
}
__device__ __forceinline__ float ds_round(dsf x) { return __fadd_rn(x.h, x.l); }
// acc + acc_lo += x * c without rounding the product: its high part goes into acc by a
// two-sum, the rounding errors (of the product and of that sum) into acc_lo
__device__ __forceinline__ void ds_accum(float& acc, float& acc_lo, dsf x, dsf c) {
  const float th = __fmul_rn(x.h, c.h);
  float tl = __fmaf_rn(x.h, c.h, -th);
  tl = __fmaf_rn(x.h, c.l, tl);
  tl = __fmaf_rn(x.l, c.h, tl);
  const dsf sm = ds_two_sum(acc, th);
  acc = sm.h;
  acc_lo = __fadd_rn(acc_lo, __fadd_rn(sm.l, tl));
}

// G(q) (and D(q) = 2 G'(q) when GRAD) of the Gaussian core for q in [0, 48], q double-single:
// Horner's rule in float for the degrees >= kGaussDsPairs, then in double-single
template <bool GRAD>
__device__ __forceinline__ void gauss_poly_ds(dsf q, dsf& G, dsf& D) {
  constexpr int N = kGaussPolyN;
  const float* tb = kGaussPolyDs;
  const int j = gauss_interval(q.h);
  const dsf t = ds_add_f(ds_mul_f(q, __ldg(tb + j)), __ldg(tb + N + j));
  constexpr int NF = kGaussDsDeg + 1 - kGaussDsPairs;      // float coefficients per function
  float g = __ldg(tb + 2 * N + j), d = GRAD ? __ldg(tb + 3 * N + j) : 0.f;
#pragma unroll
  for (int k = 1; k < NF; ++k) {
    g = __fmaf_rn(g, t.h, __ldg(tb + (2 + 2 * k) * N + j));
    if (GRAD) d = __fmaf_rn(d, t.h, __ldg(tb + (3 + 2 * k) * N + j));
  }
  dsf gg{g, 0.f}, dd{d, 0.f};
#pragma unroll
  for (int k = 0; k < kGaussDsPairs; ++k) {
    const int e = 2 + 2 * NF + 4 * k;
    gg = ds_add(ds_mul(gg, t), dsf{__ldg(tb + e * N + j), __ldg(tb + (e + 1) * N + j)});
    if (GRAD) dd = ds_add(ds_mul(dd, t), dsf{__ldg(tb + (e + 2) * N + j), __ldg(tb + (e + 3) * N + j)});
  }
  G = gg;
  D = dd;
}

// Core factor in double-single for CORE_SING, CORE_RM and CORE_GAUSS: r3 (and bbb, rounded
// to float, when GRAD), from d^2 and the radii sr, tr (tr = 0 for singular targets)
template <int C, bool GRAD>
__device__ __forceinline__ void core_ds(dsf d2, float sr, float tr, dsf& r3, float& bbb) {
  if (C == CORE_SING) {
    const dsf rs = ds_rsqrt(d2);
    const dsf rs2 = ds_mul(rs, rs);
    r3 = ds_mul(rs2, rs);
    if (GRAD) bbb = __fmul_rn(__fmul_rn(-3.0f, r3.h), rs2.h);
    return;
  }
  const dsf sig2 = ds_add(ds_prod(sr, sr), ds_prod(tr, tr));
  if (C == CORE_RM) {
    // CoreFunc.h:66-71: r2 = d^2 + sr^2 + tr^2, r3 = r2^-1.5, bbb = -3 r3 / r2
    const dsf rs = ds_rsqrt(ds_add(d2, sig2));
    const dsf rs2 = ds_mul(rs, rs);
    r3 = ds_mul(rs2, rs);
    if (GRAD) bbb = __fmul_rn(__fmul_rn(-3.0f, r3.h), rs2.h);
    return;
  }
  // Gaussian: the singular kernel beyond q = 48 (the correction is below 3e-10 there)
  if (d2.h > 48.0f * sig2.h) {
    core_ds<CORE_SING, GRAD>(d2, 0.f, 0.f, r3, bbb);
    return;
  }
  const dsf rsg = ds_rsqrt(sig2);
  const dsf rsg2 = ds_mul(rsg, rsg);
  dsf G, D;
  gauss_poly_ds<GRAD>(ds_mul(d2, rsg2), G, D);
  const dsf isig3 = ds_mul(rsg2, rsg);
  r3 = ds_mul(G, isig3);
  if (GRAD) bbb = __fmul_rn(__fmul_rn(ds_round(D), ds_round(isig3)), ds_round(rsg2));
}

}  // namespace o3g
