// o3d_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of Omega3D's Biot-Savart / BEM hot path, used by tests/, by the
// smoke check and by the CPU-baseline leg of bench.py as the checker.  It is never
// linked into, loaded by, or called from the product library (omega3d_gb300/csrc).
//
// Every function restates the reference algorithm in the reference's own arithmetic
// order so that, compiled with -ffp-contract=off, it is bit-identical to the
// reference's own code compiled the same way.  oracle/build_ref.sh builds that code
// into oracle/_ref/ and the pinning tests compare:
//   Kernels.h/CoreFunc.h/MathHelper.h: the pair and panel kernels;
//   Reflect.h: clear_inner_layer;
//   Split.h/Merge.h with nanoflann: split and merge;
//   GeomHelper.cpp/IglRefine.cpp with igl upsample: the sphere.
// Parity unpinned: the Gaussian core, which the reference does not have (checked against
// an independent closed form instead); and the BEM solve, whose Eigen GMRES is absent
// (checked against an FP64 LU of the same matrix instead).
//
// Template parameters follow the reference: S = storage/arithmetic type,
// A = accumulator type (Influence.h:67 `template <class S, class A>`).
//   prec 0 : S=float,  A=float   (the reference's Vc build, Simulation.h:41-43)
//   prec 1 : S=float,  A=double  (the reference's non-Vc build, Simulation.h:44-46)
//   prec 2 : S=double, A=double  (FP64 oracle)
//
// Array conventions (all component-major SoA, like std::array<Vector<S>,3>):
//   positions x[3*n] = {x0..x(n-1), y0.., z0..}; strengths likewise;
//   velocity u[3*n]; gradient ug[9*n] in the reference order
//   [du/dx, dv/dx, dw/dx, du/dy, dv/dy, dw/dy, du/dz, dv/dz, dw/dz] (Kernels.h:184-192).

#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstddef>
#include <vector>
#include <unordered_map>
#include <algorithm>
#include <limits>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

enum { CORE_RM = 0, CORE_WL = 1, CORE_EXP = 2, CORE_GAUSS = 3, CORE_V2 = 4 };

// ---------------------------------------------------------------------------------
// MathHelper.h:62-72,87-91,108-113,127-134,148-155,171-180 (non-Vc generic forms)
template <class S> static inline S my_recip(const S in) { return S(1.0) / in; }
template <class S> static inline S my_sqrt(const S in) { return std::sqrt(in); }
template <class S> static inline S my_rsqrt(const S in) { return S(1.0) / std::sqrt(in); }
template <class S> static inline S oor2p5(const S in) { return S(1.0) / (in * in * std::sqrt(in)); }
template <class S> static inline S oor1p5(const S in) { return S(1.0) / (in * std::sqrt(in)); }
template <class S> static inline S oor0p75(const S in) {
  const S sqd = std::sqrt(in);
  return S(1.0) / (sqd * std::sqrt(sqd));
}

// ---------------------------------------------------------------------------------
// Compact-exponential branches, CoreFunc.h:119-132 (exp_cond) and :160-174 (exp_bbb)
template <class S> static inline S exp_cond(const S ood3, const S corefac, const S reld3) {
  if (reld3 > 16.0f) return ood3;
  else if (reld3 < 0.001f) return corefac;
  else return ood3 * (1.0f - std::exp(-reld3));
}
template <class S> static inline S exp_bbb(const S r3, const S corefac, const S reld3, const S dist, const S distsq) {
  if (reld3 > 16.0f) return -3.0f * r3 / distsq;
  else if (reld3 < 0.001f) return -1.5f * dist * r3 * r3;
  else {
    const S expreld3 = std::exp(-reld3);
    return 3.0f * (corefac * expreld3 - r3) / distsq;
  }
}

// ---------------------------------------------------------------------------------
// Gaussian core.  No reference implementation exists (Core.h serves only diffusion),
// so this is the project's own definition, shared with the CUDA kernels:
//   sigma^2 = sr^2 + tr^2,  q = d^2/sigma^2,  rho = sqrt(q)
//   K(r)   = [erf(rho/sqrt2) - sqrt(2/pi) rho exp(-q/2)] / r^3
//   bbb    = (1/r) dK/dr = [sqrt(2/pi) exp(-q/2)/sigma^3 - 3K] / r^2
// with a Taylor series for q < 1 (the closed form cancels there) and the singular
// 1/r^3 form beyond q_far (where erf == 1 and the exp term is below rounding).
template <class S> struct GaussParams;
template <> struct GaussParams<float>  { static constexpr float  qfar = 48.0f; static constexpr int nterms = 9; };
template <> struct GaussParams<double> { static constexpr double qfar = 90.0;  static constexpr int nterms = 17; };

// series coefficients c_n of G(q) = sqrt(2/pi) * sum_{n>=1} c_n q^(n-1),
//   c_n = (-1)^(n+1) / ((2n+1) 2^(n-1) (n-1)!)
static inline double gauss_coef(int n) {
  double c = 1.0 / (2.0 * n + 1.0);
  for (int k = 1; k < n; ++k) c /= (2.0 * k);
  return (n % 2 == 1) ? c : -c;
}

template <class S>
static inline void gauss_core(const S distsq, const S sig2, S* r3, S* bbb) {
  const S sqrt2opi = S(0.79788456080286535588);
  const S q = distsq / sig2;
  if (q > GaussParams<S>::qfar) {
    const S d = std::sqrt(distsq);
    *r3 = S(1.0) / (distsq * d);
    *bbb = S(-3.0) * (*r3) / distsq;
  } else if (q < S(1.0)) {
    const int nt = GaussParams<S>::nterms;
    S g = S(0.0), gp = S(0.0);
    for (int n = nt; n >= 1; --n) g = g * q + S(gauss_coef(n));
    for (int n = nt; n >= 2; --n) gp = gp * q + S((n - 1) * gauss_coef(n));
    const S sig = std::sqrt(sig2);
    const S sig3 = sig2 * sig;
    *r3 = sqrt2opi * g / sig3;
    *bbb = S(2.0) * sqrt2opi * gp / (sig3 * sig2);
  } else {
    const S d = std::sqrt(distsq);
    const S rho = std::sqrt(q);
    const S e = std::exp(S(-0.5) * q);
    const S g = std::erf(rho * S(0.70710678118654752440)) - sqrt2opi * rho * e;
    const S sig = std::sqrt(sig2);
    *r3 = g / (distsq * d);
    *bbb = (sqrt2opi * e / (sig2 * sig) - S(3.0) * (*r3)) / distsq;
  }
}
template <class S>
static inline S gauss_core_v(const S distsq, const S sig2) {
  S r3, bbb;
  gauss_core<S>(distsq, sig2, &r3, &bbb);
  return r3;
}

// ---------------------------------------------------------------------------------
// core_func, velocity only, thick-cored target: CoreFunc.h:48-52 (RM), :202-209 (EXP),
// :246-252 (WL), :297-304 (V2)
template <int C, class S> static inline S core_tv(const S distsq, const S sr, const S tr) {
  if constexpr (C == CORE_RM) {
    const S r2 = distsq + sr * sr + tr * tr;
    return oor1p5(r2);
  } else if constexpr (C == CORE_WL) {
    const S r2 = sr * sr + tr * tr;
    const S d2 = distsq + r2;
    return (distsq + S(2.5) * r2) * oor2p5<S>(d2);
  } else if constexpr (C == CORE_EXP) {
    const S dist = my_sqrt(distsq);
    const S ood3 = my_recip(distsq * dist);
    const S corefac = my_recip(sr * sr * sr + tr * tr * tr);
    const S reld3 = corefac / ood3;
    return exp_cond(ood3, corefac, reld3);
  } else if constexpr (C == CORE_V2) {
    const S s2 = sr * sr;
    const S t2 = tr * tr;
    const S denom = distsq * distsq + s2 * s2 + t2 * t2;
    return oor0p75<S>(denom);
  } else {
    return gauss_core_v<S>(distsq, sr * sr + tr * tr);
  }
}
// core_func, velocity only, singular target: CoreFunc.h:56-61 (RM), :189-197 (EXP),
// :255-262 (WL), :307-314 (V2)
template <int C, class S> static inline S core_tp(const S distsq, const S sr) {
  if constexpr (C == CORE_RM) {
    const S r2 = distsq + sr * sr;
    return oor1p5(r2);
  } else if constexpr (C == CORE_WL) {
    const S r2 = sr * sr;
    const S d2 = distsq + r2;
    return (distsq + S(2.5) * r2) * oor2p5<S>(d2);
  } else if constexpr (C == CORE_EXP) {
    const S dist = my_sqrt(distsq);
    const S ood3 = my_recip(distsq * dist);
    const S corefac = my_recip(sr * sr * sr);
    const S reld3 = corefac / ood3;
    return exp_cond(ood3, corefac, reld3);
  } else if constexpr (C == CORE_V2) {
    const S s2 = sr * sr;
    const S denom = distsq * distsq + s2 * s2;
    return oor0p75<S>(denom);
  } else {
    return gauss_core_v<S>(distsq, sr * sr);
  }
}
// core_func with gradients, thick-cored target: CoreFunc.h:66-71 (RM), :226-236 (EXP),
// :266-274 (WL), :318-330 (V2)
template <int C, class S> static inline void core_tvg(const S distsq, const S sr, const S tr, S* r3, S* bbb) {
  if constexpr (C == CORE_RM) {
    const S r2 = distsq + sr * sr + tr * tr;
    *r3 = oor1p5(r2);
    *bbb = S(-3.0) * (*r3) * my_recip(r2);
  } else if constexpr (C == CORE_WL) {
    const S r2 = sr * sr + tr * tr;
    const S d2 = distsq + r2;
    const S d2top = distsq + S(2.5) * r2;
    const S dn5 = oor2p5<S>(d2);
    *r3 = d2top * dn5;
    *bbb = S(2.0) * dn5 - S(5.0) * d2top * dn5 / d2;
  } else if constexpr (C == CORE_EXP) {
    const S dist = my_sqrt(distsq);
    const S corefac = my_recip(sr * sr * sr + tr * tr * tr);
    const S d3 = distsq * dist;
    const S reld3 = d3 * corefac;
    const S ood3 = my_recip(d3);
    *r3 = exp_cond(ood3, corefac, reld3);
    *bbb = exp_bbb(*r3, corefac, reld3, dist, distsq);
  } else if constexpr (C == CORE_V2) {
    const S s2 = sr * sr;
    const S t2 = tr * tr;
    const S denom = distsq * distsq + s2 * s2 + t2 * t2;
    *r3 = oor0p75<S>(denom);
    *bbb = S(-3.0) * (*r3) * my_rsqrt(denom);
  } else {
    gauss_core<S>(distsq, sr * sr + tr * tr, r3, bbb);
  }
}
// core_func with gradients, singular target: CoreFunc.h:76-81 (RM), :211-223 (EXP),
// :279-287 (WL), :333-339 (V2)
template <int C, class S> static inline void core_tpg(const S distsq, const S sr, S* r3, S* bbb) {
  if constexpr (C == CORE_RM) {
    const S r2 = distsq + sr * sr;
    *r3 = oor1p5(r2);
    *bbb = S(-3.0) * (*r3) * my_recip(r2);
  } else if constexpr (C == CORE_WL) {
    const S r2 = sr * sr;
    const S d2 = distsq + r2;
    const S d2top = distsq + S(2.5) * r2;
    const S dn5 = oor2p5<S>(d2);
    *r3 = d2top * dn5;
    *bbb = S(2.0) * dn5 - S(5.0) * d2top * dn5 / d2;
  } else if constexpr (C == CORE_EXP) {
    const S dist = my_sqrt(distsq);
    const S corefac = my_recip(sr * sr * sr);
    const S d3 = distsq * dist;
    const S reld3 = d3 * corefac;
    const S ood3 = my_recip(d3);
    *r3 = exp_cond(ood3, corefac, reld3);
    *bbb = exp_bbb(*r3, corefac, reld3, dist, distsq);
  } else if constexpr (C == CORE_V2) {
    const S s2 = sr * sr;
    const S denom = distsq * distsq + s2 * s2;
    *r3 = oor0p75<S>(denom);
    *bbb = S(-3.0) * (*r3) * my_rsqrt(denom);
  } else {
    gauss_core<S>(distsq, sr * sr, r3, bbb);
  }
}

// ---------------------------------------------------------------------------------
// Pair kernels.  Target-radius variants (b) and singular-target variants (p) differ
// only in which core_func overload they call.

// kernel_0v_0b / kernel_0v_0p, Kernels.h:50-69 / :94-112
template <int C, bool HaveTr, class S, class A>
static inline void k_0v_0x(const S sx, const S sy, const S sz, const S sr,
                           const S ssx, const S ssy, const S ssz,
                           const S tx, const S ty, const S tz, const S tr,
                           A* tu, A* tv, A* tw) {
  const S dx = tx - sx;
  const S dy = ty - sy;
  const S dz = tz - sz;
  const S r2 = HaveTr ? core_tv<C, S>(dx * dx + dy * dy + dz * dz, sr, tr)
                      : core_tp<C, S>(dx * dx + dy * dy + dz * dz, sr);
  const S dxxw = dz * ssy - dy * ssz;
  const S dyxw = dx * ssz - dz * ssx;
  const S dzxw = dy * ssx - dx * ssy;
  *tu += r2 * dxxw;
  *tv += r2 * dyxw;
  *tw += r2 * dzxw;
}

// kernel_0v_0bg / kernel_0v_0pg, Kernels.h:155-193 / :253-290
template <int C, bool HaveTr, class S, class A>
static inline void k_0v_0xg(const S sx, const S sy, const S sz, const S sr,
                            const S ssx, const S ssy, const S ssz,
                            const S tx, const S ty, const S tz, const S tr,
                            A* acc /* 12: u v w ux vx wx uy vy wy uz vz wz */) {
  const S dx = tx - sx;
  const S dy = ty - sy;
  const S dz = tz - sz;
  S r3, bbb;
  if (HaveTr) core_tvg<C, S>(dx * dx + dy * dy + dz * dz, sr, tr, &r3, &bbb);
  else        core_tpg<C, S>(dx * dx + dy * dy + dz * dz, sr, &r3, &bbb);
  S dxxw = dz * ssy - dy * ssz;
  S dyxw = dx * ssz - dz * ssx;
  S dzxw = dy * ssx - dx * ssy;
  acc[0] += r3 * dxxw;
  acc[1] += r3 * dyxw;
  acc[2] += r3 * dzxw;
  dxxw *= bbb;
  dyxw *= bbb;
  dzxw *= bbb;
  acc[3]  += dx * dxxw;
  acc[4]  += dx * dyxw + ssz * r3;
  acc[5]  += dx * dzxw - ssy * r3;
  acc[6]  += dy * dxxw - ssz * r3;
  acc[7]  += dy * dyxw;
  acc[8]  += dy * dzxw + ssx * r3;
  acc[9]  += dz * dxxw + ssy * r3;
  acc[10] += dz * dyxw - ssx * r3;
  acc[11] += dz * dzxw;
}

// kernel_0vs_0p, Kernels.h:115-133 (vortex + source strength, singular target)
template <int C, class S, class A>
static inline void k_0vs_0p(const S sx, const S sy, const S sz, const S sr,
                            const S ssx, const S ssy, const S ssz, const S ss,
                            const S tx, const S ty, const S tz,
                            A* tu, A* tv, A* tw) {
  const S dx = tx - sx;
  const S dy = ty - sy;
  const S dz = tz - sz;
  const S r2 = core_tp<C, S>(dx * dx + dy * dy + dz * dz, sr);
  const S dxxw = dz * ssy - dy * ssz + dx * ss;
  const S dyxw = dx * ssz - dz * ssx + dy * ss;
  const S dzxw = dy * ssx - dx * ssy + dz * ss;
  *tu += r2 * dxxw;
  *tv += r2 * dyxw;
  *tw += r2 * dzxw;
}

// kernel_0vs_0pg, Kernels.h:294-345
template <int C, class S, class A>
static inline void k_0vs_0pg(const S sx, const S sy, const S sz, const S sr,
                             const S ssx, const S ssy, const S ssz, const S ss,
                             const S tx, const S ty, const S tz, A* acc) {
  const S dx = tx - sx;
  const S dy = ty - sy;
  const S dz = tz - sz;
  S r3, bbb;
  core_tpg<C, S>(dx * dx + dy * dy + dz * dz, sr, &r3, &bbb);
  S dxxw = dz * ssy - dy * ssz;
  S dyxw = dx * ssz - dz * ssx;
  S dzxw = dy * ssx - dx * ssy;
  acc[0] += r3 * (dxxw + dx * ss);
  acc[1] += r3 * (dyxw + dy * ss);
  acc[2] += r3 * (dzxw + dz * ss);
  dxxw *= bbb;
  dyxw *= bbb;
  dzxw *= bbb;
  acc[3]  += dx * dxxw;
  acc[4]  += dx * dyxw + ssz * r3;
  acc[5]  += dx * dzxw - ssy * r3;
  acc[6]  += dy * dxxw - ssz * r3;
  acc[7]  += dy * dyxw;
  acc[8]  += dy * dzxw + ssx * r3;
  acc[9]  += dz * dxxw + ssy * r3;
  acc[10] += dz * dyxw - ssx * r3;
  acc[11] += dz * dzxw;
  const S dxs = dx * bbb * ss;
  const S dys = dy * bbb * ss;
  const S dzs = dz * bbb * ss;
  const S dss = ss * r3;
  acc[3]  += dx * dxs + dss;
  acc[4]  += dx * dys;
  acc[5]  += dx * dzs;
  acc[6]  += dy * dxs;
  acc[7]  += dy * dys + dss;
  acc[8]  += dy * dzs;
  acc[9]  += dz * dxs;
  acc[10] += dz * dys;
  acc[11] += dz * dzs + dss;
}

// ---------------------------------------------------------------------------------
// Adaptive panel kernels.
// The child-triangle table and the 1/2-midpoint construction are the subdivision rule
// of Kernels.h:1085-1092 (same in :1180-1187 and :1282-1292).
static const int kChild[4][3] = {{0, 1, 3}, {1, 2, 4}, {1, 4, 3}, {3, 4, 5}};

// rkernel_2vs_0p, Kernels.h:1028-1115 (panel on point, velocity only)
template <int C, class S, class A>
static void rk_2vs_0p(const S sx0, const S sy0, const S sz0,
                      const S sx1, const S sy1, const S sz1,
                      const S sx2, const S sy2, const S sz2,
                      const S ssx, const S ssy, const S ssz, const S ss,
                      const S tx, const S ty, const S tz,
                      const S sa, const int lev, const int maxlev,
                      A* tu, A* tv, A* tw) {
  S strx = ssx, stry = ssy, strz = ssz, strs = ss;
  if (lev == 0) { strx *= sa; stry *= sa; strz *= sa; strs *= sa; }
  const S sx = (sx0 + sx1 + sx2) / S(3.0);
  const S sy = (sy0 + sy1 + sy2) / S(3.0);
  const S sz = (sz0 + sz1 + sz2) / S(3.0);
  const S trisize = my_sqrt<S>(sa);
  const S dist = my_sqrt<S>((tx - sx) * (tx - sx) + (ty - sy) * (ty - sy) + (tz - sz) * (tz - sz));
  const bool wellsep = (dist > trisize * S(4.0));
  if (wellsep || lev == maxlev) {
    k_0vs_0p<C, S, A>(sx, sy, sz, S(0.0), strx, stry, strz, strs, tx, ty, tz, tu, tv, tw);
  } else {
    strx *= S(0.25); stry *= S(0.25); strz *= S(0.25); strs *= S(0.25);
    const S sca = S(0.25) * sa;
    const S cx[6] = {sx0, S(0.5) * (sx0 + sx1), sx1, S(0.5) * (sx0 + sx2), S(0.5) * (sx1 + sx2), sx2};
    const S cy[6] = {sy0, S(0.5) * (sy0 + sy1), sy1, S(0.5) * (sy0 + sy2), S(0.5) * (sy1 + sy2), sy2};
    const S cz[6] = {sz0, S(0.5) * (sz0 + sz1), sz1, S(0.5) * (sz0 + sz2), S(0.5) * (sz1 + sz2), sz2};
    for (int i = 0; i < 4; ++i) {
      const int a = kChild[i][0], b = kChild[i][1], c = kChild[i][2];
      rk_2vs_0p<C, S, A>(cx[a], cy[a], cz[a], cx[b], cy[b], cz[b], cx[c], cy[c], cz[c],
                         strx, stry, strz, strs, tx, ty, tz, sca, lev + 1, maxlev, tu, tv, tw);
    }
  }
}

// rkernel_2vs_0pg, Kernels.h:1120-1211 (panel on point, with gradients)
template <int C, class S, class A>
static void rk_2vs_0pg(const S sx0, const S sy0, const S sz0,
                       const S sx1, const S sy1, const S sz1,
                       const S sx2, const S sy2, const S sz2,
                       const S ssx, const S ssy, const S ssz, const S ss,
                       const S tx, const S ty, const S tz,
                       const S sa, const int lev, const int maxlev, A* acc) {
  S strx = ssx, stry = ssy, strz = ssz, strs = ss;
  if (lev == 0) { strx *= sa; stry *= sa; strz *= sa; strs *= sa; }
  const S sx = (sx0 + sx1 + sx2) / S(3.0);
  const S sy = (sy0 + sy1 + sy2) / S(3.0);
  const S sz = (sz0 + sz1 + sz2) / S(3.0);
  const S trisize = my_sqrt<S>(sa);
  const S dist = my_sqrt<S>((tx - sx) * (tx - sx) + (ty - sy) * (ty - sy) + (tz - sz) * (tz - sz));
  const bool wellsep = (dist > trisize * S(4.0));
  if (wellsep || lev == maxlev) {
    k_0vs_0pg<C, S, A>(sx, sy, sz, S(0.0), strx, stry, strz, strs, tx, ty, tz, acc);
  } else {
    strx *= S(0.25); stry *= S(0.25); strz *= S(0.25); strs *= S(0.25);
    const S sca = S(0.25) * sa;
    const S cx[6] = {sx0, S(0.5) * (sx0 + sx1), sx1, S(0.5) * (sx0 + sx2), S(0.5) * (sx1 + sx2), sx2};
    const S cy[6] = {sy0, S(0.5) * (sy0 + sy1), sy1, S(0.5) * (sy0 + sy2), S(0.5) * (sy1 + sy2), sy2};
    const S cz[6] = {sz0, S(0.5) * (sz0 + sz1), sz1, S(0.5) * (sz0 + sz2), S(0.5) * (sz1 + sz2), sz2};
    for (int i = 0; i < 4; ++i) {
      const int a = kChild[i][0], b = kChild[i][1], c = kChild[i][2];
      rk_2vs_0pg<C, S, A>(cx[a], cy[a], cz[a], cx[b], cy[b], cz[b], cx[c], cy[c], cz[c],
                          strx, stry, strz, strs, tx, ty, tz, sca, lev + 1, maxlev, acc);
    }
  }
}

// rkernel_2vs_2p, Kernels.h:1217-1315 (panel on panel, velocity at target centroid)
template <int C, class S, class A>
static void rk_2vs_2p(const S sx0, const S sy0, const S sz0,
                      const S sx1, const S sy1, const S sz1,
                      const S sx2, const S sy2, const S sz2,
                      const S ssx, const S ssy, const S ssz, const S ss,
                      const S tx0, const S ty0, const S tz0,
                      const S tx1, const S ty1, const S tz1,
                      const S tx2, const S ty2, const S tz2,
                      const S sa, const S ta, const int lev, const int maxlev,
                      A* tu, A* tv, A* tw) {
  S strx = ssx, stry = ssy, strz = ssz, strs = ss;
  if (lev == 0) { strx *= sa; stry *= sa; strz *= sa; strs *= sa; }
  const S sx = (sx0 + sx1 + sx2) / S(3.0);
  const S sy = (sy0 + sy1 + sy2) / S(3.0);
  const S sz = (sz0 + sz1 + sz2) / S(3.0);
  const S tx = (tx0 + tx1 + tx2) / S(3.0);
  const S ty = (ty0 + ty1 + ty2) / S(3.0);
  const S tz = (tz0 + tz1 + tz2) / S(3.0);
  const S trisize = my_sqrt<S>(sa) + my_sqrt<S>(ta);
  const S dist = my_sqrt<S>((tx - sx) * (tx - sx) + (ty - sy) * (ty - sy) + (tz - sz) * (tz - sz));
  const bool wellsep = (dist > trisize * S(4.0));
  if (wellsep || lev == maxlev) {
    k_0vs_0p<C, S, A>(sx, sy, sz, S(0.0), strx, stry, strz, strs, tx, ty, tz, tu, tv, tw);
  } else {
    strx *= S(0.0625); stry *= S(0.0625); strz *= S(0.0625); strs *= S(0.0625);
    const S sca = S(0.25) * sa;
    const S tca = S(0.25) * ta;
    const S scx[6] = {sx0, S(0.5) * (sx0 + sx1), sx1, S(0.5) * (sx0 + sx2), S(0.5) * (sx1 + sx2), sx2};
    const S scy[6] = {sy0, S(0.5) * (sy0 + sy1), sy1, S(0.5) * (sy0 + sy2), S(0.5) * (sy1 + sy2), sy2};
    const S scz[6] = {sz0, S(0.5) * (sz0 + sz1), sz1, S(0.5) * (sz0 + sz2), S(0.5) * (sz1 + sz2), sz2};
    const S tcx[6] = {tx0, S(0.5) * (tx0 + tx1), tx1, S(0.5) * (tx0 + tx2), S(0.5) * (tx1 + tx2), tx2};
    const S tcy[6] = {ty0, S(0.5) * (ty0 + ty1), ty1, S(0.5) * (ty0 + ty2), S(0.5) * (ty1 + ty2), ty2};
    const S tcz[6] = {tz0, S(0.5) * (tz0 + tz1), tz1, S(0.5) * (tz0 + tz2), S(0.5) * (tz1 + tz2), tz2};
    for (int i = 0; i < 4; ++i) {
      for (int j = 0; j < 4; ++j) {
        const int a = kChild[i][0], b = kChild[i][1], c = kChild[i][2];
        const int d = kChild[j][0], e = kChild[j][1], f = kChild[j][2];
        rk_2vs_2p<C, S, A>(scx[a], scy[a], scz[a], scx[b], scy[b], scz[b], scx[c], scy[c], scz[c],
                           strx, stry, strz, strs,
                           tcx[d], tcy[d], tcz[d], tcx[e], tcy[e], tcz[e], tcx[f], tcy[f], tcz[f],
                           sca, tca, lev + 1, maxlev, tu, tv, tw);
      }
    }
  }
}

// ---------------------------------------------------------------------------------
// Loops.  The target loop is outermost, sources innermost, accumulate in A then
// add into the caller's arrays (+=), as in the reference's non-Vc x86 path.

// points_affect_points, Influence.h:278-309 (field points, grads), :312-366 (field
// points, vel only), :445-475 (particles, grads), :477-534 (particles, vel only)
template <int C, class S, class A>
static void ptpt(int ns, const S* sx, const S* sr, const S* ss,
                 int nt, const S* tx, const S* tr, S* tu, S* tug, int nthreads) {
  const S* sy = sx + ns; const S* sz = sx + 2 * (size_t)ns;
  const S* ssx = ss; const S* ssy = ss + ns; const S* ssz = ss + 2 * (size_t)ns;
  const S* ty = tx + nt; const S* tz = tx + 2 * (size_t)nt;
#pragma omp parallel for num_threads(nthreads) schedule(static)
  for (int i = 0; i < nt; ++i) {
    const S trad = tr ? tr[i] : S(0.0);
    if (tug) {
      A acc[12] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
      if (tr) {
        for (int j = 0; j < ns; ++j)
          k_0v_0xg<C, true, S, A>(sx[j], sy[j], sz[j], sr[j], ssx[j], ssy[j], ssz[j], tx[i], ty[i], tz[i], trad, acc);
      } else {
        for (int j = 0; j < ns; ++j)
          k_0v_0xg<C, false, S, A>(sx[j], sy[j], sz[j], sr[j], ssx[j], ssy[j], ssz[j], tx[i], ty[i], tz[i], trad, acc);
      }
      for (int d = 0; d < 3; ++d) tu[d * (size_t)nt + i] += acc[d];
      for (int d = 0; d < 9; ++d) tug[d * (size_t)nt + i] += acc[3 + d];
    } else {
      A au = 0, av = 0, aw = 0;
      if (tr) {
        for (int j = 0; j < ns; ++j)
          k_0v_0x<C, true, S, A>(sx[j], sy[j], sz[j], sr[j], ssx[j], ssy[j], ssz[j], tx[i], ty[i], tz[i], trad, &au, &av, &aw);
      } else {
        for (int j = 0; j < ns; ++j)
          k_0v_0x<C, false, S, A>(sx[j], sy[j], sz[j], sr[j], ssx[j], ssy[j], ssz[j], tx[i], ty[i], tz[i], trad, &au, &av, &aw);
      }
      tu[i] += au; tu[nt + (size_t)i] += av; tu[2 * (size_t)nt + i] += aw;
    }
  }
}

// panels_affect_points, Influence.h:948-1000 (particle targets with grads; the target
// radius is ignored, :872-873) and the field-point / velocity-only siblings, which are
// the same loop.  The sheet strength passed down is ts/area (:958), the source-sheet
// strength sss or 0 when the collection has none (:980).
template <int C, class S, class A>
static void panpt(int maxlev, int nn, const S* nx, int np, const uint32_t* idx, const S* area,
                  const S* ts, const S* sss, int nt, const S* tx, S* tu, S* tug, int nthreads) {
  const S* ny = nx + nn; const S* nz = nx + 2 * (size_t)nn;
  const S* tsx = ts; const S* tsy = ts + np; const S* tsz = ts + 2 * (size_t)np;
  const S* ty = tx + nt; const S* tz = tx + 2 * (size_t)nt;
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 16)
  for (int i = 0; i < nt; ++i) {
    A acc[12] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int j = 0; j < np; ++j) {
      const size_t p0 = idx[3 * (size_t)j], p1 = idx[3 * (size_t)j + 1], p2 = idx[3 * (size_t)j + 2];
      const S srcs = sss ? sss[j] : S(0.0);
      if (tug) {
        rk_2vs_0pg<C, S, A>(nx[p0], ny[p0], nz[p0], nx[p1], ny[p1], nz[p1], nx[p2], ny[p2], nz[p2],
                            tsx[j] / area[j], tsy[j] / area[j], tsz[j] / area[j], srcs,
                            tx[i], ty[i], tz[i], area[j], 0, maxlev, acc);
      } else {
        rk_2vs_0p<C, S, A>(nx[p0], ny[p0], nz[p0], nx[p1], ny[p1], nz[p1], nx[p2], ny[p2], nz[p2],
                           tsx[j] / area[j], tsy[j] / area[j], tsz[j] / area[j], srcs,
                           tx[i], ty[i], tz[i], area[j], 0, maxlev, &acc[0], &acc[1], &acc[2]);
      }
    }
    for (int d = 0; d < 3; ++d) tu[d * (size_t)nt + i] += acc[d];
    if (tug) for (int d = 0; d < 9; ++d) tug[d * (size_t)nt + i] += acc[3 + d];
  }
}

// points_affect_panels, Influence.h:1192-1215: the target panel is subdivided as if it
// were the source, with sheet strength = particle strength / target area, and the result
// is subtracted.  The particle core radius is not used.
template <int C, class S, class A>
static void ptpan(int maxlev, int ns, const S* sx, const S* ss,
                  int nn, const S* nx, int np, const uint32_t* idx, const S* area,
                  S* pu, int nthreads) {
  const S* sy = sx + ns; const S* sz = sx + 2 * (size_t)ns;
  const S* ssx = ss; const S* ssy = ss + ns; const S* ssz = ss + 2 * (size_t)ns;
  const S* ny = nx + nn; const S* nz = nx + 2 * (size_t)nn;
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 4)
  for (int i = 0; i < np; ++i) {
    A au = 0, av = 0, aw = 0;
    const size_t p0 = idx[3 * (size_t)i], p1 = idx[3 * (size_t)i + 1], p2 = idx[3 * (size_t)i + 2];
    for (int j = 0; j < ns; ++j) {
      rk_2vs_0p<C, S, A>(nx[p0], ny[p0], nz[p0], nx[p1], ny[p1], nz[p1], nx[p2], ny[p2], nz[p2],
                         ssx[j] / area[i], ssy[j] / area[i], ssz[j] / area[i], S(0.0),
                         sx[j], sy[j], sz[j], area[i], 0, maxlev, &au, &av, &aw);
    }
    pu[i] -= au; pu[np + (size_t)i] -= av; pu[2 * (size_t)np + i] -= aw;
  }
}

// panels_on_panels_coeff, Coefficients.h:169-447 (non-Vc branch :334-411, self terms
// :414-436, 1/4pi scale :443-447).  Output is column-major: column (j*nunk+k) holds the
// influence of unknown k of source panel j on every target row i*nunk+l.
template <int C, class S>
static void panpan_coeff(int maxlev, int nunk, int is_self,
                         int snn, const S* snx, int snp, const uint32_t* sidx, const S* sarea,
                         const S* sx1, const S* sx2,
                         int tnn, const S* tnx, int tnp, const uint32_t* tidx, const S* tarea,
                         const S* tx1, const S* tx2, const S* tnorm,
                         S* coeffs, int nthreads) {
  const S* sny = snx + snn; const S* snz = snx + 2 * (size_t)snn;
  const S* tny = tnx + tnn; const S* tnz = tnx + 2 * (size_t)tnn;
  const bool has_src = (nunk == 3);
  const size_t nrows = (size_t)tnp * nunk;
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 4)
  for (int j = 0; j < snp; ++j) {
    size_t jptr[3];
    for (int k = 0; k < nunk; ++k) jptr[k] = ((size_t)j * nunk + k) * nrows;
    const size_t a0 = sidx[3 * (size_t)j], a1 = sidx[3 * (size_t)j + 1], a2 = sidx[3 * (size_t)j + 2];
    const S x0 = snx[a0], y0 = sny[a0], z0 = snz[a0];
    const S x1 = snx[a1], y1 = sny[a1], z1 = snz[a1];
    const S x2 = snx[a2], y2 = sny[a2], z2 = snz[a2];
    const S sa = sarea[j];
    for (int i = 0; i < tnp; ++i) {
      const size_t b0 = tidx[3 * (size_t)i], b1 = tidx[3 * (size_t)i + 1], b2 = tidx[3 * (size_t)i + 2];
      const S tb1x = tx1[i], tb1y = tx1[tnp + (size_t)i], tb1z = tx1[2 * (size_t)tnp + i];
      const S tb2x = tx2[i], tb2y = tx2[tnp + (size_t)i], tb2z = tx2[2 * (size_t)tnp + i];
      for (int k = 0; k < nunk; ++k) {
        S sxv, syv, szv, ssv;
        if (k == 0)      { sxv = sx1[j]; syv = sx1[snp + (size_t)j]; szv = sx1[2 * (size_t)snp + j]; ssv = S(0.0); }
        else if (k == 1) { sxv = sx2[j]; syv = sx2[snp + (size_t)j]; szv = sx2[2 * (size_t)snp + j]; ssv = S(0.0); }
        else             { sxv = S(0.0); syv = S(0.0); szv = S(0.0); ssv = S(1.0); }
        S ru = 0.0, rv = 0.0, rw = 0.0;
        rk_2vs_2p<C, S, S>(x0, y0, z0, x1, y1, z1, x2, y2, z2, sxv, syv, szv, ssv,
                           tnx[b0], tny[b0], tnz[b0], tnx[b1], tny[b1], tnz[b1], tnx[b2], tny[b2], tnz[b2],
                           sa, tarea[i], 0, maxlev, &ru, &rv, &rw);
        coeffs[jptr[k]++] = ru * tb1x + rv * tb1y + rw * tb1z;
        coeffs[jptr[k]++] = ru * tb2x + rv * tb2y + rw * tb2z;
        if (has_src) coeffs[jptr[k]++] = ru * tnorm[i] + rv * tnorm[tnp + (size_t)i] + rw * tnorm[2 * (size_t)tnp + i];
      }
    }
    if (is_self) {
      size_t dptr = (size_t)j * tnp * nunk * nunk + (size_t)j * nunk;
      coeffs[dptr] = 0.0;
      coeffs[dptr + 1] = 2.0 * M_PI;
      if (has_src) coeffs[dptr + 2] = 0.0;
      dptr += (size_t)tnp * nunk;
      coeffs[dptr] = -2.0 * M_PI;
      coeffs[dptr + 1] = 0.0;
      if (has_src) coeffs[dptr + 2] = 0.0;
      if (has_src) {
        dptr += (size_t)tnp * nunk;
        coeffs[dptr] = 0.0;
        coeffs[dptr + 1] = 0.0;
        coeffs[dptr + 2] = 2.0 * M_PI;
      }
    }
  }
  const S fac = 1.0 / (4.0 * M_PI);
  const size_t ntot = nrows * (size_t)snp * nunk;
  for (size_t e = 0; e < ntot; ++e) coeffs[e] = coeffs[e] * fac;
}

template <int C, class S, class A>
static void dispatch_ptpt_core(int ns, const S* sx, const S* sr, const S* ss, int nt, const S* tx, const S* tr,
                               S* tu, S* tug, int nth) {
  ptpt<C, S, A>(ns, sx, sr, ss, nt, tx, tr, tu, tug, nth);
}

}  // namespace

// =================================================================================
// extern "C" surface of the oracle
// =================================================================================
#define O3O_CORE_SWITCH(core, FN, ...)                         \
  switch (core) {                                              \
    case CORE_RM: FN<CORE_RM>(__VA_ARGS__); break;             \
    case CORE_WL: FN<CORE_WL>(__VA_ARGS__); break;             \
    case CORE_EXP: FN<CORE_EXP>(__VA_ARGS__); break;           \
    case CORE_GAUSS: FN<CORE_GAUSS>(__VA_ARGS__); break;       \
    case CORE_V2: FN<CORE_V2>(__VA_ARGS__); break;             \
    default: return 1;                                         \
  }

template <int C> static void ptpt_f(int ns, const float* sx, const float* sr, const float* ss, int nt,
                                    const float* tx, const float* tr, float* tu, float* tug, int nth) {
  ptpt<C, float, float>(ns, sx, sr, ss, nt, tx, tr, tu, tug, nth);
}
template <int C> static void ptpt_fd(int ns, const float* sx, const float* sr, const float* ss, int nt,
                                     const float* tx, const float* tr, float* tu, float* tug, int nth) {
  ptpt<C, float, double>(ns, sx, sr, ss, nt, tx, tr, tu, tug, nth);
}
template <int C> static void ptpt_d(int ns, const double* sx, const double* sr, const double* ss, int nt,
                                    const double* tx, const double* tr, double* tu, double* tug, int nth) {
  ptpt<C, double, double>(ns, sx, sr, ss, nt, tx, tr, tu, tug, nth);
}

// points_affect_points.  prec 0: float/float, 1: float/double accumulators, 2: double.
// tr == NULL means field-point targets; tug == NULL means velocity only.
extern "C" int o3o_points_affect_points(int prec, int core, int ns, const void* sx, const void* sr, const void* ss,
                             int nt, const void* tx, const void* tr, void* tu, void* tug, int nthreads) {
  if (ns < 0 || nt < 0) return 1;
  if (prec == 0) {
    O3O_CORE_SWITCH(core, ptpt_f, ns, (const float*)sx, (const float*)sr, (const float*)ss, nt,
                    (const float*)tx, (const float*)tr, (float*)tu, (float*)tug, nthreads)
  } else if (prec == 1) {
    O3O_CORE_SWITCH(core, ptpt_fd, ns, (const float*)sx, (const float*)sr, (const float*)ss, nt,
                    (const float*)tx, (const float*)tr, (float*)tu, (float*)tug, nthreads)
  } else if (prec == 2) {
    O3O_CORE_SWITCH(core, ptpt_d, ns, (const double*)sx, (const double*)sr, (const double*)ss, nt,
                    (const double*)tx, (const double*)tr, (double*)tu, (double*)tug, nthreads)
  } else {
    return 1;
  }
  return 0;
}

template <int C> static void panpt_f(int ml, int nn, const float* nx, int np, const uint32_t* idx, const float* ar,
                                     const float* ts, const float* sss, int nt, const float* tx, float* tu, float* tug, int nth) {
  panpt<C, float, float>(ml, nn, nx, np, idx, ar, ts, sss, nt, tx, tu, tug, nth);
}
template <int C> static void panpt_fd(int ml, int nn, const float* nx, int np, const uint32_t* idx, const float* ar,
                                      const float* ts, const float* sss, int nt, const float* tx, float* tu, float* tug, int nth) {
  panpt<C, float, double>(ml, nn, nx, np, idx, ar, ts, sss, nt, tx, tu, tug, nth);
}
template <int C> static void panpt_d(int ml, int nn, const double* nx, int np, const uint32_t* idx, const double* ar,
                                     const double* ts, const double* sss, int nt, const double* tx, double* tu, double* tug, int nth) {
  panpt<C, double, double>(ml, nn, nx, np, idx, ar, ts, sss, nt, tx, tu, tug, nth);
}

// panels_affect_points.  ts = absolute panel vortex strengths (Surfaces::get_str),
// sss = source sheet strengths or NULL.
extern "C" int o3o_panels_affect_points(int prec, int core, int maxlev, int nn, const void* nx, int np, const uint32_t* idx,
                             const void* area, const void* ts, const void* sss, int nt, const void* tx,
                             void* tu, void* tug, int nthreads) {
  if (nn < 0 || np < 0 || nt < 0 || maxlev < 0) return 1;
  if (prec == 0) {
    O3O_CORE_SWITCH(core, panpt_f, maxlev, nn, (const float*)nx, np, idx, (const float*)area, (const float*)ts,
                    (const float*)sss, nt, (const float*)tx, (float*)tu, (float*)tug, nthreads)
  } else if (prec == 1) {
    O3O_CORE_SWITCH(core, panpt_fd, maxlev, nn, (const float*)nx, np, idx, (const float*)area, (const float*)ts,
                    (const float*)sss, nt, (const float*)tx, (float*)tu, (float*)tug, nthreads)
  } else if (prec == 2) {
    O3O_CORE_SWITCH(core, panpt_d, maxlev, nn, (const double*)nx, np, idx, (const double*)area, (const double*)ts,
                    (const double*)sss, nt, (const double*)tx, (double*)tu, (double*)tug, nthreads)
  } else {
    return 1;
  }
  return 0;
}

template <int C> static void ptpan_f(int ml, int ns, const float* sx, const float* ss, int nn, const float* nx, int np,
                                     const uint32_t* idx, const float* ar, float* pu, int nth) {
  ptpan<C, float, float>(ml, ns, sx, ss, nn, nx, np, idx, ar, pu, nth);
}
template <int C> static void ptpan_fd(int ml, int ns, const float* sx, const float* ss, int nn, const float* nx, int np,
                                      const uint32_t* idx, const float* ar, float* pu, int nth) {
  ptpan<C, float, double>(ml, ns, sx, ss, nn, nx, np, idx, ar, pu, nth);
}
template <int C> static void ptpan_d(int ml, int ns, const double* sx, const double* ss, int nn, const double* nx, int np,
                                     const uint32_t* idx, const double* ar, double* pu, int nth) {
  ptpan<C, double, double>(ml, ns, sx, ss, nn, nx, np, idx, ar, pu, nth);
}

// points_affect_panels (BEM right-hand side velocities).  Subtracts into pu[3*np].
extern "C" int o3o_points_affect_panels(int prec, int core, int maxlev, int ns, const void* sx, const void* ss,
                             int nn, const void* nx, int np, const uint32_t* idx, const void* area,
                             void* pu, int nthreads) {
  if (ns < 0 || nn < 0 || np < 0 || maxlev < 0) return 1;
  if (prec == 0) {
    O3O_CORE_SWITCH(core, ptpan_f, maxlev, ns, (const float*)sx, (const float*)ss, nn, (const float*)nx, np, idx,
                    (const float*)area, (float*)pu, nthreads)
  } else if (prec == 1) {
    O3O_CORE_SWITCH(core, ptpan_fd, maxlev, ns, (const float*)sx, (const float*)ss, nn, (const float*)nx, np, idx,
                    (const float*)area, (float*)pu, nthreads)
  } else if (prec == 2) {
    O3O_CORE_SWITCH(core, ptpan_d, maxlev, ns, (const double*)sx, (const double*)ss, nn, (const double*)nx, np, idx,
                    (const double*)area, (double*)pu, nthreads)
  } else {
    return 1;
  }
  return 0;
}

template <int C> static void coeff_f(int ml, int nunk, int self, int snn, const float* snx, int snp, const uint32_t* sidx,
                                     const float* sa, const float* sx1, const float* sx2, int tnn, const float* tnx, int tnp,
                                     const uint32_t* tidx, const float* ta, const float* tx1, const float* tx2,
                                     const float* tn, float* out, int nth) {
  panpan_coeff<C, float>(ml, nunk, self, snn, snx, snp, sidx, sa, sx1, sx2, tnn, tnx, tnp, tidx, ta, tx1, tx2, tn, out, nth);
}
template <int C> static void coeff_d(int ml, int nunk, int self, int snn, const double* snx, int snp, const uint32_t* sidx,
                                     const double* sa, const double* sx1, const double* sx2, int tnn, const double* tnx, int tnp,
                                     const uint32_t* tidx, const double* ta, const double* tx1, const double* tx2,
                                     const double* tn, double* out, int nth) {
  panpan_coeff<C, double>(ml, nunk, self, snn, snx, snp, sidx, sa, sx1, sx2, tnn, tnx, tnp, tidx, ta, tx1, tx2, tn, out, nth);
}

// panels_on_panels_coeff.  prec 0 (float) or 2 (double); the reference instantiates it
// with A == S (Coefficients.h:347 rkernel_2vs_2p<S,S>).
extern "C" int o3o_panels_on_panels_coeff(int prec, int core, int maxlev, int nunk, int is_self,
                               int snn, const void* snx, int snp, const uint32_t* sidx, const void* sarea,
                               const void* sx1, const void* sx2,
                               int tnn, const void* tnx, int tnp, const uint32_t* tidx, const void* tarea,
                               const void* tx1, const void* tx2, const void* tnorm, void* coeffs, int nthreads) {
  if (nunk != 2 && nunk != 3) return 1;
  if (snp < 0 || tnp < 0 || maxlev < 0) return 1;
  if (is_self && snp != tnp) return 1;
  if (prec == 0) {
    O3O_CORE_SWITCH(core, coeff_f, maxlev, nunk, is_self, snn, (const float*)snx, snp, sidx, (const float*)sarea,
                    (const float*)sx1, (const float*)sx2, tnn, (const float*)tnx, tnp, tidx, (const float*)tarea,
                    (const float*)tx1, (const float*)tx2, (const float*)tnorm, (float*)coeffs, nthreads)
  } else if (prec == 2) {
    O3O_CORE_SWITCH(core, coeff_d, maxlev, nunk, is_self, snn, (const double*)snx, snp, sidx, (const double*)sarea,
                    (const double*)sx1, (const double*)sx2, tnn, (const double*)tnx, tnp, tidx, (const double*)tarea,
                    (const double*)tx1, (const double*)tx2, (const double*)tnorm, (double*)coeffs, nthreads)
  } else {
    return 1;
  }
  return 0;
}

// Surfaces::compute_bases, Surfaces.h:776-816: x1 along edge 0->1, x2 orthogonalised
// toward node 2, norm = x1 x x2, area = 0.5*base*height (the 1.0/len and 0.5*
// products are evaluated in double and rounded to float, as written there).
extern "C" int o3o_compute_bases(int nn, const float* nx, int np, const uint32_t* idx,
                      float* x1out, float* x2out, float* nout, float* area) {
  if (nn < 0 || np < 0) return 1;
  for (int i = 0; i < np; ++i) {
    const size_t id0 = idx[3 * (size_t)i], id1 = idx[3 * (size_t)i + 1], id2 = idx[3 * (size_t)i + 2];
    if (id0 >= (size_t)nn || id1 >= (size_t)nn || id2 >= (size_t)nn) return 1;
    float x1[3], x2[3], nm[3];
    for (int j = 0; j < 3; ++j) x1[j] = nx[j * (size_t)nn + id1] - nx[j * (size_t)nn + id0];
    const float base = std::sqrt(x1[0] * x1[0] + x1[1] * x1[1] + x1[2] * x1[2]);
    for (int j = 0; j < 3; ++j) x1[j] *= (1.0 / base);
    for (int j = 0; j < 3; ++j) x2[j] = nx[j * (size_t)nn + id2] - nx[j * (size_t)nn + id0];
    const float dp = x2[0] * x1[0] + x2[1] * x1[1] + x2[2] * x1[2];
    for (int j = 0; j < 3; ++j) x2[j] -= dp * x1[j];
    const float height = std::sqrt(x2[0] * x2[0] + x2[1] * x2[1] + x2[2] * x2[2]);
    for (int j = 0; j < 3; ++j) x2[j] *= (1.0 / height);
    area[i] = 0.5 * base * height;
    nm[0] = x1[1] * x2[2] - x1[2] * x2[1];
    nm[1] = x1[2] * x2[0] - x1[0] * x2[2];
    nm[2] = x1[0] * x2[1] - x1[1] * x2[0];
    for (int j = 0; j < 3; ++j) {
      x1out[j * (size_t)np + i] = x1[j];
      x2out[j * (size_t)np + i] = x2[j];
      nout[j * (size_t)np + i] = nm[j];
    }
  }
  return 0;
}

// Surfaces::vortex_sheet_to_panel_strength, Surfaces.h:309-335:
//   ts = (ps0*x1 + ps1*x2) * area
extern "C" int o3o_sheet_to_panel_strength(int np, const float* ps0, const float* ps1, const float* x1, const float* x2,
                                const float* area, float* ts) {
  if (np < 0) return 1;
  for (int i = 0; i < np; ++i)
    for (int d = 0; d < 3; ++d)
      ts[d * (size_t)np + i] = (ps0[i] * x1[d * (size_t)np + i] + ps1[i] * x2[d * (size_t)np + i]) * area[i];
  return 0;
}

// vels_to_rhs_panels, RHS.h:92-110: rhs = -(u.x1, u.x2[, u.n]) per panel.
extern "C" int o3o_vels_to_rhs_panels(int np, int nunk, const float* pu, const float* x1, const float* x2,
                           const float* nrm, float* rhs) {
  if (np < 0 || nunk < 1 || nunk > 3) return 1;
  for (int i = 0; i < np; ++i) {
    const float u = pu[i], v = pu[np + (size_t)i], w = pu[2 * (size_t)np + i];
    if (nunk == 1) {
      rhs[i] = -(u * nrm[i] + v * nrm[np + (size_t)i] + w * nrm[2 * (size_t)np + i]);
    } else {
      rhs[nunk * (size_t)i + 0] = -(u * x1[i] + v * x1[np + (size_t)i] + w * x1[2 * (size_t)np + i]);
      rhs[nunk * (size_t)i + 1] = -(u * x2[i] + v * x2[np + (size_t)i] + w * x2[2 * (size_t)np + i]);
      if (nunk == 3)
        rhs[3 * (size_t)i + 2] = -(u * nrm[i] + v * nrm[np + (size_t)i] + w * nrm[2 * (size_t)np + i]);
    }
  }
  return 0;
}

// finalize_vels: ElementBase.h:187-193 (u = fs + u * (0.25/pi), evaluated in double),
// Points.h:265-277 (ug *= float(0.25/pi)), Surfaces.h:877-887 (panel vels as u).
extern "C" int o3o_finalize_vels(int n, const double* fs, float* u, float* ug) {
  if (n < 0) return 1;
  const double factor = 0.25 / M_PI;
  for (int d = 0; d < 3; ++d)
    for (int i = 0; i < n; ++i) u[d * (size_t)n + i] = fs[d] + u[d * (size_t)n + i] * factor;
  if (ug) {
    const float gfac = 0.25 / M_PI;
    for (size_t e = 0; e < 9 * (size_t)n; ++e) ug[e] = ug[e] * gfac;
  }
  return 0;
}

// First-order move of particles, ElementBase.h:253-273 + Points.h:288-351
// (used for the Ralston interim state, Convection.h:370-371).
extern "C" int o3o_points_move_euler(int n, double dt, double wt1, float* x, float* s, float* elong,
                          const float* u, const float* ug) {
  if (n < 0) return 1;
  for (int d = 0; d < 3; ++d)
    for (int i = 0; i < n; ++i) x[d * (size_t)n + i] += (float)dt * wt1 * u[d * (size_t)n + i];
  if (!ug) return 0;
  for (int i = 0; i < n; ++i) {
    float g[9], sv[3];
    for (int d = 0; d < 9; ++d) g[d] = ug[d * (size_t)n + i];
    for (int d = 0; d < 3; ++d) sv[d] = s[d * (size_t)n + i];
    float wdu[3];
    wdu[0] = sv[0] * g[0] + sv[1] * g[3] + sv[2] * g[6];
    wdu[1] = sv[0] * g[1] + sv[1] * g[4] + sv[2] * g[7];
    wdu[2] = sv[0] * g[2] + sv[1] * g[5] + sv[2] * g[8];
    const float cm = sv[0] * sv[0] + sv[1] * sv[1] + sv[2] * sv[2];
    if (cm > 0.0) {
      const float ef = (float)dt * wt1 * (sv[0] * wdu[0] + sv[1] * wdu[1] + sv[2] * wdu[2]) / cm;
      elong[i] *= 1.0 + ef;
    }
    for (int d = 0; d < 3; ++d) s[d * (size_t)n + i] = sv[d] + dt * wt1 * wdu[d];
  }
  return 0;
}

// Second-order combine, ElementBase.h:276-304 + Points.h:356-439 (Ralston final stage,
// Convection.h:401 with wt1=0.25, wt2=0.75).  u1 is overwritten with the combined
// velocity, like the reference's p1.move(..., p1, ..., p2).
extern "C" int o3o_points_move_rk2(int n, double dt, double wt1, float* u1, const float* ug1, double wt2,
                        const float* u2, const float* ug2, float* x, float* s, float* elong) {
  if (n < 0) return 1;
  for (int d = 0; d < 3; ++d)
    for (int i = 0; i < n; ++i)
      u1[d * (size_t)n + i] = wt1 * u1[d * (size_t)n + i] + wt2 * u2[d * (size_t)n + i];
  for (int d = 0; d < 3; ++d)
    for (int i = 0; i < n; ++i) x[d * (size_t)n + i] += (float)dt * u1[d * (size_t)n + i];
  if (!ug1 || !ug2) return 0;
  for (int i = 0; i < n; ++i) {
    float sv[3], g[9];
    for (int d = 0; d < 3; ++d) sv[d] = s[d * (size_t)n + i];
    for (int d = 0; d < 9; ++d) g[d] = ug1[d * (size_t)n + i];
    float w1[3], w2[3];
    w1[0] = sv[0] * g[0] + sv[1] * g[3] + sv[2] * g[6];
    w1[1] = sv[0] * g[1] + sv[1] * g[4] + sv[2] * g[7];
    w1[2] = sv[0] * g[2] + sv[1] * g[5] + sv[2] * g[8];
    for (int d = 0; d < 9; ++d) g[d] = ug2[d * (size_t)n + i];
    w2[0] = sv[0] * g[0] + sv[1] * g[3] + sv[2] * g[6];
    w2[1] = sv[0] * g[1] + sv[1] * g[4] + sv[2] * g[7];
    w2[2] = sv[0] * g[2] + sv[1] * g[5] + sv[2] * g[8];
    float wdu[3];
    for (int d = 0; d < 3; ++d) wdu[d] = wt1 * w1[d] + wt2 * w2[d];
    const float cm = sv[0] * sv[0] + sv[1] * sv[1] + sv[2] * sv[2];
    if (cm > 0.0) {
      const float ef = (float)dt * (sv[0] * wdu[0] + sv[1] * wdu[1] + sv[2] * wdu[2]) / cm;
      elong[i] *= 1.0 + ef;
    }
    for (int d = 0; d < 3; ++d) s[d * (size_t)n + i] = sv[d] + dt * wdu[d];
  }
  return 0;
}

// Icosahedral sphere, GeomHelper.cpp:41-91 + IglRefine.cpp:31-77 + igl upsample
// (lib/igl/upsample.cpp:17-105).  Writes nodes (component-major, 3*nn) and idx (3*np);
// nn = 10*4^L+2, np = 20*4^L.  Level-0 table: Icosahedron.h:27-63.
extern "C" int o3o_generate_ovoid(int levels, float rx, float ry, float rz, float* xout, uint32_t* idxout) {
  if (levels < 0 || levels > 10) return 1;
  const float a = 4.2532550e-01f, b = 2.6286550e-01f;
  std::vector<float> x = {a, 0, b,  0, b, a,  0, -b, a,  0, b, -a,  -a, 0, -b,  -b, a, 0,
                          0, -b, -a,  -a, 0, b,  -b, -a, 0,  a, 0, -b,  b, a, 0,  b, -a, 0};
  std::vector<uint32_t> f = {0, 1, 2,  3, 4, 5,  4, 3, 6,  7, 4, 8,  9, 3, 10,  9, 6, 3,  0, 9, 10,
                             7, 2, 1,  2, 8, 11,  3, 5, 10,  10, 5, 1,  6, 9, 11,  8, 4, 6,  0, 10, 1,
                             11, 0, 2,  7, 5, 4,  7, 1, 5,  6, 11, 8,  9, 0, 11,  2, 7, 8};
  for (int lev = 0; lev < levels; ++lev) {
    const size_t nv = x.size() / 3, nf = f.size() / 3;
    // edge (i,j) -> new vertex number, assigned in first-encounter order over
    // (face, edge j = (F(i,j), F(i,(j+1)%3))), upsample.cpp:38-55
    std::unordered_map<uint64_t, uint32_t> edge;
    edge.reserve(nf * 2);
    std::vector<uint32_t> ni(3 * nf);
    uint32_t counter = 0;
    for (size_t i = 0; i < nf; ++i) {
      for (int j = 0; j < 3; ++j) {
        const uint32_t p = f[3 * i + j], q = f[3 * i + (j + 1) % 3];
        const uint64_t key = ((uint64_t)std::min(p, q) << 32) | std::max(p, q);
        auto it = edge.find(key);
        if (it == edge.end()) { edge.emplace(key, counter); ni[3 * i + j] = counter++; }
        else ni[3 * i + j] = it->second;
      }
    }
    std::vector<float> nx(3 * (nv + counter));
    for (size_t e = 0; e < 3 * nv; ++e) nx[e] = x[e];
    // new vertex = 0.5*V(p) + 0.5*V(q) in double, rounded to float (IglRefine.cpp:60-64)
    for (size_t i = 0; i < nf; ++i) {
      for (int j = 0; j < 3; ++j) {
        const uint32_t p = f[3 * i + j], q = f[3 * i + (j + 1) % 3];
        const size_t v = nv + ni[3 * i + j];
        for (int d = 0; d < 3; ++d) nx[3 * v + d] = (float)(0.5 * (double)x[3 * p + d] + 0.5 * (double)x[3 * q + d]);
      }
    }
    // child faces (v0,m0,m2),(v1,m1,m0),(m0,m1,m2),(m1,v2,m2), upsample.cpp:84-101
    std::vector<uint32_t> nf4(12 * nf);
    for (size_t i = 0; i < nf; ++i) {
      const uint32_t v0 = f[3 * i], v1 = f[3 * i + 1], v2 = f[3 * i + 2];
      const uint32_t m0 = nv + ni[3 * i], m1 = nv + ni[3 * i + 1], m2 = nv + ni[3 * i + 2];
      const uint32_t t[12] = {v0, m0, m2, v1, m1, m0, m0, m1, m2, m1, v2, m2};
      for (int k = 0; k < 12; ++k) nf4[12 * i + k] = t[k];
    }
    // re-project to r = 0.5 (GeomHelper.cpp:57-66): rad from std::pow in double, then float
    for (size_t v = 0; v < nx.size() / 3; ++v) {
      const float rad = std::sqrt(std::pow(nx[3 * v], 2) + std::pow(nx[3 * v + 1], 2) + std::pow(nx[3 * v + 2], 2));
      const float scale = 0.5 / rad;
      nx[3 * v] *= scale;
      nx[3 * v + 1] *= scale;
      nx[3 * v + 2] *= scale;
    }
    x.swap(nx);
    f.swap(nf4);
  }
  const size_t nv = x.size() / 3;
  for (size_t v = 0; v < nv; ++v) {
    xout[v] = x[3 * v] * rx;
    xout[nv + v] = x[3 * v + 1] * ry;
    xout[2 * nv + v] = x[3 * v + 2] * rz;
  }
  std::memcpy(idxout, f.data(), f.size() * sizeof(uint32_t));
  return 0;
}

// Flop counts per interaction at the reference's own accounting: 54 + core for a
// vel+grad pair (Kernels.h:155 / :253 plus CoreFunc.h flops_t{v,p}_grads), 23 + core
// for a velocity-only pair (Kernels.h:49 / :93).  The Gaussian count is this
// project's own tally of its closed-form branch.
extern "C" int o3o_flops_per_pair(int core, int grads, int have_tr) {
  static const int tvg[5] = {9, 16, 14, 15, 13};
  static const int tpg[5] = {7, 14, 11, 13, 10};
  static const int tv[5] = {7, 10, 12, 11, 11};
  static const int tp[5] = {5, 8, 9, 9, 8};
  if (core < 0 || core > 4) return -1;
  if (grads) return 54 + (have_tr ? tvg[core] : tpg[core]);
  return 23 + (have_tr ? tv[core] : tp[core]);
}


// ---------------------------------------------------------------------------------------
// clear_inner_layer, method 1 (Reflect.h:446-656): push every point that lies below the
// cutoff layer of the closest panels out along their mean normal.  Called by
// Convection::advect_2nd_ralston after the interim move and after the combine
// (Convection.h:372,381,423-424) with cutoff_mult = 0.5/sqrt(2 pi).
namespace {

template <class S> S rdot(S a0, S a1, S a2, S b0, S b1, S b2) { return a0 * b0 + a1 * b1 + a2 * b2; }

// closest point of triangle (0,1,2) with unit normal n to t: Reflect.h:56-183
// (corners, then edges, then the interior prism; later tests overwrite earlier ones)
template <class S>
void closest_on_panel(S x0, S y0, S z0, S x1, S y1, S z1, S x2, S y2, S z2, S nx, S ny, S nz, S tx, S ty, S tz,
                      S* distsq, S* cx, S* cy, S* cz) {
  S best = (S)9.9e+9, px = 0, py = 0, pz = 0;
  const S a0 = tx - x0, a1 = ty - y0, a2 = tz - z0;
  const S b0 = tx - x1, b1 = ty - y1, b2 = tz - z1;
  const S c0 = tx - x2, c1 = ty - y2, c2 = tz - z2;
  const S da = rdot(a0, a1, a2, a0, a1, a2);
  if (da < best) { best = da; px = x0; py = y0; pz = z0; }
  const S db = rdot(b0, b1, b2, b0, b1, b2);
  if (db < best) { best = db; px = x1; py = y1; pz = z1; }
  const S dc = rdot(c0, c1, c2, c0, c1, c2);
  if (dc < best) { best = dc; px = x2; py = y2; pz = z2; }
  // edges: squared distance to the line |e x d|^2 / |e|^2, kept when the foot lies inside
  auto edge = [&](S e0, S e1, S e2, S d0, S d1, S d2, S ox, S oy, S oz) {
    const S inv = (S)(1.0 / rdot(e0, e1, e2, e0, e1, e2));
    const S r0 = e1 * d2 - e2 * d1, r1 = e2 * d0 - e0 * d2, r2 = e0 * d1 - e1 * d0;
    const S dl = rdot(r0, r1, r2, r0, r1, r2) * inv;
    if (dl < best) {
      const S t = rdot(e0, e1, e2, d0, d1, d2) * inv;
      if (0.0 < t && t < 1.0) {
        best = dl;
        px = ox + t * e0; py = oy + t * e1; pz = oz + t * e2;
      }
    }
  };
  const S e01x = x1 - x0, e01y = y1 - y0, e01z = z1 - z0;
  edge(e01x, e01y, e01z, a0, a1, a2, x0, y0, z0);
  const S e12x = x2 - x1, e12y = y2 - y1, e12z = z2 - z1;
  edge(e12x, e12y, e12z, b0, b1, b2, x1, y1, z1);
  const S e20x = x0 - x2, e20y = y0 - y2, e20z = z0 - z2;
  edge(e20x, e20y, e20z, c0, c1, c2, x2, y2, z2);
  // inside all three edge half-spaces: the foot of the normal
  auto side = [&](S e0, S e1, S e2, S d0, S d1, S d2) {
    const S i0 = ny * e2 - nz * e1, i1 = nz * e0 - nx * e2, i2 = nx * e1 - ny * e0;
    return rdot(d0, d1, d2, i0, i1, i2);
  };
  const S s01 = side(e01x, e01y, e01z, a0, a1, a2);
  const S s12 = side(e12x, e12y, e12z, b0, b1, b2);
  const S s20 = side(e20x, e20y, e20z, c0, c1, c2);
  if (s01 > 0.0 && s12 > 0.0 && s20 > 0.0) {
    const S h = rdot(a0, a1, a2, nx, ny, nz);
    best = h * h;
    px = tx - nx * h; py = ty - ny * h; pz = tz - nz * h;
  }
  *distsq = best; *cx = px; *cy = py; *cz = pz;
}

template <class S>
int clear_inner(int n, S* x, int nn, const S* nodes, int np, const uint32_t* idx, const S* norm, S cutoff_mult, S ips,
                int nthreads) {
  const S* nx = nodes; const S* ny = nodes + nn; const S* nz = nodes + 2 * (size_t)nn;
  const S* snx = norm; const S* sny = norm + np; const S* snz = norm + 2 * (size_t)np;
  S* tx = x; S* ty = x + n; S* tz = x + 2 * (size_t)n;
  const S eps = (S)(10.0 * std::numeric_limits<S>::epsilon());
  const S cut = cutoff_mult * ips;
  int pushed = 0;
#pragma omp parallel for num_threads(nthreads) reduction(+:pushed) schedule(dynamic, 64)
  for (int i = 0; i < n; ++i) {
    S mind = std::numeric_limits<S>::max();
    S mn[3] = {0, 0, 0}, mc[3] = {0, 0, 0};
    int nh = 0;
    for (int j = 0; j < np; ++j) {
      const uint32_t p0 = idx[3 * (size_t)j], p1 = idx[3 * (size_t)j + 1], p2 = idx[3 * (size_t)j + 2];
      S d2, cx, cy, cz;
      closest_on_panel<S>(nx[p0], ny[p0], nz[p0], nx[p1], ny[p1], nz[p1], nx[p2], ny[p2], nz[p2], snx[j], sny[j],
                          snz[j], tx[i], ty[i], tz[i], &d2, &cx, &cy, &cz);
      if (d2 < mind - eps) {
        // a new closest set: the running sums restart from this panel
        mind = d2;
        mn[0] = (S)0 + snx[j]; mn[1] = (S)0 + sny[j]; mn[2] = (S)0 + snz[j];
        mc[0] = (S)0 + cx; mc[1] = (S)0 + cy; mc[2] = (S)0 + cz;
        nh = 1;
      } else if (d2 < mind + eps) {
        mn[0] += snx[j]; mn[1] += sny[j]; mn[2] += snz[j];
        mc[0] += cx; mc[1] += cy; mc[2] += cz;
        ++nh;
      }
    }
    if (nh == 0) continue;
    // normalizeVec (MathHelper.h:186-192): 1/sqrt in double, rounded to S
    const S len = (S)(1.0 / std::sqrt(mn[0] * mn[0] + mn[1] * mn[1] + mn[2] * mn[2]));
    for (int d = 0; d < 3; ++d) mn[d] *= len;
    for (int d = 0; d < 3; ++d) mc[d] /= (S)nh;
    const S dx0 = tx[i] - mc[0], dx1 = ty[i] - mc[1], dx2 = tz[i] - mc[2];
    const S dotp = rdot(mn[0], mn[1], mn[2], dx0, dx1, dx2) - cut;
    if (dotp < 0.0) {
      tx[i] -= dotp * mn[0];
      ty[i] -= dotp * mn[1];
      tz[i] -= dotp * mn[2];
      ++pushed;
    }
  }
  return pushed;
}

}  // namespace

// x: [3][n] points (moved in place); returns the number pushed, or -1 on bad arguments
extern "C" int o3o_clear_inner_layer(int prec, int n, void* x, int nn, const void* nodes, int np, const uint32_t* idx,
                                     const void* norm, double cutoff_mult, double ips, int nthreads) {
  if (n < 0 || np < 1 || nn < 3) return -1;
  if (prec == 2)
    return clear_inner<double>(n, (double*)x, nn, (const double*)nodes, np, idx, (const double*)norm, cutoff_mult, ips,
                               nthreads);
  return clear_inner<float>(n, (float*)x, nn, (const float*)nodes, np, idx, (const float*)norm, (float)cutoff_mult,
                            (float)ips, nthreads);
}

// Surfaces::represent_as_particles, Surfaces.h:959-1008 (float S): centroid in float sums
// times (1./3.) in double, pushed by offset along the normal; strength ts (+ the reactive
// boundary-condition sheet when bc1/bc2 are given)
extern "C" int o3o_represent_as_particles(int nn, const float* nodes, int np, const uint32_t* idx, const float* area,
                                          const float* x1, const float* x2, const float* norm, float offset,
                                          const float* ts, const float* bc1, const float* bc2, float* px,
                                          float* ps) {
  if (np < 0 || nn < 0) return 1;
  for (int i = 0; i < np; ++i) {
    const uint32_t id0 = idx[3 * (size_t)i], id1 = idx[3 * (size_t)i + 1], id2 = idx[3 * (size_t)i + 2];
    for (int j = 0; j < 3; ++j) {
      const float* xj = nodes + (size_t)j * nn;
      float p = (float)((1. / 3.) * (xj[id0] + xj[id1] + xj[id2]));
      p += offset * norm[(size_t)j * np + i];
      px[(size_t)j * np + i] = p;
    }
    for (int j = 0; j < 3; ++j) {
      float v = ts[(size_t)j * np + i];
      if (bc1 && bc2) v += (bc1[i] * x1[(size_t)j * np + i] + bc2[i] * x2[(size_t)j * np + i]) * area[i];
      ps[(size_t)j * np + i] = v;
    }
  }
  return 0;
}

// ---------------------------------------------------------------------------------
// Split.h / Merge.h: particle split and merge (float S, the instantiation the simulation
// uses, Simulation.cpp:833 and Diffusion.h:298,355).
//
// Both operators find neighbours with a radius search over the particle positions as
// they were when the operator started (the reference builds a nanoflann kd-tree over a
// copy of them, Split.h:65-76, Merge.h:76-87).  The match criterion is nanoflann 1.3.1's
// (lib/nanoflann/nanoflann.hpp): d2 = ((q0-p0)^2 + (q1-p1)^2) + (q2-p2)^2 in float
// (L2_Adaptor::evalMetric, :383-405, query minus point) and d2 < radius (strict,
// RadiusResultSet::addPoint, :249-253).  Matches are visited in increasing d2
// (params.sorted, :1285-1286).  The default search is a uniform cell list that finds the
// same match set and takes equal d2 in increasing index, as the kernels do; the
// reference's order for such ties depends on its kd-tree layout, which OracleKdTree
// restates for the tie_order = 1 variant.
namespace {

struct OracleCells {
  double lo[3] = {0, 0, 0};
  double inv_h = 1.0;
  std::vector<uint64_t> keys;   // sorted cell keys
  std::vector<int> order;       // particle index per sorted key

  static constexpr int64_t kMaxCell = (1 << 21) - 1;

  void coords(float px, float py, float pz, int64_t c[3]) const {
    const double p[3] = {px, py, pz};
    for (int d = 0; d < 3; ++d) {
      double u = std::floor((p[d] - lo[d]) * inv_h);
      if (!(u >= 0.0)) u = 0.0;
      if (u > (double)kMaxCell) u = (double)kMaxCell;
      c[d] = (int64_t)u;
    }
  }
  static uint64_t key(int64_t cx, int64_t cy, int64_t cz) {
    return ((uint64_t)cx << 42) | ((uint64_t)cy << 21) | (uint64_t)cz;
  }
  // cell size: the largest search radius, enlarged so that float rounding of a match's
  // distance can never put it two cells away
  void build(int n, const float* x, const float* y, const float* z, double rmax) {
    const double h = rmax > 0.0 ? rmax * (1.0 + 1.0 / 1024.0) : 1.0;
    inv_h = 1.0 / h;
    for (int d = 0; d < 3; ++d) lo[d] = std::numeric_limits<double>::max();
    for (int i = 0; i < n; ++i) {
      lo[0] = std::min(lo[0], (double)x[i]);
      lo[1] = std::min(lo[1], (double)y[i]);
      lo[2] = std::min(lo[2], (double)z[i]);
    }
    std::vector<std::pair<uint64_t, int>> kv((size_t)n);
    for (int i = 0; i < n; ++i) {
      int64_t c[3];
      coords(x[i], y[i], z[i], c);
      kv[i] = {key(c[0], c[1], c[2]), i};
    }
    std::sort(kv.begin(), kv.end());
    keys.resize(n);
    order.resize(n);
    for (int i = 0; i < n; ++i) { keys[i] = kv[i].first; order[i] = kv[i].second; }
  }
  // (d2, j) for every j with d2(q - p_j) < thr, sorted by (d2, j)
  void search(float qx, float qy, float qz, float thr, const float* x, const float* y, const float* z,
              std::vector<std::pair<float, int>>& out) const {
    out.clear();
    int64_t c[3];
    coords(qx, qy, qz, c);
    for (int64_t cx = std::max<int64_t>(c[0] - 1, 0); cx <= std::min<int64_t>(c[0] + 1, kMaxCell); ++cx)
      for (int64_t cy = std::max<int64_t>(c[1] - 1, 0); cy <= std::min<int64_t>(c[1] + 1, kMaxCell); ++cy) {
        const uint64_t k0 = key(cx, cy, std::max<int64_t>(c[2] - 1, 0));
        const uint64_t k1 = key(cx, cy, std::min<int64_t>(c[2] + 1, kMaxCell));
        auto b = std::lower_bound(keys.begin(), keys.end(), k0);
        auto e = std::upper_bound(keys.begin(), keys.end(), k1);
        for (auto it = b; it != e; ++it) {
          const int j = order[it - keys.begin()];
          const float d0 = qx - x[j], d1 = qy - y[j], d2 = qz - z[j];
          float dist = d0 * d0;
          dist += d1 * d1;
          dist += d2 * d2;
          if (dist < thr) out.push_back({dist, j});
        }
      }
    std::sort(out.begin(), out.end());
  }
};

// The reference's own visiting order, for inputs with equal-distance neighbours: a
// restatement of nanoflann 1.3.1's KDTreeSingleIndexAdaptor as KDTreeEigenMatrixAdaptor
// instantiates it in Split.h:74-76 / Merge.h:85-87 (3 float dimensions, leaf_max_size 10,
// Eigen Index = int64 indices, L2_Adaptor metric, eps 0).
//   build:  vind = 0..n-1 (init_vind, :1308-1315); root box = the points' min/max
//           (computeBoundingBox, :1317-1336); divideTree (:858-908) with middleSplit_
//           (:910-957) and planeSplit (:968-1004), which permute vind in place;
//   search: findNeighbors + searchLevel (:1222-1242, :1346-1408): leaves in best-child-first
//           depth-first order, in-leaf order of vind, a subtree skipped when its incremental
//           float lower bound exceeds the radius; then radiusSearch's std::sort by distance
//           alone (:1279-1288, IndexDist_Sorter :208-214), which leaves ties as the
//           traversal and this C++ library's sort put them.
// Without ties the order is the cell list's; with ties only this reproduces the reference.
struct OracleKdTree {
  struct Node {
    int64_t left = 0, right = 0;  // leaf: its vind range
    int feat = -1;                // internal: divfeat; -1 marks a leaf
    float divlow = 0.f, divhigh = 0.f;
    int child1 = -1, child2 = -1;
  };
  static constexpr int64_t kLeafMax = 10;
  const float* pt[3] = {nullptr, nullptr, nullptr};
  std::vector<int64_t> vind;
  std::vector<Node> nodes;
  float root_lo[3] = {0, 0, 0}, root_hi[3] = {0, 0, 0};
  int root = -1;

  float at(int64_t j, int d) const { return pt[d][j]; }

  void build(int64_t n, const float* x, const float* y, const float* z) {
    pt[0] = x; pt[1] = y; pt[2] = z;
    vind.resize((size_t)n);
    for (int64_t i = 0; i < n; ++i) vind[(size_t)i] = i;
    nodes.clear();
    root = -1;
    if (n == 0) return;
    for (int d = 0; d < 3; ++d) root_lo[d] = root_hi[d] = at(0, d);
    for (int64_t k = 1; k < n; ++k)
      for (int d = 0; d < 3; ++d) {
        if (at(k, d) < root_lo[d]) root_lo[d] = at(k, d);
        if (at(k, d) > root_hi[d]) root_hi[d] = at(k, d);
      }
    root = divide(0, n, root_lo, root_hi);
  }

  void min_max(const int64_t* ind, int64_t count, int d, float& mn, float& mx) const {
    mn = mx = at(ind[0], d);
    for (int64_t i = 1; i < count; ++i) {
      const float v = at(ind[i], d);
      if (v < mn) mn = v;
      if (v > mx) mx = v;
    }
  }

  // two in-place passes: [0, lim1) below cut, [lim1, lim2) equal, [lim2, count) above;
  // "!right" ends a pass at position 0 as the unsigned-index guard does
  void plane_split(int64_t* ind, int64_t count, int d, float cut, int64_t& lim1, int64_t& lim2) const {
    int64_t left = 0, right = count - 1;
    for (;;) {
      while (left <= right && at(ind[left], d) < cut) ++left;
      while (right && left <= right && at(ind[right], d) >= cut) --right;
      if (left > right || !right) break;
      std::swap(ind[left], ind[right]);
      ++left;
      --right;
    }
    lim1 = left;
    right = count - 1;
    for (;;) {
      while (left <= right && at(ind[left], d) <= cut) ++left;
      while (right && left <= right && at(ind[right], d) > cut) --right;
      if (left > right || !right) break;
      std::swap(ind[left], ind[right]);
      ++left;
      --right;
    }
    lim2 = left;
  }

  // the cut dimension: among those whose box span is within a factor (1 - 1e-5) of the
  // largest, the first with the largest point spread; the cut at the box middle clamped
  // to the points' range; the split index nearest the middle that keeps equal values
  // together where it can
  void middle_split(int64_t* ind, int64_t count, int64_t& index, int& feat, float& cut, const float lo[3],
                    const float hi[3]) const {
    const float eps = 0.00001f;
    float max_span = hi[0] - lo[0];
    for (int d = 1; d < 3; ++d)
      if (hi[d] - lo[d] > max_span) max_span = hi[d] - lo[d];
    float max_spread = -1;
    feat = 0;
    for (int d = 0; d < 3; ++d) {
      if (hi[d] - lo[d] > (1 - eps) * max_span) {
        float mn, mx;
        min_max(ind, count, d, mn, mx);
        if (mx - mn > max_spread) {
          feat = d;
          max_spread = mx - mn;
        }
      }
    }
    const float mid = (lo[feat] + hi[feat]) / 2;
    float mn, mx;
    min_max(ind, count, feat, mn, mx);
    cut = mid < mn ? mn : (mid > mx ? mx : mid);
    int64_t lim1, lim2;
    plane_split(ind, count, feat, cut, lim1, lim2);
    index = lim1 > count / 2 ? lim1 : (lim2 < count / 2 ? lim2 : count / 2);
  }

  // returns the node; lo/hi come in as the box handed down (the parent's, cut at the
  // split value) and leave as the actual box of the node's points
  int divide(int64_t left, int64_t right, float lo[3], float hi[3]) {
    const int id = (int)nodes.size();
    nodes.emplace_back();
    if (right - left <= kLeafMax) {
      for (int d = 0; d < 3; ++d) lo[d] = hi[d] = at(vind[(size_t)left], d);
      for (int64_t k = left + 1; k < right; ++k)
        for (int d = 0; d < 3; ++d) {
          const float v = at(vind[(size_t)k], d);
          if (lo[d] > v) lo[d] = v;
          if (hi[d] < v) hi[d] = v;
        }
      nodes[id].left = left;
      nodes[id].right = right;
      return id;
    }
    int64_t idx;
    int feat;
    float cut;
    middle_split(vind.data() + left, right - left, idx, feat, cut, lo, hi);
    float llo[3], lhi[3], rlo[3], rhi[3];
    for (int d = 0; d < 3; ++d) { llo[d] = rlo[d] = lo[d]; lhi[d] = rhi[d] = hi[d]; }
    lhi[feat] = cut;
    const int c1 = divide(left, left + idx, llo, lhi);
    rlo[feat] = cut;
    const int c2 = divide(left + idx, right, rlo, rhi);
    Node& nd = nodes[id];
    nd.feat = feat;
    nd.child1 = c1;
    nd.child2 = c2;
    nd.divlow = lhi[feat];
    nd.divhigh = rlo[feat];
    for (int d = 0; d < 3; ++d) {
      lo[d] = std::min(llo[d], rlo[d]);
      hi[d] = std::max(lhi[d], rhi[d]);
    }
    return id;
  }

  void level(const float q[3], float radius, int node, float mindistsq, float dists[3],
             std::vector<std::pair<int64_t, float>>& out) const {
    const Node& nd = nodes[node];
    if (nd.feat < 0) {
      for (int64_t i = nd.left; i < nd.right; ++i) {
        const int64_t j = vind[(size_t)i];
        float dist = 0.f;
        for (int d = 0; d < 3; ++d) {
          const float diff = q[d] - at(j, d);
          dist += diff * diff;
        }
        if (dist < radius) out.push_back({j, dist});
      }
      return;
    }
    const int f = nd.feat;
    const float val = q[f];
    const float diff1 = val - nd.divlow, diff2 = val - nd.divhigh;
    int best, other;
    float cut_dist;
    if (diff1 + diff2 < 0) {
      best = nd.child1;
      other = nd.child2;
      cut_dist = (val - nd.divhigh) * (val - nd.divhigh);
    } else {
      best = nd.child2;
      other = nd.child1;
      cut_dist = (val - nd.divlow) * (val - nd.divlow);
    }
    level(q, radius, best, mindistsq, dists, out);
    const float dst = dists[f];
    mindistsq = mindistsq + cut_dist - dst;
    dists[f] = cut_dist;
    if (mindistsq * 1.0f <= radius) level(q, radius, other, mindistsq, dists, out);
    dists[f] = dst;
  }

  struct ByDistance {
    bool operator()(const std::pair<int64_t, float>& a, const std::pair<int64_t, float>& b) const {
      return a.second < b.second;
    }
  };

  // (d2, j) in the reference's visiting order
  void search(float qx, float qy, float qz, float radius, std::vector<std::pair<int64_t, float>>& scratch,
              std::vector<std::pair<float, int>>& out) const {
    scratch.clear();
    out.clear();
    if (root < 0) return;
    const float q[3] = {qx, qy, qz};
    float dists[3] = {0.f, 0.f, 0.f};
    float distsq = 0.f;
    for (int d = 0; d < 3; ++d) {
      if (q[d] < root_lo[d]) {
        dists[d] = (q[d] - root_lo[d]) * (q[d] - root_lo[d]);
        distsq += dists[d];
      }
      if (q[d] > root_hi[d]) {
        dists[d] = (q[d] - root_hi[d]) * (q[d] - root_hi[d]);
        distsq += dists[d];
      }
    }
    level(q, radius, root, distsq, dists, scratch);
    std::sort(scratch.begin(), scratch.end(), ByDistance());
    for (const auto& m : scratch) out.push_back({m.second, (int)m.first});
  }
};

// the neighbour search of both operators: the cell list (ties in increasing index) or the
// restated kd-tree (ties in the reference's order)
struct OracleSearch {
  bool kd = false;
  OracleCells cells;
  OracleKdTree tree;
  mutable std::vector<std::pair<int64_t, float>> scratch;

  void build(int n, const float* x, const float* y, const float* z, double rmax, int tie_order) {
    kd = tie_order != 0;
    if (kd) tree.build(n, x, y, z);
    else cells.build(n, x, y, z, rmax);
  }
  void search(float qx, float qy, float qz, float thr, const float* x, const float* y, const float* z,
              std::vector<std::pair<float, int>>& out) const {
    if (kd) tree.search(qx, qy, qz, thr, scratch, out);
    else cells.search(qx, qy, qz, thr, x, y, z, out);
  }
};

// get_core_coefficient<float> (Core.h:32-35): CoreType gaussian = 0, compactg = 1
float core_coefficient(int core) {
  return core == 0 ? (float)(1.0 / (M_PI * std::sqrt(M_PI))) : (float)0.23873241;
}

}  // namespace

// split_elongated<float> (Split.h:44-270).  Arrays have room for cap particles; the split
// ones are halved and moved in place and their children appended at [n, n + nsplit).
// tie_order 0 visits equal-distance neighbours in increasing index, 1 in the reference's
// kd-tree order.  Returns nsplit, or -1 when cap is too small or the arguments are bad.
extern "C" int o3o_split_elongated(int n, int cap, float* x, float* y, float* z, float* r, float* elong, float* sx,
                                   float* sy, float* sz, int core, float overlap, float threshold, int tie_order) {
  if (n < 0 || cap < n) return -1;
  int m = 0;
  double rmax = 0.0;
  for (int i = 0; i < n; ++i)
    if (elong[i] > threshold) {
      ++m;
      const float nom_sep = r[i] / overlap;
      rmax = std::max(rmax, (double)(float)(3.0 * nom_sep));
    }
  if (n + m > cap) return -1;
  if (m == 0) return 0;
  // the search runs on the positions before any split (the kd-tree's copy)
  const std::vector<float> px(x, x + n), py(y, y + n), pz(z, z + n);
  OracleSearch cells;
  cells.build(n, px.data(), py.data(), pz.data(), rmax, tie_order);
  const float coef = core_coefficient(core);
  std::vector<std::pair<float, int>> matches;
  int k = n;
  for (int i = 0; i < n; ++i) {
    if (!(elong[i] > threshold)) continue;
    // normalizeVec (MathHelper.h:186-192)
    float axis[3] = {sx[i], sy[i], sz[i]};
    const float len = (float)(1.0 / std::sqrt(axis[0] * axis[0] + axis[1] * axis[1] + axis[2] * axis[2]));
    for (int d = 0; d < 3; ++d) axis[d] *= len;
    const float nom_sep = r[i] / overlap;
    const float halfd = (float)(0.25 * elong[i] * nom_sep);
    const float search_rad = (float)(3.0 * nom_sep);
    const float thr = (float)std::pow(search_rad, 2);
    cells.search(x[i], y[i], z[i], thr, px.data(), py.data(), pz.data(), matches);
    float dVol = 0.0f;
    float curv[3] = {0.0f, 0.0f, 0.0f};
    for (const auto& mt : matches) {
      const int j = mt.second;
      const float dx[3] = {x[i] - x[j], y[i] - y[j], z[i] - z[j]};
      const float s0 = sx[j], s1 = sy[j], s2 = sz[j];
      const float factor = std::sqrt(mt.first / (r[j] * r[i])) * overlap;
      const float fac2 = (float)(coef * std::exp(-(std::pow(factor, 3))));
      const float tStr = std::sqrt(s0 * s0 + s1 * s1 + s2 * s2);
      const float wgt = axis[0] * s0 + axis[1] * s1 + axis[2] * s2;
      if (tStr > 1.e-15 && wgt > 0.0) {
        const float dsx = axis[0] - sx[j] / tStr;
        const float dsy = axis[1] - sy[j] / tStr;
        const float dsz = axis[2] - sz[j] / tStr;
        const float thisfac = wgt * fac2 * tStr;
        curv[0] += thisfac * (dx[1] * dsz - dx[2] * dsy);
        curv[1] += thisfac * (dx[2] * dsx - dx[0] * dsz);
        curv[2] += thisfac * (dx[0] * dsy - dx[1] * dsx);
        dVol += thisfac;
      }
    }
    x[k] = x[i] - halfd * axis[0];
    y[k] = y[i] - halfd * axis[1];
    z[k] = z[i] - halfd * axis[2];
    r[k] = r[i];
    elong[k] = (float)(0.5 * elong[i]);
    sx[k] = (float)(0.5 * sx[i]);
    sy[k] = (float)(0.5 * sy[i]);
    sz[k] = (float)(0.5 * sz[i]);
    x[i] += halfd * axis[0];
    y[i] += halfd * axis[1];
    z[i] += halfd * axis[2];
    elong[i] *= 0.5;
    sx[i] *= 0.5;
    sy[i] *= 0.5;
    sz[i] *= 0.5;
    if (dVol > 1e-15) {
      for (int d = 0; d < 3; ++d) curv[d] /= dVol;
      const float f = (float)(overlap * 0.398967 / r[i]);
      for (int d = 0; d < 3; ++d) curv[d] *= f;
      const float dsx = sy[i] * curv[2] - sz[i] * curv[1];
      const float dsy = sz[i] * curv[0] - sx[i] * curv[2];
      const float dsz = sx[i] * curv[1] - sy[i] * curv[0];
      sx[k] += dsx;
      sy[k] += dsy;
      sz[k] += dsz;
      sx[i] -= dsx;
      sy[i] -= dsy;
      sz[i] -= dsz;
    }
    ++k;
  }
  return m;
}

// merge_close_particles<float> (Merge.h:45-218): greedy merge in index order, then the
// survivors compacted in place; tie_order as for the split.  Returns the number removed, or
// -1 on bad arguments.
extern "C" int o3o_merge_close_particles(int n, float* x, float* y, float* z, float* sx, float* sy, float* sz,
                                         float* r, float overlap, float threshold, int adapt_radii, int tie_order) {
  if (n < 0) return -1;
  if (n == 0) return 0;
  const float initial_thresh = 0.5f;
  const float always_thresh = 0.1f;
  float meanstr = 0.0f;
  for (int i = 0; i < n; ++i) meanstr += std::sqrt(sx[i] * sx[i] + sy[i] * sy[i] + sz[i] * sz[i]);
  meanstr /= (float)n;
  double rmax = 0.0;
  for (int i = 0; i < n; ++i) rmax = std::max(rmax, (double)((r[i] / overlap) * initial_thresh));
  const std::vector<float> px(x, x + n), py(y, y + n), pz(z, z + n);
  OracleSearch cells;
  cells.build(n, px.data(), py.data(), pz.data(), rmax, tie_order);
  std::vector<char> erase((size_t)n, 0);
  std::vector<std::pair<float, int>> matches;
  for (int i = 0; i < n; ++i) {
    if (erase[i]) continue;
    const float nom_sep = r[i] / overlap;
    const float search_rad = nom_sep * initial_thresh;
    const float thr = (float)std::pow(search_rad, 2);
    cells.search(x[i], y[i], z[i], thr, px.data(), py.data(), pz.data(), matches);
    if (matches.size() <= 1) continue;
    for (const auto& mt : matches) {
      const int j = mt.second;
      if (j == i || erase[j]) continue;
      const float dist = std::sqrt(mt.first);
      if (!(dist < initial_thresh * r[j] / overlap)) continue;
      const float si = std::sqrt(sx[i] * sx[i] + sy[i] * sy[i] + sz[i] * sz[i]) + std::numeric_limits<float>::epsilon();
      const float so = std::sqrt(sx[j] * sx[j] + sy[j] * sy[j] + sz[j] * sz[j]) + std::numeric_limits<float>::epsilon();
      const float frac = so / (si + so);
      bool do_merge = false;
      const float min_rad = std::min(r[j], r[i]) / overlap;
      if (dist * frac * si < threshold * meanstr * min_rad) do_merge = true;
      if (dist < always_thresh * min_rad) do_merge = true;
      if (!do_merge) continue;
      const float omfrac = (float)(1.0 - frac);
      const float nx = x[i] * omfrac + x[j] * frac;
      const float ny = y[i] * omfrac + y[j] * frac;
      const float nz = z[i] * omfrac + z[j] * frac;
      x[i] = nx;
      y[i] = ny;
      z[i] = nz;
      if (adapt_radii) r[i] = (float)std::cbrt(omfrac * std::pow(r[i], 3) + frac * std::pow(r[j], 3));
      sx[i] = sx[i] + sx[j];
      sy[i] = sy[i] + sy[j];
      sz[i] = sz[i] + sz[j];
      erase[j] = 1;
    }
  }
  int copyto = 0;
  for (int i = 0; i < n; ++i) {
    if (erase[i]) continue;
    x[copyto] = x[i]; y[copyto] = y[i]; z[copyto] = z[i]; r[copyto] = r[i];
    sx[copyto] = sx[i]; sy[copyto] = sy[i]; sz[copyto] = sz[i];
    ++copyto;
  }
  return n - copyto;
}
