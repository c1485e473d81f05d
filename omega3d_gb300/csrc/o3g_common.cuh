// o3g_common.cuh -- shared host/device helpers of the sm_103a Biot-Savart / BEM library.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>
#include <string>

#include "../../include/o3dgpu.h"
#include "o3g_gauss_poly.h"

#include <type_traits>

namespace o3g {

// ------------------------------------------------------------------------------
// error plumbing (host)
void set_error(const char* what);
void set_error_cuda(const char* where, cudaError_t e);

#define O3G_CUDA_TRY(call)                                 \
  do {                                                     \
    cudaError_t e__ = (call);                              \
    if (e__ != cudaSuccess) {                              \
      ::o3g::set_error_cuda(#call, e__);                   \
      return O3G_ERR_CUDA;                                 \
    }                                                      \
  } while (0)

#define O3G_TRY(expr)                                      \
  do {                                                     \
    int32_t s__ = (expr);                                  \
    if (s__ != O3G_OK) return s__;                         \
  } while (0)

// ------------------------------------------------------------------------------
// per-(device, stream) grow-only device workspace.  Every call on a stream reuses the
// same buffer; calls on one stream are ordered by the stream, so they never overlap.
struct Workspace {
  char* base = nullptr;
  size_t cap = 0;
  size_t used = 0;
};
// Returns a workspace with at least `bytes` capacity for (current device, stream).
int32_t workspace_get(cudaStream_t stream, size_t bytes, Workspace** ws);
// Sub-allocation helper: 256-byte aligned carve-outs from a reserved workspace.
inline size_t align_up(size_t x, size_t a = 256) { return (x + a - 1) / a * a; }

struct Carve {
  char* base;
  size_t off = 0;
  explicit Carve(char* b) : base(b) {}
  template <class T> T* take(size_t count) {
    T* p = reinterpret_cast<T*>(base + off);
    off += align_up(count * sizeof(T));
    return p;
  }
};

// device facts (cached per device)
struct DeviceFacts {
  int device = -1;
  int num_sms = 0;
  int clock_khz = 0;
  int cc_major = 0, cc_minor = 0;
};
int32_t device_facts(DeviceFacts* f);

// resident blocks per SM of `kernel` at `block` threads (cached)
int32_t occupancy_blocks(const void* kernel, int block, int* nb);

// optional timing of the main kernel of a call
struct KernelTimer {
  cudaEvent_t start = nullptr, stop = nullptr;
  bool active = false;
  void begin(cudaStream_t s);
  void end(cudaStream_t s);
};
KernelTimer& thread_timer();

// count of kernels this thread has launched through the library
void note_launch(int n = 1);

// device allocations: every cudaMalloc / cudaMallocAsync the library makes goes through
// these, which count the successful ones for o3g_alloc_count
cudaError_t dev_alloc(void** p, size_t bytes);
cudaError_t dev_alloc_async(void** p, size_t bytes, cudaStream_t st);

// tensor-core update C -= A B (o3g_tcgemm.cu): column-major FP32 operands, TF32 products,
// FP32 sums; `at` holds tc_gemm_scratch_floats(m, k) floats, `err` is a device error word
size_t tc_gemm_scratch_floats(int m, int k);
int32_t tc_gemm_sub(int m, int n, int k, const float* A, long long lda, const float* B, long long ldb, float* C,
                    long long ldc, float* at, int* err, cudaStream_t st);

// wait test (o3g_debug_wait_test): when on, the bounded device-side waits of the BEM
// factorisation and solves and of the particle split wait for a condition nothing fulfils,
// with a short limit, so that they run out and the call returns O3G_ERR_TIMEOUT
bool wait_test_on();

// ------------------------------------------------------------------------------
// vector types
template <class T> struct V4;
template <> struct alignas(16) V4<float> { float x, y, z, w; };
template <> struct alignas(32) V4<double> { double x, y, z, w; };

// output pointer set: 3 velocity + 9 gradient component arrays
template <class T> struct OutPtrs { T* p[12]; };

// ------------------------------------------------------------------------------
// Core functions.  All cores share the form used by Kernels.h: velocity
//   u += r3 * (d x s),  grad += bbb * d (x) (d x s) + antisymmetric(r3 * s)
// where d = target - source.  `cst` is the combined core parameter of the pair:
//   RM, WL, GAUSS: sr^2 + tr^2;   EXP: sr^3 + tr^3;   V2: sr^4 + tr^4
// (CoreFunc.h:66-71, :266-274, :226-236, :318-330).
enum { CORE_RM = 0, CORE_WL = 1, CORE_EXP = 2, CORE_GAUSS = 3, CORE_V2 = 4 };

template <int C, class T>
__host__ __device__ __forceinline__ T core_param(T r) {
  if (C == CORE_EXP) return r * r * r;
  if (C == CORE_V2) { const T s2 = r * r; return s2 * s2; }
  return r * r;
}

// Gaussian core series coefficients c_n of G(q) = sqrt(2/pi) sum_{n>=1} c_n q^(n-1),
// c_n = (-1)^(n+1) / ((2n+1) 2^(n-1) (n-1)!): the Taylor expansion of
// [erf(rho/sqrt2) - sqrt(2/pi) rho exp(-rho^2/2)] / rho^3 in q = rho^2.
__host__ __device__ constexpr double gauss_coef(int n) {
  double c = 1.0 / (2.0 * n + 1.0);
  for (int k = 1; k < n; ++k) c /= (2.0 * k);
  return (n % 2 == 1) ? c : -c;
}
template <class T> struct GaussP;
template <> struct GaussP<float>  { static constexpr float  qfar = 48.0f; static constexpr int nterms = 9; };
template <> struct GaussP<double> { static constexpr double qfar = 90.0;  static constexpr int nterms = 17; };

// reciprocal square root: plain = hardware approximation (MUFU.RSQ, <= 2 ulp);
// accurate = one Newton-Raphson step on top (y' = y + y/2 (1 - x y^2)), ~1 ulp.
template <bool ACC>
__device__ __forceinline__ float rsq(float x) {
  float y = rsqrtf(x);
  if (ACC) {
    const float h = x * y;
    const float e = fmaf(-h, y, 1.0f);
    y = fmaf(0.5f * y, e, y);
  }
  return y;
}
template <bool ACC>
__device__ __forceinline__ double rsq(double x) { return rsqrt(x); }

// exp(x) for float x in [-20, 0], rounded once from a float-float value accurate to about
// 2^-35 relative: so it is the correctly rounded float in all but about 5 of 100,000
// arguments, and 1 ulp from it otherwise (beyond |x| = 22, n hi(ln2/32) below is no longer
// exact and the accuracy drops).  The plain FP32 exponential core evaluates the
// reference's 1 - exp(-x) with it: that form magnifies a difference of one ulp in exp(-x)
// by exp(-x) / (1 - exp(-x)) (1000x at x = 0.001), so the result tracks the host library's
// float exp (glibc's is within 0.502 ulp) only if this one is as close to correct rounding.
// Method: Tang's table-driven exponential (ACM TOMS 15(2), 1989): x = (32 k + j) ln2/32 + r
// with |r| <= ln2/64, exp(x) = 2^k 2^(j/32) exp(r); 2^(j/32) as a (hi, lo) float pair,
// ln2/32 split so that n hi is exact, exp(r) - 1 = r + r^2/2 + r^3/6 + r^4/24.
__device__ const __align__(16) float2 kExp2Frac[32] = {
    {1.000000000e+00f, 0.000000000e+00f},
    {1.021897197e+00f, -4.811559862e-08f},
    {1.044273734e+00f, 4.833470157e-08f},
    {1.067140460e+00f, -5.933751979e-08f},
    {1.090507746e+00f, -1.307753994e-08f},
    {1.114386797e+00f, -5.435540018e-08f},
    {1.138788581e+00f, 5.386222313e-08f},
    {1.163724899e+00f, -4.051441493e-08f},
    {1.189207077e+00f, 3.797635273e-08f},
    {1.215247393e+00f, -3.267394888e-08f},
    {1.241857767e+00f, 4.496838102e-08f},
    {1.269050956e+00f, 1.419333318e-09f},
    {1.296839595e+00f, -4.018999533e-08f},
    {1.325236678e+00f, -3.496373324e-08f},
    {1.354255557e+00f, -1.012334927e-08f},
    {1.383909941e+00f, -5.875577358e-08f},
    {1.414213538e+00f, 2.420323497e-08f},
    {1.445180774e+00f, 3.324199938e-08f},
    {1.476826191e+00f, -4.500898854e-08f},
    {1.509164453e+00f, -2.495937323e-08f},
    {1.542210817e+00f, 8.070904833e-09f},
    {1.575980902e+00f, -5.661025426e-08f},
    {1.610490322e+00f, 9.836217174e-09f},
    {1.645755529e+00f, -5.124972091e-08f},
    {1.681792855e+00f, -2.475532668e-08f},
    {1.718619347e+00f, -4.849617596e-08f},
    {1.756252170e+00f, -9.235770371e-09f},
    {1.794709086e+00f, -1.141504491e-08f},
    {1.834008098e+00f, -1.123927795e-08f},
    {1.874167681e+00f, -4.663005626e-08f},
    {1.915206552e+00f, 9.845328108e-09f},
    {1.957144141e+00f, -1.702180441e-08f}
};
__device__ __forceinline__ float exp_tang(float x) {
  const float nf = rintf(x * 4.616624069e+01f);        // 32 / ln2
  const int n = (int)nf;
  const float rh = fmaf(-nf, 2.166175842e-02f, x);     // x - n hi(ln2/32): exact
  const float rl = -nf * -9.090303479e-07f;            // - n lo(ln2/32)
  const float r = rh + rl;
  const float q = (r * r) * fmaf(r, fmaf(r, 4.166666791e-02f, 1.666666716e-01f), 0.5f);
  const float slo = rl + q;                            // exp(r) - 1 = rh + slo
  const float2 T = __ldg(&kExp2Frac[n & 31]);
  const float p = __fmul_rn(T.x, rh);                  // (no contraction: the error terms
  const float pe = fmaf(T.x, rh, -p);                  //  below need p and h rounded)
  const float h = __fadd_rn(T.x, p);                   // T.x rh = p + pe exactly; |p| < T.x:
  const float l0 = __fadd_rn(__fsub_rn(T.x, h), p);    // Fast2Sum, T.x + p = h + l0
  const float tail = fmaf(T.x, slo, T.y + T.y * rh);
  const float res = h + ((l0 + pe) + tail);
  return res * __int_as_float((127 + (n >> 5)) << 23);  // times 2^k, exact for normal results
}

// x / 3 correctly rounded, without a division: q = x RN(1/3), the residual x - 3 q exactly
// (one fma), then q + residual RN(1/3) rounded once (Markstein's correction step for a
// constant divisor, with the correctly rounded reciprocal 0x3EAAAAAB).  Checked against IEEE
// x / 3.0f for all 2^32 float inputs; zero is passed through to keep its sign.
__device__ __forceinline__ float div3_rn(float x) {
  const float y = 0.333333343f;
  const float q = __fmul_rn(x, y);
  const float r = __fmaf_rn(-q, 3.0f, x);
  return x == 0.0f ? x : __fmaf_rn(r, y, q);
}

// dx dx + dy dy + dz dz with every product and sum rounded, left to right: the reference's
// expression (Kernels.h:167-170) as an uncontracted build evaluates it
__device__ __forceinline__ float dist2_ref(float dx, float dy, float dz) {
  return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}
__device__ __forceinline__ double dist2_ref(double dx, double dy, double dz) {
  return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

__device__ __forceinline__ float dev_erf(float x) { return erff(x); }
__device__ __forceinline__ double dev_erf(double x) { return erf(x); }
__device__ __forceinline__ float dev_exp(float x) { return expf(x); }
__device__ __forceinline__ double dev_exp(double x) { return exp(x); }
__device__ __forceinline__ float dev_expm1(float x) { return expm1f(x); }
__device__ __forceinline__ double dev_expm1(double x) { return expm1(x); }
__device__ __forceinline__ float dev_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double dev_sqrt(double x) { return sqrt(x); }

// G(q) and D(q) = 2 G'(q) of the Gaussian core for q in [0, qfar] in FP32, from the
// piecewise polynomials of o3g_gauss_poly.h (Horner's rule in t = q s_j + o_j): branch-free,
// no erf/exp/division.
//
// Interval of q: j covers [j, j + 1) up to [47, 48], so j is the integer part of q (q >= 0)
// capped at the last; the fits are checked 1e-4 of their width beyond both ends.
__device__ __forceinline__ int gauss_interval(float q) { return min((int)q, kGaussPolyLast); }

// G(q) and D(q) by Horner's rule in t.  The table holds float pairs (s, o), (G_k, D_k),
// coefficient-major (pair e2 of interval j at e2 * N + j), so the lanes of a warp, whatever
// their intervals (neighbouring targets and sources give neighbouring q), read each pair
// from a few cache lines or banks, and the two chains advance together in packed FMAs (FFMA2: each
// lane rounds like FFMA, so G and D are bit-identical to two scalar chains).  `tab`: a
// block's shared-memory copy of kGaussPoly (stage_gauss_table, 8-byte aligned), or nullptr
// for the global table through the read-only cache.
__device__ __forceinline__ float2 gtab_ld2(const float* tab, int i2) {
  return tab ? reinterpret_cast<const float2*>(tab)[i2] : __ldg(reinterpret_cast<const float2*>(kGaussPoly) + i2);
}
__device__ __forceinline__ float gtab_ld(const float* tab, int i) { return tab ? tab[i] : __ldg(kGaussPoly + i); }
__device__ __forceinline__ void gauss_poly(float q, float& G, float& D, const float* tab = nullptr) {
  constexpr int N = kGaussPolyN;
  const int j = gauss_interval(q);   // pair e2 of this interval: e2 * N + j
  const float2 so = gtab_ld2(tab, j);
  const float t = fmaf(q, so.x, so.y);
  const float2 tt = make_float2(t, t);
  float2 gd = gtab_ld2(tab, N + j);
#pragma unroll
  for (int k = 1; k <= kGaussPolyDeg; ++k) gd = __ffma2_rn(gd, tt, gtab_ld2(tab, (1 + k) * N + j));
  G = gd.x;
  D = gd.y;
}
__device__ __forceinline__ float gauss_poly_g(float q, const float* tab = nullptr) {
  constexpr int N = kGaussPolyN;
  const int j = gauss_interval(q);
  const float2 so = gtab_ld2(tab, j);
  const float t = fmaf(q, so.x, so.y);
  float g = gtab_ld(tab, 2 * (N + j));
#pragma unroll
  for (int k = 1; k <= kGaussPolyDeg; ++k) g = fmaf(g, t, gtab_ld(tab, 2 * ((1 + k) * N + j)));
  return g;
}
// copies the polynomial table into a block's shared array (all threads call; synchronise
// before the first use)
__device__ __forceinline__ void stage_gauss_table(float* s) {
  for (int i = threadIdx.x; i < kGaussPolyStride * kGaussPolyN; i += blockDim.x) s[i] = kGaussPoly[i];
}

// Gaussian core with gradient factor (the project's own definition, see o3dgpu.h):
// r3 = G(q) / sigma^3, bbb = 2 G'(q) / sigma^5 with q = d^2 / sigma^2; the singular kernel
// beyond q = qfar.  FP32 evaluates G from the polynomials above; FP64 (the comparator) from
// the Taylor series for q < 1 and the closed form with erf/exp beyond.
template <bool ACC, class T>
__device__ __forceinline__ void gauss_g(T distsq, T sig2, T& r3, T& bbb, const float* tab = nullptr) {
  const T c = T(0.79788456080286535588);  // sqrt(2/pi)
  if (distsq > GaussP<T>::qfar * sig2) {   // q > qfar without the division
    const T rs = rsq<ACC>(distsq);
    const T rs2 = rs * rs;
    r3 = rs2 * rs;
    bbb = T(-3.0) * r3 * rs2;
    return;
  }
  if constexpr (std::is_same<T, float>::value) {
    const float rsg = rsq<ACC>(sig2);
    const float rsg2 = rsg * rsg;
    float G, D;
    gauss_poly(distsq * rsg2, G, D, tab);
    const float isig3 = rsg2 * rsg;
    r3 = G * isig3;
    bbb = D * isig3 * rsg2;
    return;
  }
  const T q = distsq / sig2;
  if (q < T(1.0)) {
    T g = T(0), gp = T(0);
#pragma unroll
    for (int n = GaussP<T>::nterms; n >= 1; --n) g = g * q + T(gauss_coef(n));
#pragma unroll
    for (int n = GaussP<T>::nterms; n >= 2; --n) gp = gp * q + T((n - 1) * gauss_coef(n));
    const T rsg = rsq<ACC>(sig2);
    const T isig3 = rsg * rsg * rsg;
    r3 = c * g * isig3;
    bbb = T(2.0) * c * gp * isig3 * (rsg * rsg);
  } else {
    const T rs = rsq<ACC>(distsq);
    const T rs2 = rs * rs;
    const T rho = dev_sqrt(q);
    const T e = dev_exp(T(-0.5) * q);
    const T g = dev_erf(rho * T(0.70710678118654752440)) - c * rho * e;
    const T rsg = rsq<ACC>(sig2);
    r3 = g * rs2 * rs;
    bbb = (c * e * (rsg * rsg * rsg) - T(3.0) * r3) * rs2;
  }
}
template <bool ACC, class T>
__device__ __forceinline__ T gauss_v(T distsq, T sig2, const float* tab = nullptr) {
  const T c = T(0.79788456080286535588);
  if (distsq > GaussP<T>::qfar * sig2) {
    const T rs = rsq<ACC>(distsq);
    return rs * rs * rs;
  }
  if constexpr (std::is_same<T, float>::value) {
    const float rsg = rsq<ACC>(sig2);
    const float rsg2 = rsg * rsg;
    return gauss_poly_g(distsq * rsg2, tab) * (rsg2 * rsg);
  }
  const T q = distsq / sig2;
  if (q < T(1.0)) {
    T g = T(0);
#pragma unroll
    for (int n = GaussP<T>::nterms; n >= 1; --n) g = g * q + T(gauss_coef(n));
    const T rsg = rsq<ACC>(sig2);
    return c * g * rsg * rsg * rsg;
  } else {
    const T rs = rsq<ACC>(distsq);
    const T rho = dev_sqrt(q);
    const T e = dev_exp(T(-0.5) * q);
    const T g = dev_erf(rho * T(0.70710678118654752440)) - c * rho * e;
    return g * rs * rs * rs;
  }
}

// r3 and bbb of one pair; dx,dy,dz = target - source; cst as above.
template <int C, bool ACC, class T>
__device__ __forceinline__ void core_g(T dx, T dy, T dz, T cst, T& r3, T& bbb, const float* gtab = nullptr) {
  if (C == CORE_RM) {
    // CoreFunc.h:66-71: r2 = d^2 + sr^2 + tr^2, r3 = r2^-1.5, bbb = -3 r3 / r2
    const T r2 = fma(dx, dx, fma(dy, dy, fma(dz, dz, cst)));
    const T rs = rsq<ACC>(r2);
    const T rs2 = rs * rs;
    r3 = rs2 * rs;
    bbb = T(-3.0) * r3 * rs2;
  } else if (C == CORE_WL) {
    // CoreFunc.h:266-274: d2 = d^2 + r^2; r3 = (d^2 + 2.5 r^2) d2^-2.5; bbb = 2 d2^-2.5 - 5 r3 / d2
    const T distsq = fma(dx, dx, fma(dy, dy, dz * dz));
    const T d2 = distsq + cst;
    const T d2top = fma(T(2.5), cst, distsq);
    const T rs = rsq<ACC>(d2);
    const T rs2 = rs * rs;
    const T dn5 = rs2 * rs2 * rs;
    r3 = d2top * dn5;
    bbb = fma(T(-5.0) * r3, rs2, T(2.0) * dn5);
  } else if (C == CORE_EXP) {
    // CoreFunc.h:226-236 with the branches of exp_cond / exp_bbb (:119-174).  The core
    // jumps by reld3/2 (5e-4) where it switches form at reld3 = 0.001, so distsq is formed
    // in the reference's operation order, each operation rounded (Kernels.h:167-170), and
    // each branch is taken where the reference's build of the same precision takes it.
    // Plain FP32 also evaluates the middle branch as the reference does (REF).
    constexpr bool REF = !ACC && std::is_same<T, float>::value;
    const T distsq = dist2_ref(dx, dy, dz);
    const T dist = dev_sqrt(distsq);
    const T corefac = T(1.0) / cst;
    const T d3 = distsq * dist;
    const T reld3 = d3 * corefac;
    const T ood3 = T(1.0) / d3;
    // the thresholds are the float literals 16.0f and 0.001f of the reference's exp_cond /
    // exp_bbb (CoreFunc.h:121-132, :164-177), also in its double build
    if (reld3 > T(16.0f)) {
      r3 = ood3;
      bbb = T(-3.0) * r3 / distsq;
    } else if (reld3 < T(0.001f)) {
      r3 = corefac;
      bbb = T(-1.5) * dist * r3 * r3;
    } else if (REF) {
      // plain FP32: the reference's own float arithmetic, 1 - exp(-x) and corefac exp(-x)
      // (exp_cond / exp_bbb, CoreFunc.h:127-128, :175-177), exp nearly correctly rounded
      const float e = exp_tang((float)-reld3);
      const float r3f = __fmul_rn((float)ood3, __fsub_rn(1.0f, e));
      r3 = (T)r3f;
      bbb = (T)(__fdiv_rn(__fmul_rn(3.0f, __fsub_rn(__fmul_rn((float)corefac, e), r3f)), (float)distsq));
    } else {
      // compensated and FP64: 1 - exp(-x) through expm1, which keeps the digits that
      // float 1 - exp(-x) loses (about eps/x) near the core
      const T em1 = dev_expm1(-reld3);
      r3 = ood3 * (-em1);
      bbb = T(3.0) * (corefac * (em1 + T(1.0)) - r3) / distsq;
    }
  } else if (C == CORE_V2) {
    // CoreFunc.h:318-330: denom = d^4 + sr^4 + tr^4; r3 = denom^-0.75; bbb = -3 r3 denom^-0.5
    const T distsq = fma(dx, dx, fma(dy, dy, dz * dz));
    const T denom = fma(distsq, distsq, cst);
    const T rs = rsq<ACC>(denom);
    r3 = rs * dev_sqrt(rs);
    bbb = T(-3.0) * r3 * rs;
  } else {
    const T distsq = fma(dx, dx, fma(dy, dy, dz * dz));
    gauss_g<ACC, T>(distsq, cst, r3, bbb, gtab);
  }
}

// r3 only (velocity-only kernels): CoreFunc.h:48-52, :246-252, :202-209, :297-304
template <int C, bool ACC, class T>
__device__ __forceinline__ T core_v(T dx, T dy, T dz, T cst, const float* gtab = nullptr) {
  if (C == CORE_RM) {
    const T r2 = fma(dx, dx, fma(dy, dy, fma(dz, dz, cst)));
    const T rs = rsq<ACC>(r2);
    return rs * rs * rs;
  } else if (C == CORE_WL) {
    const T distsq = fma(dx, dx, fma(dy, dy, dz * dz));
    const T d2 = distsq + cst;
    const T rs = rsq<ACC>(d2);
    const T rs2 = rs * rs;
    return fma(T(2.5), cst, distsq) * (rs2 * rs2 * rs);
  } else if (C == CORE_EXP) {
    constexpr bool REF = !ACC && std::is_same<T, float>::value;   // as in core_g
    const T distsq = dist2_ref(dx, dy, dz);
    const T dist = dev_sqrt(distsq);
    const T ood3 = T(1.0) / (distsq * dist);
    const T corefac = T(1.0) / cst;
    const T reld3 = corefac / ood3;
    if (reld3 > T(16.0f)) return ood3;
    if (reld3 < T(0.001f)) return corefac;
    if (REF) return (T)__fmul_rn((float)ood3, __fsub_rn(1.0f, exp_tang((float)-reld3)));
    return ood3 * (-dev_expm1(-reld3));
  } else if (C == CORE_V2) {
    const T distsq = fma(dx, dx, fma(dy, dy, dz * dz));
    const T rs = rsq<ACC>(fma(distsq, distsq, cst));
    return rs * dev_sqrt(rs);
  } else {
    const T distsq = fma(dx, dx, fma(dy, dy, dz * dz));
    return gauss_v<ACC, T>(distsq, cst, gtab);
  }
}

}  // namespace o3g
