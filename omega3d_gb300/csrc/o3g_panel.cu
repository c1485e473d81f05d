// o3g_panel.cu -- adaptive panel kernels: panels_affect_points (Influence.h:557-1099,
// rkernel_2vs_0pg / rkernel_2vs_0p, Kernels.h:1028-1211) and points_affect_panels
// (Influence.h:1107-1221, the same kernel used backwards for the BEM right-hand side).
//
// Subdivision follows the reference per pair: a (sub)triangle is evaluated as one
// singular vortex+source point at its centroid when dist(target, centroid) >
// 4*sqrt(area) or its level reached maxlev, otherwise it splits into the four children
// {0,1,3},{1,2,4},{1,4,3},{3,4,5} of its corner/midpoint list (Kernels.h:1085-1092),
// each with a quarter of the strength and area, visited depth first in that order.
// The well-separation test is computed with the reference's operation order and no
// fused multiply-adds (__fmul_rn/__fadd_rn), so every split decision is the reference's.
// With the source core radius 0 every core of CoreFunc.h reduces to the singular kernel,
// so the leaves here use 1/d^3 for all cores.
//
// Layout: per panel a 32-byte far record (centroid, 4*sqrt(area), absolute strength,
// source strength) staged in shared memory, and a 48-byte near record (corners, area)
// read from global memory only when a panel must be subdivided.
#include "o3g_common.cuh"

namespace o3g {

constexpr int kPB = 128;          // threads per block / panels (or particles) per tile
constexpr int kMaxLev = 6;        // deepest subdivision accepted by the C-ABI
constexpr int kStack = 3 * kMaxLev + 1;

struct PanelFar {
  float4 c;   // centroid x, y, z; 4*sqrt(area)
  float4 s;   // absolute strength x, y, z (sheet * area); source strength * area
};
struct PanelNear {
  float4 a;   // x0 y0 z0 x1
  float4 b;   // y1 z1 x2 y2
  float4 d;   // z2, area, -, -
};

struct Tri {
  float x0, y0, z0, x1, y1, z1, x2, y2, z2, area;
  int lev;
};

// centroid and well-separation test in the reference's order (Kernels.h:1141-1158)
__device__ __forceinline__ void centroid(const Tri& t, float& cx, float& cy, float& cz) {
  cx = div3_rn(__fadd_rn(__fadd_rn(t.x0, t.x1), t.x2));
  cy = div3_rn(__fadd_rn(__fadd_rn(t.y0, t.y1), t.y2));
  cz = div3_rn(__fadd_rn(__fadd_rn(t.z0, t.z1), t.z2));
}
__device__ __forceinline__ float dist_rn(float tx, float ty, float tz, float cx, float cy, float cz) {
  const float dx = __fsub_rn(tx, cx), dy = __fsub_rn(ty, cy), dz = __fsub_rn(tz, cz);
  return __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
}
__device__ __forceinline__ bool well_sep(float tx, float ty, float tz, float cx, float cy, float cz, float area) {
  return dist_rn(tx, ty, tz, cx, cy, cz) > __fmul_rn(__fsqrt_rn(area), 4.0f);
}

// singular vortex+source point at (cx,cy,cz) with strength (sx,sy,sz), ss on target t:
// kernel_0vs_0pg with sr = 0 (Kernels.h:294-345); a[0..2] velocity, a[3..11] gradient
template <bool GRADS, bool SRC, bool ACC = false>
__device__ __forceinline__ void leaf(float tx, float ty, float tz, float cx, float cy, float cz, float sx, float sy,
                                     float sz, float ss, float* a) {
  const float dx = tx - cx, dy = ty - cy, dz = tz - cz;
  const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
  const float rs = rsq<ACC>(r2);
  const float rs2 = rs * rs;
  const float r3 = rs2 * rs;
  float cxw = dz * sy - dy * sz;
  float cyw = dx * sz - dz * sx;
  float czw = dy * sx - dx * sy;
  if (SRC) {
    a[0] = fmaf(r3, fmaf(dx, ss, cxw), a[0]);
    a[1] = fmaf(r3, fmaf(dy, ss, cyw), a[1]);
    a[2] = fmaf(r3, fmaf(dz, ss, czw), a[2]);
  } else {
    a[0] = fmaf(r3, cxw, a[0]);
    a[1] = fmaf(r3, cyw, a[1]);
    a[2] = fmaf(r3, czw, a[2]);
  }
  if (GRADS) {
    const float bbb = -3.0f * r3 * rs2;
    if (SRC) {
      // bbb * d (x) (s x d + ss d) + ss r3 I
      cxw = fmaf(dx, ss, cxw);
      cyw = fmaf(dy, ss, cyw);
      czw = fmaf(dz, ss, czw);
    }
    cxw *= bbb; cyw *= bbb; czw *= bbb;
    const float rsx = r3 * sx, rsy = r3 * sy, rsz = r3 * sz;
    const float dss = SRC ? ss * r3 : 0.f;
    a[3] = fmaf(dx, cxw, a[3] + dss);
    a[4] = fmaf(dx, cyw, a[4] + rsz);
    a[5] = fmaf(dx, czw, a[5] - rsy);
    a[6] = fmaf(dy, cxw, a[6] - rsz);
    a[7] = fmaf(dy, cyw, a[7] + dss);
    a[8] = fmaf(dy, czw, a[8] + rsx);
    a[9] = fmaf(dz, cxw, a[9] + rsy);
    a[10] = fmaf(dz, cyw, a[10] - rsx);
    a[11] = fmaf(dz, czw, a[11] + dss);
  }
}

// depth-first subdivision of a triangle that failed the level-0 test
template <bool GRADS, bool SRC, bool ACC = false>
__device__ __noinline__ void subdivide(float tx, float ty, float tz, const Tri& root, float sx, float sy, float sz,
                                       float ss, int maxlev, float* a) {
  Tri st[kStack];
  int sp = 0;
  // push the children of `t` in reverse so child 0 is visited first
  auto push_children = [&](const Tri& t) {
    const float mx01 = 0.5f * (t.x0 + t.x1), my01 = 0.5f * (t.y0 + t.y1), mz01 = 0.5f * (t.z0 + t.z1);
    const float mx02 = 0.5f * (t.x0 + t.x2), my02 = 0.5f * (t.y0 + t.y2), mz02 = 0.5f * (t.z0 + t.z2);
    const float mx12 = 0.5f * (t.x1 + t.x2), my12 = 0.5f * (t.y1 + t.y2), mz12 = 0.5f * (t.z1 + t.z2);
    const float ca = 0.25f * t.area;
    const int cl = t.lev + 1;
    // corner/midpoint list {v0, m01, v1, m02, m12, v2}; children {0,1,3},{1,2,4},{1,4,3},{3,4,5}
    st[sp++] = Tri{mx02, my02, mz02, mx12, my12, mz12, t.x2, t.y2, t.z2, ca, cl};         // {3,4,5}
    st[sp++] = Tri{mx01, my01, mz01, mx12, my12, mz12, mx02, my02, mz02, ca, cl};         // {1,4,3}
    st[sp++] = Tri{mx01, my01, mz01, t.x1, t.y1, t.z1, mx12, my12, mz12, ca, cl};         // {1,2,4}
    st[sp++] = Tri{t.x0, t.y0, t.z0, mx01, my01, mz01, mx02, my02, mz02, ca, cl};         // {0,1,3}
  };
  push_children(root);
  while (sp > 0) {
    const Tri t = st[--sp];
    float cx, cy, cz;
    centroid(t, cx, cy, cz);
    if (t.lev >= maxlev || well_sep(tx, ty, tz, cx, cy, cz, t.area)) {
      // 0.25^lev, exact powers of two (the reference scales by 0.25 per split, Kernels.h:1072-1075)
      const float f = __int_as_float((127 - 2 * t.lev) << 23);
      leaf<GRADS, SRC, ACC>(tx, ty, tz, cx, cy, cz, sx * f, sy * f, sz * f, ss * f, a);
    } else if (sp + 4 <= kStack) {
      push_children(t);
    }
  }
}

// error-free a + b = s + e (Knuth's two-sum)
__device__ __forceinline__ void two_sum_f(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// compensated mode: fold the plain partial sums of one tile into (hi, lo) and restart them
template <int NC>
__device__ __forceinline__ void fold_tile(float* a, float* hi, float* lo) {
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    float sum, err;
    two_sum_f(hi[c], a[c], sum, err);
    hi[c] = sum;
    lo[c] += err;
    a[c] = 0.f;
  }
}

__global__ void k_pack_panels(int np, const float* __restrict__ nx, const float* __restrict__ ny,
                              const float* __restrict__ nz, const uint32_t* __restrict__ idx,
                              const float* __restrict__ area, const float* __restrict__ tsx,
                              const float* __restrict__ tsy, const float* __restrict__ tsz,
                              const float* __restrict__ sss, int np_pad, PanelFar* far, PanelNear* nearr) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= np_pad) return;
  PanelFar f;
  PanelNear n;
  if (j < np) {
    const uint32_t p0 = idx[3 * (size_t)j], p1 = idx[3 * (size_t)j + 1], p2 = idx[3 * (size_t)j + 2];
    Tri t{nx[p0], ny[p0], nz[p0], nx[p1], ny[p1], nz[p1], nx[p2], ny[p2], nz[p2], area[j], 0};
    float cx, cy, cz;
    centroid(t, cx, cy, cz);
    const float sa = area[j];
    // sheet strength = ts / area (Influence.h:958), absolute again at level 0 (Kernels.h:1040-1046)
    const float sx = __fmul_rn(__fdiv_rn(tsx[j], sa), sa);
    const float sy = __fmul_rn(__fdiv_rn(tsy[j], sa), sa);
    const float sz = __fmul_rn(__fdiv_rn(tsz[j], sa), sa);
    const float s3 = sss ? __fmul_rn(sss[j], sa) : 0.f;
    f.c = make_float4(cx, cy, cz, __fmul_rn(__fsqrt_rn(sa), 4.0f));
    f.s = make_float4(sx, sy, sz, s3);
    n.a = make_float4(t.x0, t.y0, t.z0, t.x1);
    n.b = make_float4(t.y1, t.z1, t.x2, t.y2);
    n.d = make_float4(t.z2, sa, 0.f, 0.f);
  } else {
    // a padding panel with zero strength far away contributes exactly zero
    f.c = make_float4(1.0e18f, 1.0e18f, 1.0e18f, 0.f);
    f.s = make_float4(0.f, 0.f, 0.f, 0.f);
    n.a = make_float4(1.0e18f, 1.0e18f, 1.0e18f, 1.0e18f);
    n.b = make_float4(1.0e18f, 1.0e18f, 1.0e18f, 1.0e18f);
    n.d = make_float4(1.0e18f, 1.0f, 0.f, 0.f);
  }
  far[j] = f;
  nearr[j] = n;
}

template <bool GRADS, bool SRC, bool ACC>
__global__ void __launch_bounds__(kPB) k_panpt(const PanelFar* __restrict__ far, const PanelNear* __restrict__ nearr,
                                               int ntiles, int tiles_per_split, int maxlev, int nt,
                                               const float* __restrict__ tx, const float* __restrict__ ty,
                                               const float* __restrict__ tz, float* partial, int nt_pad,
                                               OutPtrs<float> out) {
  constexpr int NC = GRADS ? 12 : 3;
  constexpr int NH = ACC ? NC : 1;
  __shared__ PanelFar sf[kPB];
  const int i = blockIdx.x * kPB + threadIdx.x;
  const bool live = i < nt;
  const float px = live ? tx[i] : 0.f, py = live ? ty[i] : 0.f, pz = live ? tz[i] : 0.f;
  float a[12];
#pragma unroll
  for (int c = 0; c < 12; ++c) a[c] = 0.f;
  float hi[NH], lo[NH];
#pragma unroll
  for (int c = 0; c < NH; ++c) { hi[c] = 0.f; lo[c] = 0.f; }
  const int t0 = blockIdx.y * tiles_per_split;
  const int t1 = min(ntiles, t0 + tiles_per_split);
  for (int tile = t0; tile < t1; ++tile) {
    __syncthreads();
    sf[threadIdx.x] = far[(size_t)tile * kPB + threadIdx.x];
    __syncthreads();
#pragma unroll 2
    for (int jj = 0; jj < kPB; ++jj) {
      const PanelFar f = sf[jj];
      if (maxlev == 0 || dist_rn(px, py, pz, f.c.x, f.c.y, f.c.z) > f.c.w) {
        leaf<GRADS, SRC, ACC>(px, py, pz, f.c.x, f.c.y, f.c.z, f.s.x, f.s.y, f.s.z, f.s.w, a);
      } else {
        const PanelNear nr = nearr[(size_t)tile * kPB + jj];
        const Tri root{nr.a.x, nr.a.y, nr.a.z, nr.a.w, nr.b.x, nr.b.y, nr.b.z, nr.b.w, nr.d.x, nr.d.y, 0};
        // the out-of-line subdivision works on a copy of the sums (in local memory); handing
        // it `a` itself would put every far pair's sums in local memory too
        float as[12];
#pragma unroll
        for (int c = 0; c < 12; ++c) as[c] = a[c];
        subdivide<GRADS, SRC, ACC>(px, py, pz, root, f.s.x, f.s.y, f.s.z, f.s.w, maxlev, as);
#pragma unroll
        for (int c = 0; c < 12; ++c) a[c] = as[c];
      }
    }
    if (ACC) fold_tile<NC>(a, hi, lo);
  }
  if (partial) {
    if (ACC) {
      float* base = partial + (size_t)blockIdx.y * 2 * NC * nt_pad;
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        base[(size_t)c * nt_pad + i] = hi[c];
        base[(size_t)(NC + c) * nt_pad + i] = lo[c];
      }
    } else {
      float* base = partial + (size_t)blockIdx.y * NC * nt_pad;
#pragma unroll
      for (int c = 0; c < NC; ++c) base[(size_t)c * nt_pad + i] = a[c];
    }
  } else if (live) {
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      if (ACC) out.p[c][i] = (float)((double)out.p[c][i] + ((double)hi[c] + (double)lo[c]));
      else     out.p[c][i] += a[c];
    }
  }
}

// points_affect_panels: thread per target panel, sweep particle tiles; the panel is the
// subdivided "source" with the particle's strength, evaluated at the particle, negated.
template <bool ACC>
__global__ void __launch_bounds__(kPB) k_ptpan(const PanelFar* __restrict__ far, const PanelNear* __restrict__ nearr,
                                               int np, const float4* __restrict__ ppos, int ntiles,
                                               int tiles_per_split, int maxlev, float* partial, int np_pad,
                                               OutPtrs<float> out) {
  constexpr int NH = ACC ? 3 : 1;
  __shared__ float4 sp[kPB], sw[kPB];
  const int i = blockIdx.x * kPB + threadIdx.x;
  const PanelFar f = far[i];
  const PanelNear nr = nearr[i];
  float a[12];
#pragma unroll
  for (int c = 0; c < 3; ++c) a[c] = 0.f;
  float hi[NH], lo[NH];
#pragma unroll
  for (int c = 0; c < NH; ++c) { hi[c] = 0.f; lo[c] = 0.f; }
  const int t0 = blockIdx.y * tiles_per_split;
  const int t1 = min(ntiles, t0 + tiles_per_split);
  for (int tile = t0; tile < t1; ++tile) {
    __syncthreads();
    sp[threadIdx.x] = ppos[2 * ((size_t)tile * kPB + threadIdx.x)];
    sw[threadIdx.x] = ppos[2 * ((size_t)tile * kPB + threadIdx.x) + 1];
    __syncthreads();
#pragma unroll 2
    for (int jj = 0; jj < kPB; ++jj) {
      const float4 p = sp[jj], w = sw[jj];
      if (maxlev == 0 || dist_rn(p.x, p.y, p.z, f.c.x, f.c.y, f.c.z) > f.c.w) {
        leaf<false, false, ACC>(p.x, p.y, p.z, f.c.x, f.c.y, f.c.z, w.x, w.y, w.z, 0.f, a);
      } else {
        const Tri root{nr.a.x, nr.a.y, nr.a.z, nr.a.w, nr.b.x, nr.b.y, nr.b.z, nr.b.w, nr.d.x, nr.d.y, 0};
        float as[3];   // a copy for the out-of-line subdivision, as in k_panpt
#pragma unroll
        for (int c = 0; c < 3; ++c) as[c] = a[c];
        subdivide<false, false, ACC>(p.x, p.y, p.z, root, w.x, w.y, w.z, 0.f, maxlev, as);
#pragma unroll
        for (int c = 0; c < 3; ++c) a[c] = as[c];
      }
    }
    if (ACC) fold_tile<3>(a, hi, lo);
  }
  if (partial) {
    if (ACC) {
      float* base = partial + (size_t)blockIdx.y * 6 * np_pad;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        base[(size_t)c * np_pad + i] = hi[c];
        base[(size_t)(3 + c) * np_pad + i] = lo[c];
      }
    } else {
      float* base = partial + (size_t)blockIdx.y * 3 * np_pad;
#pragma unroll
      for (int c = 0; c < 3; ++c) base[(size_t)c * np_pad + i] = a[c];
    }
  } else if (i < np) {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      if (ACC) out.p[c][i] = (float)((double)out.p[c][i] - ((double)hi[c] + (double)lo[c]));
      else     out.p[c][i] -= a[c];
    }
  }
}

__global__ void k_pack_particles(int n, int n_pad, const float* __restrict__ x, const float* __restrict__ y,
                                 const float* __restrict__ z, const float* __restrict__ sx,
                                 const float* __restrict__ sy, const float* __restrict__ sz, float4* pp) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n_pad) return;
  if (j < n) {
    pp[2 * (size_t)j] = make_float4(x[j], y[j], z[j], 0.f);
    pp[2 * (size_t)j + 1] = make_float4(sx[j], sy[j], sz[j], 0.f);
  } else {
    pp[2 * (size_t)j] = make_float4(1.0e18f, 1.0e18f, 1.0e18f, 0.f);
    pp[2 * (size_t)j + 1] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

template <int NC, int SIGN, bool ACC>
__global__ void k_reduce_panel(const float* __restrict__ partial, int nsplit, int n, int n_pad, OutPtrs<float> out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = blockIdx.y;
  if (i >= n) return;
  if (ACC) {
    double s = 0.0;
    for (int k = 0; k < nsplit; ++k) {
      s += (double)partial[((size_t)k * 2 * NC + c) * n_pad + i];
      s += (double)partial[((size_t)k * 2 * NC + NC + c) * n_pad + i];
    }
    out.p[c][i] = (float)((double)out.p[c][i] + SIGN * s);
  } else {
    float s = 0.f;
    for (int k = 0; k < nsplit; ++k) s += partial[((size_t)k * NC + c) * n_pad + i];
    out.p[c][i] += SIGN * s;
  }
}

static void plan_split(int nunits_outer, int ninner_tiles, int slots, int* nsplit, int* tps) {
  long want = 6L * slots;
  long ns = (want + nunits_outer - 1) / nunits_outer;
  const long mx = ninner_tiles >= 2 ? ninner_tiles / 2 : 1;
  if (ns > mx) ns = mx;
  if (ns < 1) ns = 1;
  *tps = (int)((ninner_tiles + ns - 1) / ns);
  *nsplit = (ninner_tiles + *tps - 1) / *tps;
}

}  // namespace o3g

using namespace o3g;

extern "C" int32_t o3g_panels_affect_points(int32_t prec, int32_t mem, int32_t maxlev, int32_t nn, const float* nx,
                                            const float* ny, const float* nz, int32_t np, const uint32_t* idx,
                                            const float* area, const float* tsx, const float* tsy, const float* tsz,
                                            const float* sss, int32_t nt, const float* tx, const float* ty,
                                            const float* tz, float* tu, float* tv, float* tw, float* const* tug,
                                            void* stream) {
  if ((mem != O3G_MEM_HOST && mem != O3G_MEM_DEVICE) || maxlev < 0 || maxlev > kMaxLev || nn < 0 || np < 0 ||
      nt < 0 || (prec != O3G_PREC_PLAIN && prec != O3G_PREC_COMPENSATED)) {
    set_error("panels_affect_points: bad precision (PLAIN or COMPENSATED), mem, maxlev (0..6) or negative count");
    return O3G_ERR_INVALID_ARG;
  }
  const bool comp = prec == O3G_PREC_COMPENSATED;
  if (np > 0 && (!nx || !ny || !nz || !idx || !area || !tsx || !tsy || !tsz)) {
    set_error("panels_affect_points: null panel array");
    return O3G_ERR_INVALID_ARG;
  }
  if (nt > 0 && (!tx || !ty || !tz || !tu || !tv || !tw)) {
    set_error("panels_affect_points: null target array");
    return O3G_ERR_INVALID_ARG;
  }
  const bool grads = tug != nullptr;
  if (grads && nt > 0)
    for (int k = 0; k < 9; ++k)
      if (!tug[k]) { set_error("panels_affect_points: null gradient component"); return O3G_ERR_INVALID_ARG; }
  if (np == 0 || nt == 0) return O3G_OK;
  if (mem == O3G_MEM_HOST) {
    for (int j = 0; j < 3 * np; ++j)
      if (idx[j] >= (uint32_t)nn) { set_error("panels_affect_points: panel index out of range"); return O3G_ERR_INVALID_ARG; }
  }
  DeviceFacts df;
  O3G_TRY(device_facts(&df));
  cudaStream_t st = (cudaStream_t)stream;
  const int NC = grads ? 12 : 3;
  const int ntiles = (np + kPB - 1) / kPB, np_pad = ntiles * kPB;
  const int tb = (nt + kPB - 1) / kPB, nt_pad = tb * kPB;
  int nb = 0;
  const void* kp;
  if (comp) kp = grads ? (sss ? (const void*)&k_panpt<true, true, true> : (const void*)&k_panpt<true, false, true>)
                       : (sss ? (const void*)&k_panpt<false, true, true> : (const void*)&k_panpt<false, false, true>);
  else kp = grads ? (sss ? (const void*)&k_panpt<true, true, false> : (const void*)&k_panpt<true, false, false>)
                  : (sss ? (const void*)&k_panpt<false, true, false> : (const void*)&k_panpt<false, false, false>);
  O3G_TRY(occupancy_blocks(kp, kPB, &nb));
  const int PC = comp ? 2 * NC : NC;   // partial components per split
  int nsplit = 1, tps = ntiles;
  plan_split(tb, ntiles, nb * df.num_sms, &nsplit, &tps);

  size_t bytes = align_up((size_t)np_pad * sizeof(PanelFar)) + align_up((size_t)np_pad * sizeof(PanelNear));
  if (nsplit > 1) bytes += align_up((size_t)nsplit * PC * nt_pad * sizeof(float));
  size_t staging = 0;
  if (mem == O3G_MEM_HOST)
    staging = 3 * align_up((size_t)nn * 4) + align_up((size_t)np * 12) + 4 * align_up((size_t)np * 4) +
              (sss ? align_up((size_t)np * 4) : 0) + 3 * align_up((size_t)nt * 4) + NC * align_up((size_t)nt * 4);
  Workspace* ws = nullptr;
  O3G_TRY(workspace_get(st, staging + bytes, &ws));
  Carve cv(ws->base);
  const float *dnx = nx, *dny = ny, *dnz = nz, *dar = area, *dtsx = tsx, *dtsy = tsy, *dtsz = tsz, *dsss = sss;
  const float *dtx = tx, *dty = ty, *dtz = tz;
  const uint32_t* didx = idx;
  OutPtrs<float> out;
  out.p[0] = tu; out.p[1] = tv; out.p[2] = tw;
  for (int k = 0; k < 9; ++k) out.p[3 + k] = grads ? tug[k] : nullptr;
  OutPtrs<float> hout = out;
  if (mem == O3G_MEM_HOST) {
    auto up = [&](const float* h, size_t n) -> const float* {
      float* d = cv.take<float>(n);
      cudaMemcpyAsync(d, h, n * 4, cudaMemcpyHostToDevice, st);
      return d;
    };
    dnx = up(nx, nn); dny = up(ny, nn); dnz = up(nz, nn);
    uint32_t* di = cv.take<uint32_t>((size_t)3 * np);
    O3G_CUDA_TRY(cudaMemcpyAsync(di, idx, (size_t)np * 12, cudaMemcpyHostToDevice, st));
    didx = di;
    dar = up(area, np); dtsx = up(tsx, np); dtsy = up(tsy, np); dtsz = up(tsz, np);
    if (sss) dsss = up(sss, np);
    dtx = up(tx, nt); dty = up(ty, nt); dtz = up(tz, nt);
    for (int c = 0; c < NC; ++c) out.p[c] = const_cast<float*>(up(hout.p[c], nt));
    O3G_CUDA_TRY(cudaGetLastError());
  }
  Carve cw(ws->base + staging);
  PanelFar* far = cw.take<PanelFar>(np_pad);
  PanelNear* nearr = cw.take<PanelNear>(np_pad);
  float* partial = nsplit > 1 ? cw.take<float>((size_t)nsplit * PC * nt_pad) : nullptr;
  k_pack_panels<<<(np_pad + 255) / 256, 256, 0, st>>>(np, dnx, dny, dnz, didx, dar, dtsx, dtsy, dtsz, dsss, np_pad,
                                                     far, nearr);
  note_launch();
  dim3 grid(tb, nsplit);
  KernelTimer& tm = thread_timer();
  tm.begin(st);
  {
    int ntl = ntiles, mxl = maxlev, ntt = nt, ntp = nt_pad;
    void* args[] = {&far, &nearr, &ntl, &tps, &mxl, &ntt, &dtx, &dty, &dtz, &partial, &ntp, &out};
    O3G_CUDA_TRY(cudaLaunchKernel(kp, grid, dim3(kPB), args, 0, st));
  }
  note_launch();
  tm.end(st);
  if (nsplit > 1) {
    const dim3 rg((nt + 255) / 256, NC);
    if (comp) {
      if (grads) k_reduce_panel<12, 1, true><<<rg, 256, 0, st>>>(partial, nsplit, nt, nt_pad, out);
      else       k_reduce_panel<3, 1, true><<<rg, 256, 0, st>>>(partial, nsplit, nt, nt_pad, out);
    } else {
      if (grads) k_reduce_panel<12, 1, false><<<rg, 256, 0, st>>>(partial, nsplit, nt, nt_pad, out);
      else       k_reduce_panel<3, 1, false><<<rg, 256, 0, st>>>(partial, nsplit, nt, nt_pad, out);
    }
    note_launch();
  }
  O3G_CUDA_TRY(cudaGetLastError());
  if (mem == O3G_MEM_HOST) {
    for (int c = 0; c < NC; ++c)
      O3G_CUDA_TRY(cudaMemcpyAsync(hout.p[c], out.p[c], (size_t)nt * 4, cudaMemcpyDeviceToHost, st));
    O3G_CUDA_TRY(cudaStreamSynchronize(st));
  }
  return O3G_OK;
}

extern "C" int32_t o3g_points_affect_panels(int32_t prec, int32_t mem, int32_t maxlev, int32_t ns, const float* sx,
                                            const float* sy, const float* sz, const float* ssx, const float* ssy,
                                            const float* ssz, int32_t nn, const float* nx, const float* ny,
                                            const float* nz, int32_t np, const uint32_t* idx, const float* area,
                                            float* pu, float* pv, float* pw, void* stream) {
  if ((mem != O3G_MEM_HOST && mem != O3G_MEM_DEVICE) || maxlev < 0 || maxlev > kMaxLev || nn < 0 || np < 0 ||
      ns < 0 || (prec != O3G_PREC_PLAIN && prec != O3G_PREC_COMPENSATED)) {
    set_error("points_affect_panels: bad precision (PLAIN or COMPENSATED), mem, maxlev (0..6) or negative count");
    return O3G_ERR_INVALID_ARG;
  }
  const bool comp = prec == O3G_PREC_COMPENSATED;
  if (ns > 0 && (!sx || !sy || !sz || !ssx || !ssy || !ssz)) {
    set_error("points_affect_panels: null particle array");
    return O3G_ERR_INVALID_ARG;
  }
  if (np > 0 && (!nx || !ny || !nz || !idx || !area || !pu || !pv || !pw)) {
    set_error("points_affect_panels: null panel array");
    return O3G_ERR_INVALID_ARG;
  }
  if (np == 0 || ns == 0) return O3G_OK;
  if (mem == O3G_MEM_HOST) {
    for (int j = 0; j < 3 * np; ++j)
      if (idx[j] >= (uint32_t)nn) { set_error("points_affect_panels: panel index out of range"); return O3G_ERR_INVALID_ARG; }
  }
  DeviceFacts df;
  O3G_TRY(device_facts(&df));
  cudaStream_t st = (cudaStream_t)stream;
  const int ptiles = (ns + kPB - 1) / kPB, ns_pad = ptiles * kPB;
  const int tb = (np + kPB - 1) / kPB, np_pad = tb * kPB;
  int nb = 0;
  const void* kp = comp ? (const void*)&k_ptpan<true> : (const void*)&k_ptpan<false>;
  O3G_TRY(occupancy_blocks(kp, kPB, &nb));
  int nsplit = 1, tps = ptiles;
  plan_split(tb, ptiles, nb * df.num_sms, &nsplit, &tps);
  const int PC = comp ? 6 : 3;
  size_t bytes = align_up((size_t)np_pad * sizeof(PanelFar)) + align_up((size_t)np_pad * sizeof(PanelNear)) +
                 align_up((size_t)ns_pad * 2 * sizeof(float4));
  if (nsplit > 1) bytes += align_up((size_t)nsplit * PC * np_pad * sizeof(float));
  // zero strengths for the panel pack (the panels here are targets)
  bytes += align_up((size_t)np * sizeof(float));
  size_t staging = 0;
  if (mem == O3G_MEM_HOST)
    staging = 3 * align_up((size_t)nn * 4) + align_up((size_t)np * 12) + align_up((size_t)np * 4) +
              6 * align_up((size_t)ns * 4) + 3 * align_up((size_t)np * 4);
  Workspace* ws = nullptr;
  O3G_TRY(workspace_get(st, staging + bytes, &ws));
  Carve cv(ws->base);
  const float *dnx = nx, *dny = ny, *dnz = nz, *dar = area;
  const float *dsx = sx, *dsy = sy, *dsz = sz, *dssx = ssx, *dssy = ssy, *dssz = ssz;
  const uint32_t* didx = idx;
  OutPtrs<float> out;
  out.p[0] = pu; out.p[1] = pv; out.p[2] = pw;
  OutPtrs<float> hout = out;
  if (mem == O3G_MEM_HOST) {
    auto up = [&](const float* h, size_t n) -> const float* {
      float* d = cv.take<float>(n);
      cudaMemcpyAsync(d, h, n * 4, cudaMemcpyHostToDevice, st);
      return d;
    };
    dnx = up(nx, nn); dny = up(ny, nn); dnz = up(nz, nn);
    uint32_t* di = cv.take<uint32_t>((size_t)3 * np);
    O3G_CUDA_TRY(cudaMemcpyAsync(di, idx, (size_t)np * 12, cudaMemcpyHostToDevice, st));
    didx = di;
    dar = up(area, np);
    dsx = up(sx, ns); dsy = up(sy, ns); dsz = up(sz, ns);
    dssx = up(ssx, ns); dssy = up(ssy, ns); dssz = up(ssz, ns);
    for (int c = 0; c < 3; ++c) out.p[c] = const_cast<float*>(up(hout.p[c], np));
    O3G_CUDA_TRY(cudaGetLastError());
  }
  Carve cw(ws->base + staging);
  PanelFar* far = cw.take<PanelFar>(np_pad);
  PanelNear* nearr = cw.take<PanelNear>(np_pad);
  float4* pp = cw.take<float4>((size_t)ns_pad * 2);
  float* partial = nsplit > 1 ? cw.take<float>((size_t)nsplit * PC * np_pad) : nullptr;
  float* zero = cw.take<float>(np);
  O3G_CUDA_TRY(cudaMemsetAsync(zero, 0, (size_t)np * sizeof(float), st));
  k_pack_panels<<<(np_pad + 255) / 256, 256, 0, st>>>(np, dnx, dny, dnz, didx, dar, zero, zero, zero, nullptr, np_pad,
                                                     far, nearr);
  k_pack_particles<<<(ns_pad + 255) / 256, 256, 0, st>>>(ns, ns_pad, dsx, dsy, dsz, dssx, dssy, dssz, pp);
  note_launch(2);
  KernelTimer& tm = thread_timer();
  tm.begin(st);
  if (comp) k_ptpan<true><<<dim3(tb, nsplit), kPB, 0, st>>>(far, nearr, np, pp, ptiles, tps, maxlev, partial, np_pad, out);
  else      k_ptpan<false><<<dim3(tb, nsplit), kPB, 0, st>>>(far, nearr, np, pp, ptiles, tps, maxlev, partial, np_pad, out);
  note_launch();
  tm.end(st);
  if (nsplit > 1) {
    if (comp) k_reduce_panel<3, -1, true><<<dim3((np + 255) / 256, 3), 256, 0, st>>>(partial, nsplit, np, np_pad, out);
    else      k_reduce_panel<3, -1, false><<<dim3((np + 255) / 256, 3), 256, 0, st>>>(partial, nsplit, np, np_pad, out);
    note_launch();
  }
  O3G_CUDA_TRY(cudaGetLastError());
  if (mem == O3G_MEM_HOST) {
    for (int c = 0; c < 3; ++c)
      O3G_CUDA_TRY(cudaMemcpyAsync(hout.p[c], out.p[c], (size_t)np * 4, cudaMemcpyDeviceToHost, st));
    O3G_CUDA_TRY(cudaStreamSynchronize(st));
  }
  return O3G_OK;
}
