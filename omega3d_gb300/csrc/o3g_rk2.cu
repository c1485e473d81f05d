// o3g_rk2.cu -- inviscid Ralston RK2 convection of vortex particles and field points:
// Convection::advect_2nd_ralston (Convection.h:349-425) with finalize_vels
// (ElementBase.h:187-193, Points.h:265-277) and the first- and second-order moves with
// vortex stretching (ElementBase.h:253-304, Points.h:288-439).
//
// The element-wise kernels reproduce the reference's float/double arithmetic exactly
// (explicit _rn intrinsics: no contraction), so given the same velocities the new
// positions, strengths and elongations are bit-identical to the reference's.  A step runs
//   zero -> pair sums (vel+grad) -> finalize -> Euler move to t + 2dt/3 ->
//   zero -> pair sums at the interim state -> finalize -> 0.25/0.75 combine + stretch
// and is captured once into a CUDA graph that later steps replay (o3g_rk2_step).
#include "o3g_batch.cuh"

#include <cmath>
#include <cstring>
#include <vector>

namespace o3g {

int32_t clear_inner_layer_dev(int n, float* x, float* y, float* z, const o3g_surface_t& surf, float cut,
                              int* dev_count, cudaStream_t st);

template <int C>
int32_t ptpt_core_f(const PtPtCall& c, const float* sx, const float* sy, const float* sz, const float* sr,
                    const float* ssx, const float* ssy, const float* ssz, const float* tx, const float* ty,
                    const float* tz, const float* tr, OutPtrs<float> out, size_t* need, char* ws);

struct V3 { float* p[3]; };
struct G9 { float* p[9]; };

__global__ void k_finalize(int n, double fx, double fy, double fz, V3 u, G9 ug, int grads) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double factor = 0.25 / 3.14159265358979323846;
  u.p[0][i] = (float)__dadd_rn(fx, __dmul_rn((double)u.p[0][i], factor));
  u.p[1][i] = (float)__dadd_rn(fy, __dmul_rn((double)u.p[1][i], factor));
  u.p[2][i] = (float)__dadd_rn(fz, __dmul_rn((double)u.p[2][i], factor));
  if (grads) {
    const float gfac = (float)factor;
#pragma unroll
    for (int d = 0; d < 9; ++d) ug.p[d][i] = __fmul_rn(ug.p[d][i], gfac);
  }
}

// s . grad (row vector times the 3x3 gradient in the reference's component order)
__device__ __forceinline__ void s_dot_g(const float s[3], const float* const g[9], int i, float w[3]) {
#pragma unroll
  for (int k = 0; k < 3; ++k)
    w[k] = __fadd_rn(__fadd_rn(__fmul_rn(s[0], g[k][i]), __fmul_rn(s[1], g[3 + k][i])), __fmul_rn(s[2], g[6 + k][i]));
}
__device__ __forceinline__ float dot3_rn(const float a[3], const float b[3]) {
  return __fadd_rn(__fadd_rn(__fmul_rn(a[0], b[0]), __fmul_rn(a[1], b[1])), __fmul_rn(a[2], b[2]));
}

// first-order move (ElementBase.h:253-273, Points.h:288-351): x += dt*wt1*u, stretch with ug
__global__ void k_move_euler(int n, double dt, double wt1, V3 xin, V3 xout, V3 sin_, V3 sout, const float* ein,
                             float* eout, V3 u, G9 ug, int stretch) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double dtw = __dmul_rn((double)(float)dt, wt1);
#pragma unroll
  for (int d = 0; d < 3; ++d) xout.p[d][i] = (float)__dadd_rn((double)xin.p[d][i], __dmul_rn(dtw, (double)u.p[d][i]));
  if (!stretch) return;
  const float s[3] = {sin_.p[0][i], sin_.p[1][i], sin_.p[2][i]};
  float w[3];
  s_dot_g(s, ug.p, i, w);
  const float cm = dot3_rn(s, s);
  float e = ein[i];
  if (cm > 0.0f) {
    const float ef = (float)__ddiv_rn(__dmul_rn(dtw, (double)dot3_rn(s, w)), (double)cm);
    e = (float)__dmul_rn((double)e, __dadd_rn(1.0, (double)ef));
  }
  eout[i] = e;
  const double dw = __dmul_rn(dt, wt1);
#pragma unroll
  for (int d = 0; d < 3; ++d) sout.p[d][i] = (float)__dadd_rn((double)s[d], __dmul_rn(dw, (double)w[d]));
}

// second-order combine (ElementBase.h:276-304, Points.h:356-439); u1 <- wt1 u1 + wt2 u2
__global__ void k_move_rk2(int n, double dt, double wt1, double wt2, V3 x, V3 s_, float* elong, V3 u1, G9 ug1, V3 u2,
                           G9 ug2, int stretch) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float fdt = (float)dt;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const float u = (float)__dadd_rn(__dmul_rn(wt1, (double)u1.p[d][i]), __dmul_rn(wt2, (double)u2.p[d][i]));
    u1.p[d][i] = u;
    x.p[d][i] = __fadd_rn(x.p[d][i], __fmul_rn(fdt, u));
  }
  if (!stretch) return;
  const float s[3] = {s_.p[0][i], s_.p[1][i], s_.p[2][i]};
  float w1[3], w2[3], w[3];
  s_dot_g(s, ug1.p, i, w1);
  s_dot_g(s, ug2.p, i, w2);
#pragma unroll
  for (int d = 0; d < 3; ++d) w[d] = (float)__dadd_rn(__dmul_rn(wt1, (double)w1[d]), __dmul_rn(wt2, (double)w2[d]));
  const float cm = dot3_rn(s, s);
  if (cm > 0.0f) {
    const float ef = __fdiv_rn(__fmul_rn(fdt, dot3_rn(s, w)), cm);
    elong[i] = (float)__dmul_rn((double)elong[i], __dadd_rn(1.0, (double)ef));
  }
#pragma unroll
  for (int d = 0; d < 3; ++d) s_.p[d][i] = (float)__dadd_rn((double)s[d], __dmul_rn(dt, (double)w[d]));
}

static int32_t ptpt_dev(int core, int prec, int ns, const float* const* sx, const float* sr, const float* const* ss,
                        int nt, const float* const* tx, const float* tr, float* const* u, float* const* ug,
                        cudaStream_t st) {
  PtPtCall c;
  c.mode = prec;
  c.grads = ug != nullptr;
  c.ns = ns;
  c.nt = nt;
  c.same = (ns == nt && sx[0] == tx[0] && sx[1] == tx[1] && sx[2] == tx[2] && sr == tr);
  c.st = st;
  OutPtrs<float> out;
  for (int d = 0; d < 3; ++d) out.p[d] = u[d];
  for (int d = 0; d < 9; ++d) out.p[3 + d] = ug ? ug[d] : nullptr;
  auto run = [&](size_t* need, char* ws) -> int32_t {
    switch (core) {
      case CORE_RM: return ptpt_core_f<CORE_RM>(c, sx[0], sx[1], sx[2], sr, ss[0], ss[1], ss[2], tx[0], tx[1], tx[2], tr, out, need, ws);
      case CORE_WL: return ptpt_core_f<CORE_WL>(c, sx[0], sx[1], sx[2], sr, ss[0], ss[1], ss[2], tx[0], tx[1], tx[2], tr, out, need, ws);
      case CORE_EXP: return ptpt_core_f<CORE_EXP>(c, sx[0], sx[1], sx[2], sr, ss[0], ss[1], ss[2], tx[0], tx[1], tx[2], tr, out, need, ws);
      case CORE_GAUSS: return ptpt_core_f<CORE_GAUSS>(c, sx[0], sx[1], sx[2], sr, ss[0], ss[1], ss[2], tx[0], tx[1], tx[2], tr, out, need, ws);
      default: return ptpt_core_f<CORE_V2>(c, sx[0], sx[1], sx[2], sr, ss[0], ss[1], ss[2], tx[0], tx[1], tx[2], tr, out, need, ws);
    }
  };
  size_t need = 0;
  O3G_TRY(run(&need, nullptr));
  Workspace* ws = nullptr;
  O3G_TRY(workspace_get(st, need, &ws));
  return run(nullptr, ws->base);
}

}  // namespace o3g

using namespace o3g;

// ---- element-wise entry points ---------------------------------------------------------
extern "C" int32_t o3g_points_finalize(int32_t n, const double* fs, float* const* u, float* const* ug, void* stream) {
  if (n < 0 || !fs || (n > 0 && (!u || !u[0] || !u[1] || !u[2]))) {
    set_error("o3g_points_finalize: bad arguments");
    return O3G_ERR_INVALID_ARG;
  }
  if (n == 0) return O3G_OK;
  V3 uv{{u[0], u[1], u[2]}};
  G9 gv{};
  if (ug) for (int d = 0; d < 9; ++d) gv.p[d] = ug[d];
  k_finalize<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(n, fs[0], fs[1], fs[2], uv, gv, ug ? 1 : 0);
  note_launch();
  O3G_CUDA_TRY(cudaGetLastError());
  return O3G_OK;
}

extern "C" int32_t o3g_points_move_euler(int32_t n, double dt, double wt1, float* const* x, float* const* s,
                                         float* elong, float* const* u, float* const* ug, void* stream) {
  if (n < 0 || (n > 0 && (!x || !u))) {
    set_error("o3g_points_move_euler: bad arguments");
    return O3G_ERR_INVALID_ARG;
  }
  if (n == 0) return O3G_OK;
  const int stretch = (s && elong && ug) ? 1 : 0;
  V3 xv{{x[0], x[1], x[2]}}, uv{{u[0], u[1], u[2]}}, sv{};
  G9 gv{};
  if (stretch) {
    for (int d = 0; d < 3; ++d) sv.p[d] = s[d];
    for (int d = 0; d < 9; ++d) gv.p[d] = ug[d];
  }
  k_move_euler<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(n, dt, wt1, xv, xv, sv, sv, elong, elong, uv, gv,
                                                                 stretch);
  note_launch();
  O3G_CUDA_TRY(cudaGetLastError());
  return O3G_OK;
}

extern "C" int32_t o3g_points_move_rk2(int32_t n, double dt, double wt1, float* const* u1, float* const* ug1,
                                       double wt2, float* const* u2, float* const* ug2, float* const* x,
                                       float* const* s, float* elong, void* stream) {
  if (n < 0 || (n > 0 && (!x || !u1 || !u2))) {
    set_error("o3g_points_move_rk2: bad arguments");
    return O3G_ERR_INVALID_ARG;
  }
  if (n == 0) return O3G_OK;
  const int stretch = (s && elong && ug1 && ug2) ? 1 : 0;
  V3 xv{{x[0], x[1], x[2]}}, a{{u1[0], u1[1], u1[2]}}, b{{u2[0], u2[1], u2[2]}}, sv{};
  G9 g1{}, g2{};
  if (stretch) {
    for (int d = 0; d < 3; ++d) sv.p[d] = s[d];
    for (int d = 0; d < 9; ++d) { g1.p[d] = ug1[d]; g2.p[d] = ug2[d]; }
  }
  k_move_rk2<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(n, dt, wt1, wt2, xv, sv, elong, a, g1, b, g2,
                                                               stretch);
  note_launch();
  O3G_CUDA_TRY(cudaGetLastError());
  return O3G_OK;
}

// ---- the RK2 handle -----------------------------------------------------------------------
struct o3g_rk2 {
  int core = 0, prec = 0, n = 0, nf = 0;
  float* x[3];
  float* s[3];
  float* r = nullptr;
  float* elong = nullptr;
  float* f[3];                  // field points (may be empty)
  float* buf = nullptr;         // owned stage storage
  float *u1[3], *ug1[9], *u2[3], *ug2[9], *xi[3], *si[3], *ei;
  float *fu1[3], *fug1[9], *fu2[3], *fug2[9], *fxi[3];
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  double gdt = 0.0, gfs[3] = {0, 0, 0};
  cudaStream_t gstream = nullptr;
  bool use_graph = true;
  bool warmed = false;
  cudaStream_t warm_stream = nullptr;   // stream whose workspace the warm-up step sized
  size_t na = 0, fa = 0;                // bytes per particle / field-point component array
  o3g_batch_t* batch = nullptr;         // many independent systems: one plan, bindings 0 (x) and 1 (xi)
  struct Body {
    o3g_surface_t surf;                 // caller's device arrays
    int nunk = 2, maxlev = 3;
    o3g_bem_t* bem = nullptr;           // caller's handle, assembled and factorised at attach
    double tol = 1e-10;
    int max_iter = 30;
    float* buf = nullptr;
    float *pu[3], *rhs, *sol, *ts[3], *sss;
    float cut = 0.0f;                   // cutoff height of clear_inner_layer (0: not applied)
    int* pushed = nullptr;              // device count of points pushed
    long long solves = 0;
    int last_iters = 0;
    double last_relres = 0.0, max_relres = 0.0;
  };
  Body* body = nullptr;
};

// Surfaces::set_str + vortex_sheet_to_panel_strength (Surfaces.h:267-335) in float without
// contraction: ts = (ps0 x1 + ps1 x2) * area; the source sheet strength of nunk == 3
__global__ void k_set_str(int np, int nunk, const float* __restrict__ sol, const float* __restrict__ x1x,
                          const float* __restrict__ x1y, const float* __restrict__ x1z, const float* __restrict__ x2x,
                          const float* __restrict__ x2y, const float* __restrict__ x2z,
                          const float* __restrict__ area, float* tsx, float* tsy, float* tsz, float* sss) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const float p0 = sol[(size_t)nunk * i], p1 = sol[(size_t)nunk * i + 1], a = area[i];
  tsx[i] = __fmul_rn(__fadd_rn(__fmul_rn(p0, x1x[i]), __fmul_rn(p1, x2x[i])), a);
  tsy[i] = __fmul_rn(__fadd_rn(__fmul_rn(p0, x1y[i]), __fmul_rn(p1, x2y[i])), a);
  tsz[i] = __fmul_rn(__fadd_rn(__fmul_rn(p0, x1z[i]), __fmul_rn(p1, x2z[i])), a);
  if (nunk == 3) sss[i] = sol[3 * (size_t)i + 2];
}

// solve_bem (BEMHelper.h:43-265) for the stage state (x, s): strengths into body->ts / sss
static int32_t body_solve(o3g_rk2_t* h, float* const* x, float* const* s, const double* fs, cudaStream_t st) {
  o3g_rk2::Body& b = *h->body;
  const o3g_surface_t& g = b.surf;
  const int np = g.np;
  O3G_CUDA_TRY(cudaMemsetAsync(b.pu[0], 0, 3 * align_up((size_t)np * sizeof(float)), st));
  O3G_TRY(o3g_points_affect_panels(h->prec, O3G_MEM_DEVICE, b.maxlev, h->n, x[0], x[1], x[2], s[0], s[1], s[2],
                                   g.nn, g.x, g.y, g.z, np, g.idx, g.area, b.pu[0], b.pu[1], b.pu[2], st));
  O3G_TRY(o3g_panel_vels_to_rhs(np, b.nunk, fs, b.pu[0], b.pu[1], b.pu[2], &g, b.rhs, st));
  int it = 0;
  double rr = 0.0;
  O3G_TRY(o3g_bem_solve(b.bem, b.rhs, b.sol, nullptr, O3G_MEM_DEVICE, b.tol, b.max_iter, &it, &rr, st));
  b.solves += 1;
  b.last_iters = it;
  b.last_relres = rr;
  if (rr > b.max_relres) b.max_relres = rr;
  k_set_str<<<(np + 255) / 256, 256, 0, st>>>(np, b.nunk, b.sol, g.x1x, g.x1y, g.x1z, g.x2x, g.x2y, g.x2z, g.area,
                                              b.ts[0], b.ts[1], b.ts[2], b.sss);
  note_launch();
  O3G_CUDA_TRY(cudaGetLastError());
  return O3G_OK;
}

static int32_t body_velocities(o3g_rk2_t* h, int nt, float* const* t, float* const* u, float* const* ug,
                               cudaStream_t st) {
  o3g_rk2::Body& b = *h->body;
  const o3g_surface_t& g = b.surf;
  return o3g_panels_affect_points(h->prec, O3G_MEM_DEVICE, b.maxlev, g.nn, g.x, g.y, g.z, g.np, g.idx, g.area,
                                  b.ts[0], b.ts[1], b.ts[2], b.nunk == 3 ? b.sss : nullptr, nt, t[0], t[1], t[2],
                                  u[0], u[1], u[2], ug, st);
}

// velocities and gradients (zeroed first) of stage 0 (state x, s -> u1, fu1) or stage 1
// (interim state xi, si -> u2, fu2); the 3 + 9 component arrays of a stage are contiguous
static int32_t rk2_eval(o3g_rk2_t* h, int stage, const double* fs, cudaStream_t st) {
  const int n = h->n, nf = h->nf;
  float** u = stage == 0 ? h->u1 : h->u2;
  float** ug = stage == 0 ? h->ug1 : h->ug2;
  float** fu = stage == 0 ? h->fu1 : h->fu2;
  float** fug = stage == 0 ? h->fug1 : h->fug2;
  O3G_CUDA_TRY(cudaMemsetAsync(u[0], 0, 12 * h->na, st));
  if (nf > 0) O3G_CUDA_TRY(cudaMemsetAsync(fu[0], 0, 12 * h->fa, st));
  if (h->batch) return batch_run(h->batch, stage, st);
  float** x = stage == 0 ? h->x : h->xi;
  float** s = stage == 0 ? h->s : h->si;
  float** f = stage == 0 ? h->f : h->fxi;
  if (h->body) O3G_TRY(body_solve(h, x, s, fs, st));
  // vorticity first, then the boundary (Convection.h:158-168)
  O3G_TRY(ptpt_dev(h->core, h->prec, n, x, h->r, s, n, x, h->r, u, ug, st));
  if (h->body) O3G_TRY(body_velocities(h, n, x, u, ug, st));
  if (nf > 0) {
    O3G_TRY(ptpt_dev(h->core, h->prec, n, x, h->r, s, nf, f, nullptr, fu, fug, st));
    if (h->body) O3G_TRY(body_velocities(h, nf, f, fu, fug, st));
  }
  return O3G_OK;
}

static int32_t rk2_one_step(o3g_rk2_t* h, double dt, const double* fs, cudaStream_t st) {
  const int n = h->n, nf = h->nf;
  O3G_TRY(rk2_eval(h, 0, fs, st));
  O3G_TRY(o3g_points_finalize(n, fs, h->u1, h->ug1, st));
  if (nf > 0) O3G_TRY(o3g_points_finalize(nf, fs, h->fu1, h->fug1, st));
  // interim state at t + 2dt/3 (Convection.h:366-378)
  const double dt2 = 2.0 / 3.0 * dt;
  {
    V3 xin{{h->x[0], h->x[1], h->x[2]}}, xo{{h->xi[0], h->xi[1], h->xi[2]}};
    V3 sin_{{h->s[0], h->s[1], h->s[2]}}, so{{h->si[0], h->si[1], h->si[2]}}, uv{{h->u1[0], h->u1[1], h->u1[2]}};
    G9 gv;
    for (int d = 0; d < 9; ++d) gv.p[d] = h->ug1[d];
    k_move_euler<<<(n + 255) / 256, 256, 0, st>>>(n, dt2, 1.0, xin, xo, sin_, so, h->elong, h->ei, uv, gv, 1);
    note_launch();
    if (nf > 0) {
      V3 fin{{h->f[0], h->f[1], h->f[2]}}, fo{{h->fxi[0], h->fxi[1], h->fxi[2]}}, fu{{h->fu1[0], h->fu1[1], h->fu1[2]}};
      k_move_euler<<<(nf + 255) / 256, 256, 0, st>>>(nf, dt2, 1.0, fin, fo, V3{}, V3{}, nullptr, nullptr, fu, G9{}, 0);
      note_launch();
    }
  }
  // push interim particles and field points out of the body (Convection.h:372,381)
  if (h->body && h->body->cut > 0.0f) {
    O3G_TRY(clear_inner_layer_dev(n, h->xi[0], h->xi[1], h->xi[2], h->body->surf, h->body->cut, h->body->pushed, st));
    if (nf > 0)
      O3G_TRY(clear_inner_layer_dev(nf, h->fxi[0], h->fxi[1], h->fxi[2], h->body->surf, h->body->cut, h->body->pushed,
                                    st));
  }
  O3G_TRY(rk2_eval(h, 1, fs, st));
  O3G_TRY(o3g_points_finalize(n, fs, h->u2, h->ug2, st));
  if (nf > 0) O3G_TRY(o3g_points_finalize(nf, fs, h->fu2, h->fug2, st));
  // 0.25 / 0.75 combine with stretching by the stage-0 strengths (Convection.h:389-425)
  O3G_TRY(o3g_points_move_rk2(n, dt, 0.25, h->u1, h->ug1, 0.75, h->u2, h->ug2, h->x, h->s, h->elong, st));
  if (nf > 0) O3G_TRY(o3g_points_move_rk2(nf, dt, 0.25, h->fu1, nullptr, 0.75, h->fu2, nullptr, h->f, nullptr,
                                          nullptr, st));
  // and the final positions (Convection.h:423-424)
  if (h->body && h->body->cut > 0.0f) {
    O3G_TRY(clear_inner_layer_dev(n, h->x[0], h->x[1], h->x[2], h->body->surf, h->body->cut, h->body->pushed, st));
    if (nf > 0)
      O3G_TRY(clear_inner_layer_dev(nf, h->f[0], h->f[1], h->f[2], h->body->surf, h->body->cut, h->body->pushed, st));
  }
  return O3G_OK;
}

static int32_t rk2_alloc(int32_t core, int32_t prec, int32_t n, float* const* x, float* const* s, float* r,
                         float* elong, int32_t nf, float* const* fx, int32_t use_graph, o3g_rk2_t** out) {
  DeviceFacts df;
  O3G_TRY(device_facts(&df));
  o3g_rk2_t* h = new o3g_rk2_t();
  h->core = core; h->prec = prec; h->n = n; h->nf = nf; h->r = r; h->elong = elong; h->use_graph = use_graph != 0;
  for (int d = 0; d < 3; ++d) { h->x[d] = x[d]; h->s[d] = s[d]; h->f[d] = nf > 0 ? fx[d] : nullptr; }
  const size_t na = align_up((size_t)n * sizeof(float)), fa = align_up((size_t)(nf > 0 ? nf : 1) * sizeof(float));
  h->na = na;
  h->fa = fa;
  const size_t total = na * (3 + 9 + 3 + 9 + 3 + 3 + 1) + fa * (3 + 9 + 3 + 9 + 3);
  cudaError_t e = o3g::dev_alloc((void**)&h->buf, total);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    set_error_cuda("o3g_rk2_create: cudaMalloc", e);
    delete h;
    return O3G_ERR_ALLOC;
  }
  char* p = (char*)h->buf;
  auto take = [&](size_t b) { float* q = (float*)p; p += b; return q; };
  for (int d = 0; d < 3; ++d) h->u1[d] = take(na);
  for (int d = 0; d < 9; ++d) h->ug1[d] = take(na);
  for (int d = 0; d < 3; ++d) h->u2[d] = take(na);
  for (int d = 0; d < 9; ++d) h->ug2[d] = take(na);
  for (int d = 0; d < 3; ++d) h->xi[d] = take(na);
  for (int d = 0; d < 3; ++d) h->si[d] = take(na);
  h->ei = take(na);
  for (int d = 0; d < 3; ++d) h->fu1[d] = take(fa);
  for (int d = 0; d < 9; ++d) h->fug1[d] = take(fa);
  for (int d = 0; d < 3; ++d) h->fu2[d] = take(fa);
  for (int d = 0; d < 9; ++d) h->fug2[d] = take(fa);
  for (int d = 0; d < 3; ++d) h->fxi[d] = take(fa);
  *out = h;
  return O3G_OK;
}

extern "C" int32_t o3g_rk2_create(int32_t core, int32_t prec, int32_t n, float* const* x, float* const* s, float* r,
                                  float* elong, int32_t nf, float* const* fx, int32_t use_graph, o3g_rk2_t** out) {
  if (!out || core < 0 || core > 4 || (prec != O3G_PREC_PLAIN && prec != O3G_PREC_COMPENSATED) || n <= 0 || nf < 0 ||
      !x || !s || !r || !elong || (nf > 0 && !fx)) {
    set_error("o3g_rk2_create: bad arguments");
    return O3G_ERR_INVALID_ARG;
  }
  return rk2_alloc(core, prec, n, x, s, r, elong, nf, fx, use_graph, out);
}

// Many independent systems stored back to back: system i owns particles [P_i, P_i + np[i])
// and field points [F_i, F_i + nf[i]) of the concatenated arrays (P_i, F_i prefix sums).
// Each stage's velocities come from ONE batched persistent launch over all systems.
extern "C" int32_t o3g_batch_rk2_create(int32_t core, int32_t prec, int32_t nsys, const int32_t* np,
                                        const int32_t* nf, float* const* x, float* const* s, float* r, float* elong,
                                        float* const* fx, int32_t use_graph, o3g_rk2_t** out) {
  if (!out || core < 0 || core > 4 || (prec != O3G_PREC_PLAIN && prec != O3G_PREC_COMPENSATED) || nsys < 1 || !np ||
      !nf || !x || !s || !r || !elong) {
    set_error("o3g_batch_rk2_create: bad arguments");
    return O3G_ERR_INVALID_ARG;
  }
  long long tp = 0, tf = 0;
  for (int i = 0; i < nsys; ++i) {
    if (np[i] < 0 || nf[i] < 0) {
      set_error("o3g_batch_rk2_create: negative count");
      return O3G_ERR_INVALID_ARG;
    }
    tp += np[i];
    tf += nf[i];
  }
  if (tp < 1 || tp >= (1LL << 30) || tf >= (1LL << 30) || (tf > 0 && !fx)) {
    set_error("o3g_batch_rk2_create: need 1 <= total particles < 2^30 and field arrays when nf > 0");
    return O3G_ERR_INVALID_ARG;
  }
  o3g_rk2_t* h = nullptr;
  O3G_TRY(rk2_alloc(core, prec, (int)tp, x, s, r, elong, (int)tf, fx, use_graph, &h));
  std::vector<BatchSysDev> b0(nsys), b1(nsys);
  int P = 0, F = 0;
  for (int i = 0; i < nsys; ++i) {
    for (int stage = 0; stage < 2; ++stage) {
      BatchSysDev& d = stage == 0 ? b0[i] : b1[i];
      float* const* xs = stage == 0 ? h->x : h->xi;
      float* const* ss = stage == 0 ? h->s : h->si;
      float* const* fs = stage == 0 ? h->f : h->fxi;
      float* const* u = stage == 0 ? h->u1 : h->u2;
      float* const* ug = stage == 0 ? h->ug1 : h->ug2;
      float* const* fu = stage == 0 ? h->fu1 : h->fu2;
      float* const* fug = stage == 0 ? h->fug1 : h->fug2;
      d = BatchSysDev{};
      for (int k = 0; k < 3; ++k) {
        d.p[k] = xs[k] + P;
        d.p[4 + k] = ss[k] + P;
        d.out[k] = u[k] + P;
        d.f[k] = tf > 0 ? fs[k] + F : nullptr;
        d.fout[k] = tf > 0 ? fu[k] + F : nullptr;
      }
      d.p[3] = h->r + P;
      for (int k = 0; k < 9; ++k) {
        d.out[3 + k] = ug[k] + P;
        d.fout[3 + k] = tf > 0 ? fug[k] + F : nullptr;
      }
      d.np = np[i];
      d.nf = nf[i];
    }
    P += np[i];
    F += nf[i];
  }
  const BatchSysDev* binds[2] = {b0.data(), b1.data()};
  const int32_t rc = batch_create(core, prec, true, nsys, binds, 2, &h->batch);
  if (rc != O3G_OK) {
    o3g_rk2_destroy(h);
    return rc;
  }
  *out = h;
  return O3G_OK;
}

extern "C" int32_t o3g_rk2_destroy(o3g_rk2_t* h) {
  if (!h) return O3G_OK;
  cudaDeviceSynchronize();
  if (h->exec) cudaGraphExecDestroy(h->exec);
  if (h->graph) cudaGraphDestroy(h->graph);
  if (h->batch) o3g_batch_destroy(h->batch);
  if (h->body) {
    cudaFree(h->body->buf);
    delete h->body;
  }
  cudaFree(h->buf);
  delete h;
  return O3G_OK;
}

// Advance `nsteps` Ralston steps of size dt with freestream fs.  The first call runs one
// step directly (it sizes the workspaces); after that the step is captured into a graph for
// (dt, fs, stream) and replayed.  Asynchronous on `stream`.
extern "C" int32_t o3g_rk2_step(o3g_rk2_t* h, double dt, const double* fs, int32_t nsteps, void* stream) {
  if (!h || !fs || nsteps < 0) {
    set_error("o3g_rk2_step: bad arguments");
    return O3G_ERR_INVALID_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  int done = 0;
  if (h->body) {
    for (; done < nsteps; ++done) O3G_TRY(rk2_one_step(h, dt, fs, st));
    return O3G_OK;
  }
  if (!h->warmed || !h->use_graph || h->warm_stream != st) {
    // direct steps; with graphs, one direct step on this stream sizes its workspace so the
    // capture below never allocates
    for (; done < (h->use_graph ? 1 : nsteps) && done < nsteps; ++done) O3G_TRY(rk2_one_step(h, dt, fs, st));
    h->warmed = true;
    h->warm_stream = st;
    if (done == nsteps) return O3G_OK;
  }
  const bool same = h->exec && h->gdt == dt && h->gstream == st && std::memcmp(h->gfs, fs, sizeof(h->gfs)) == 0;
  if (!same) {
    if (h->exec) { cudaGraphExecDestroy(h->exec); h->exec = nullptr; }
    if (h->graph) { cudaGraphDestroy(h->graph); h->graph = nullptr; }
    if (st == nullptr) {
      set_error("o3g_rk2_step: graph capture needs a non-default stream (or use_graph = 0)");
      return O3G_ERR_INVALID_ARG;
    }
    O3G_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    const int32_t rc = rk2_one_step(h, dt, fs, st);
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(st, &g);
    if (rc != O3G_OK) { if (g) cudaGraphDestroy(g); return rc; }
    if (ce != cudaSuccess) { set_error_cuda("cudaStreamEndCapture", ce); return O3G_ERR_CUDA; }
    h->graph = g;
    O3G_CUDA_TRY(cudaGraphInstantiate(&h->exec, h->graph, 0));
    h->gdt = dt;
    std::memcpy(h->gfs, fs, sizeof(h->gfs));
    h->gstream = st;
  }
  for (; done < nsteps; ++done) O3G_CUDA_TRY(cudaGraphLaunch(h->exec, st));
  return O3G_OK;
}

extern "C" int32_t o3g_rk2_velocities(o3g_rk2_t* h, float** u, float** ug) {
  if (!h || !u) return O3G_ERR_INVALID_ARG;
  for (int d = 0; d < 3; ++d) u[d] = h->u1[d];
  if (ug) for (int d = 0; d < 9; ++d) ug[d] = h->ug1[d];
  return O3G_OK;
}

extern "C" int32_t o3g_rk2_attach_body(o3g_rk2_t* h, const o3g_surface_t* surf, int32_t nunk, int32_t maxlev,
                                       o3g_bem_t* bem, double tol, int32_t max_iter, float ips, void* stream) {
  if (!h || !surf || !bem || (nunk != 2 && nunk != 3) || maxlev < 0 || maxlev > 4 || surf->np < 1 ||
      !(tol >= 0.0) || max_iter < 1 || !(ips >= 0.0f) || (ips > 0.0f && (!surf->nx || !surf->ny || !surf->nz))) {
    set_error("o3g_rk2_attach_body: bad arguments (nunk 2 or 3, maxlev 0..4, np >= 1, ips >= 0, normals)");
    return O3G_ERR_INVALID_ARG;
  }
  if (h->batch || h->body) {
    set_error("o3g_rk2_attach_body: the handle is batched or has a body already");
    return O3G_ERR_STATE;
  }
  int64_t n = 0;
  O3G_TRY(o3g_bem_size(bem, &n));
  if (n != (int64_t)surf->np * nunk) {
    set_error("o3g_rk2_attach_body: the BEM system must have np * nunk unknowns");
    return O3G_ERR_INVALID_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  float* A = nullptr;
  int64_t ld = 0;
  O3G_TRY(o3g_bem_matrix(bem, &A, &ld));
  O3G_TRY(o3g_panels_on_panels_coeff(maxlev, nunk, 1, surf, surf, A, ld, st));
  O3G_TRY(o3g_bem_factor(bem, st));
  o3g_rk2::Body* b = new o3g_rk2::Body();
  b->surf = *surf;
  b->nunk = nunk;
  b->maxlev = maxlev;
  b->bem = bem;
  b->tol = tol;
  b->max_iter = max_iter;
  const size_t pa = align_up((size_t)surf->np * sizeof(float));
  const size_t ua = align_up((size_t)surf->np * nunk * sizeof(float));
  cudaError_t e = o3g::dev_alloc((void**)&b->buf, 7 * pa + 2 * ua + 256);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    delete b;
    set_error_cuda("o3g_rk2_attach_body: cudaMalloc", e);
    return O3G_ERR_ALLOC;
  }
  char* p = (char*)b->buf;
  for (int d = 0; d < 3; ++d) { b->pu[d] = (float*)p; p += pa; }
  b->rhs = (float*)p; p += ua;
  b->sol = (float*)p; p += ua;
  for (int d = 0; d < 3; ++d) { b->ts[d] = (float*)p; p += pa; }
  b->sss = (float*)p;
  p += pa;
  b->pushed = (int*)p;
  // the reference passes 0.5/sqrt(2 pi) as S and multiplies by _ips in S (Convection.h:372)
  b->cut = ips > 0.0f ? (float)(0.5 / std::sqrt(2.0 * 3.14159265358979323846)) * ips : 0.0f;
  e = cudaMemset(b->pushed, 0, sizeof(int));
  if (e != cudaSuccess) {
    cudaFree(b->buf);
    delete b;
    set_error_cuda("o3g_rk2_attach_body: cudaMemset", e);
    return O3G_ERR_CUDA;
  }
  h->body = b;
  h->use_graph = false;
  return O3G_OK;
}

extern "C" int32_t o3g_rk2_body_stats(const o3g_rk2_t* h, int64_t* solves, int32_t* last_iters, double* last_relres,
                                      double* max_relres, int64_t* pushed) {
  if (!h || !h->body) return O3G_ERR_STATE;
  if (pushed) {
    int v = 0;
    O3G_CUDA_TRY(cudaDeviceSynchronize());
    O3G_CUDA_TRY(cudaMemcpy(&v, h->body->pushed, sizeof(int), cudaMemcpyDeviceToHost));
    *pushed = v;
  }
  if (solves) *solves = h->body->solves;
  if (last_iters) *last_iters = h->body->last_iters;
  if (last_relres) *last_relres = h->body->last_relres;
  if (max_relres) *max_relres = h->body->max_relres;
  return O3G_OK;
}

extern "C" int32_t o3g_rk2_body_strengths(const o3g_rk2_t* h, float* const* ts, float* solution, void* stream) {
  if (!h || !h->body) return O3G_ERR_STATE;
  cudaStream_t st = (cudaStream_t)stream;
  const size_t np = (size_t)h->body->surf.np;
  if (ts)
    for (int d = 0; d < 3; ++d)
      if (ts[d]) O3G_CUDA_TRY(cudaMemcpyAsync(ts[d], h->body->ts[d], np * sizeof(float), cudaMemcpyDefault, st));
  if (solution)
    O3G_CUDA_TRY(cudaMemcpyAsync(solution, h->body->sol, np * h->body->nunk * sizeof(float), cudaMemcpyDefault, st));
  O3G_CUDA_TRY(cudaStreamSynchronize(st));
  return O3G_OK;
}
