// o3g_reflect.cu -- clear_inner_layer, method 1 (Reflect.h:446-656): every point lying
// below the cutoff layer of its closest panels is pushed out along their mean normal.
// Convection::advect_2nd_ralston calls it after the interim move and after the combine
// (Convection.h:372,381,423-424) with cutoff = 0.5/sqrt(2 pi) * ips.
//
// One thread per point sweeps all panels in order (tiles of 128 panels staged in shared
// memory), computing the closest point of each triangle exactly as panel_point_distance
// does (Reflect.h:56-183: corners, then edges, then the interior prism, later tests
// overwriting earlier ones) and keeping, like the reference's hit list, running sums of the
// normals and contact points of every panel within 10 float epsilon of the running
// minimum (a new minimum restarts the sums).  All float arithmetic uses the _rn
// intrinsics in the reference's operation order (no contraction) and its 1/x in double,
// so the pushed positions are bit-identical to the reference's.
#include "o3g_common.cuh"

#include <cfloat>

namespace o3g {

constexpr int kRB = 128;

// per panel: corners, normal, and the panel-only terms of Reflect.h:56-183 -- the edge
// vectors and their inverse squared lengths 1.0 / |e|^2 (formed in double and rounded to
// float, as the reference does per call) -- computed once here with the same operations
struct PanelTri {
  float4 a;   // x0 y0 z0 x1
  float4 b;   // y1 z1 x2 y2
  float4 c;   // z2 nx ny nz
  float4 e;   // e01 (x1 - x0), inv01
  float4 f;   // e12 (x2 - x1), inv12
  float4 g;   // e20 (x0 - x2), inv20
};

__device__ __forceinline__ float dot_rn(float a0, float a1, float a2, float b0, float b1, float b2) {
  return __fadd_rn(__fadd_rn(__fmul_rn(a0, b0), __fmul_rn(a1, b1)), __fmul_rn(a2, b2));
}

__device__ __forceinline__ float4 edge_rec(float ax, float ay, float az, float bx, float by, float bz) {
  const float ex = __fsub_rn(bx, ax), ey = __fsub_rn(by, ay), ez = __fsub_rn(bz, az);
  return make_float4(ex, ey, ez, __double2float_rn(__ddiv_rn(1.0, (double)dot_rn(ex, ey, ez, ex, ey, ez))));
}

__global__ void k_pack_tri(int np, const float* __restrict__ x, const float* __restrict__ y,
                           const float* __restrict__ z, const uint32_t* __restrict__ idx, const float* __restrict__ nx,
                           const float* __restrict__ ny, const float* __restrict__ nz, PanelTri* out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= np) return;
  const uint32_t p0 = idx[3 * (size_t)j], p1 = idx[3 * (size_t)j + 1], p2 = idx[3 * (size_t)j + 2];
  PanelTri t;
  t.a = make_float4(x[p0], y[p0], z[p0], x[p1]);
  t.b = make_float4(y[p1], z[p1], x[p2], y[p2]);
  t.c = make_float4(z[p2], nx[j], ny[j], nz[j]);
  t.e = edge_rec(x[p0], y[p0], z[p0], x[p1], y[p1], z[p1]);
  t.f = edge_rec(x[p1], y[p1], z[p1], x[p2], y[p2], z[p2]);
  t.g = edge_rec(x[p2], y[p2], z[p2], x[p0], y[p0], z[p0]);
  out[j] = t;
}

// squared distance |e x d|^2 / |e|^2 to the edge's line, kept when the foot lies on the edge
__device__ __forceinline__ void edge_rn(float e0, float e1, float e2, float inv, float d0, float d1, float d2, float ox,
                                        float oy, float oz, float& best, float& px, float& py, float& pz) {
  const float r0 = __fsub_rn(__fmul_rn(e1, d2), __fmul_rn(e2, d1));
  const float r1 = __fsub_rn(__fmul_rn(e2, d0), __fmul_rn(e0, d2));
  const float r2 = __fsub_rn(__fmul_rn(e0, d1), __fmul_rn(e1, d0));
  const float dl = __fmul_rn(dot_rn(r0, r1, r2, r0, r1, r2), inv);
  if (dl < best) {
    const float t = __fmul_rn(dot_rn(e0, e1, e2, d0, d1, d2), inv);
    if (0.0f < t && t < 1.0f) {
      best = dl;
      px = __fadd_rn(ox, __fmul_rn(t, e0));
      py = __fadd_rn(oy, __fmul_rn(t, e1));
      pz = __fadd_rn(oz, __fmul_rn(t, e2));
    }
  }
}

__device__ __forceinline__ float side_rn(float nx, float ny, float nz, float e0, float e1, float e2, float d0, float d1,
                                         float d2) {
  const float i0 = __fsub_rn(__fmul_rn(ny, e2), __fmul_rn(nz, e1));
  const float i1 = __fsub_rn(__fmul_rn(nz, e0), __fmul_rn(nx, e2));
  const float i2 = __fsub_rn(__fmul_rn(nx, e1), __fmul_rn(ny, e0));
  return dot_rn(d0, d1, d2, i0, i1, i2);
}

__device__ __forceinline__ void closest_rn(const PanelTri& p, float tx, float ty, float tz, float& d2, float& px,
                                           float& py, float& pz) {
  const float x0 = p.a.x, y0 = p.a.y, z0 = p.a.z, x1 = p.a.w, y1 = p.b.x, z1 = p.b.y;
  const float x2 = p.b.z, y2 = p.b.w, z2 = p.c.x, nx = p.c.y, ny = p.c.z, nz = p.c.w;
  float best = 9.9e+9f;
  px = 0.f; py = 0.f; pz = 0.f;
  const float a0 = __fsub_rn(tx, x0), a1 = __fsub_rn(ty, y0), a2 = __fsub_rn(tz, z0);
  const float b0 = __fsub_rn(tx, x1), b1 = __fsub_rn(ty, y1), b2 = __fsub_rn(tz, z1);
  const float c0 = __fsub_rn(tx, x2), c1 = __fsub_rn(ty, y2), c2 = __fsub_rn(tz, z2);
  const float da = dot_rn(a0, a1, a2, a0, a1, a2);
  if (da < best) { best = da; px = x0; py = y0; pz = z0; }
  const float db = dot_rn(b0, b1, b2, b0, b1, b2);
  if (db < best) { best = db; px = x1; py = y1; pz = z1; }
  const float dc = dot_rn(c0, c1, c2, c0, c1, c2);
  if (dc < best) { best = dc; px = x2; py = y2; pz = z2; }
  const float e01x = p.e.x, e01y = p.e.y, e01z = p.e.z;
  edge_rn(e01x, e01y, e01z, p.e.w, a0, a1, a2, x0, y0, z0, best, px, py, pz);
  const float e12x = p.f.x, e12y = p.f.y, e12z = p.f.z;
  edge_rn(e12x, e12y, e12z, p.f.w, b0, b1, b2, x1, y1, z1, best, px, py, pz);
  const float e20x = p.g.x, e20y = p.g.y, e20z = p.g.z;
  edge_rn(e20x, e20y, e20z, p.g.w, c0, c1, c2, x2, y2, z2, best, px, py, pz);
  const float s01 = side_rn(nx, ny, nz, e01x, e01y, e01z, a0, a1, a2);
  const float s12 = side_rn(nx, ny, nz, e12x, e12y, e12z, b0, b1, b2);
  const float s20 = side_rn(nx, ny, nz, e20x, e20y, e20z, c0, c1, c2);
  if (s01 > 0.0f && s12 > 0.0f && s20 > 0.0f) {
    const float h = dot_rn(a0, a1, a2, nx, ny, nz);
    best = __fmul_rn(h, h);
    px = __fsub_rn(tx, __fmul_rn(nx, h));
    py = __fsub_rn(ty, __fmul_rn(ny, h));
    pz = __fsub_rn(tz, __fmul_rn(nz, h));
  }
  d2 = best;
}

__global__ void __launch_bounds__(kRB) k_clear_inner(int n, float* x, float* y, float* z,
                                                     const PanelTri* __restrict__ tri, int np, float cut,
                                                     int* pushed) {
  __shared__ PanelTri st[kRB];
  const int i = blockIdx.x * kRB + threadIdx.x;
  const bool live = i < n;
  const float tx = live ? x[i] : 0.f, ty = live ? y[i] : 0.f, tz = live ? z[i] : 0.f;
  const float eps = 10.0f * FLT_EPSILON;   // the reference's 10 * epsilon, exact in float
  float mind = FLT_MAX;
  float mn0 = 0.f, mn1 = 0.f, mn2 = 0.f, mc0 = 0.f, mc1 = 0.f, mc2 = 0.f;
  int nh = 0;
  for (int j0 = 0; j0 < np; j0 += kRB) {
    __syncthreads();
    if (j0 + (int)threadIdx.x < np) st[threadIdx.x] = tri[j0 + threadIdx.x];
    __syncthreads();
    const int m = min(kRB, np - j0);
    for (int jj = 0; jj < m; ++jj) {
      const PanelTri p = st[jj];
      float d2, cx, cy, cz;
      closest_rn(p, tx, ty, tz, d2, cx, cy, cz);
      if (d2 < __fsub_rn(mind, eps)) {
        mind = d2;
        mn0 = __fadd_rn(0.f, p.c.y); mn1 = __fadd_rn(0.f, p.c.z); mn2 = __fadd_rn(0.f, p.c.w);
        mc0 = __fadd_rn(0.f, cx); mc1 = __fadd_rn(0.f, cy); mc2 = __fadd_rn(0.f, cz);
        nh = 1;
      } else if (d2 < __fadd_rn(mind, eps)) {
        mn0 = __fadd_rn(mn0, p.c.y); mn1 = __fadd_rn(mn1, p.c.z); mn2 = __fadd_rn(mn2, p.c.w);
        mc0 = __fadd_rn(mc0, cx); mc1 = __fadd_rn(mc1, cy); mc2 = __fadd_rn(mc2, cz);
        ++nh;
      }
    }
  }
  if (!live || nh == 0) return;
  // normalizeVec (MathHelper.h:186-192): 1/sqrt with the division in double
  const float len = __double2float_rn(__ddiv_rn(1.0, (double)__fsqrt_rn(dot_rn(mn0, mn1, mn2, mn0, mn1, mn2))));
  mn0 = __fmul_rn(mn0, len); mn1 = __fmul_rn(mn1, len); mn2 = __fmul_rn(mn2, len);
  const float fh = (float)nh;
  mc0 = __fdiv_rn(mc0, fh); mc1 = __fdiv_rn(mc1, fh); mc2 = __fdiv_rn(mc2, fh);
  const float dotp = __fsub_rn(dot_rn(mn0, mn1, mn2, __fsub_rn(tx, mc0), __fsub_rn(ty, mc1), __fsub_rn(tz, mc2)), cut);
  if (dotp < 0.0f) {
    x[i] = __fsub_rn(tx, __fmul_rn(dotp, mn0));
    y[i] = __fsub_rn(ty, __fmul_rn(dotp, mn1));
    z[i] = __fsub_rn(tz, __fmul_rn(dotp, mn2));
    if (pushed) atomicAdd(pushed, 1);
  }
}

// Queues the clearing of n points against `surf` on `st`; adds the number pushed to
// *dev_count (device) when it is given.
int32_t clear_inner_layer_dev(int n, float* x, float* y, float* z, const o3g_surface_t& surf, float cut,
                              int* dev_count, cudaStream_t st) {
  const int np = surf.np;
  Workspace* ws = nullptr;
  O3G_TRY(workspace_get(st, align_up((size_t)np * sizeof(PanelTri)), &ws));
  PanelTri* tri = (PanelTri*)ws->base;
  if (n == 0) return O3G_OK;
  k_pack_tri<<<(np + 255) / 256, 256, 0, st>>>(np, surf.x, surf.y, surf.z, surf.idx, surf.nx, surf.ny, surf.nz, tri);
  k_clear_inner<<<(n + kRB - 1) / kRB, kRB, 0, st>>>(n, x, y, z, tri, np, cut, dev_count);
  note_launch(2);
  O3G_CUDA_TRY(cudaGetLastError());
  return O3G_OK;
}

}  // namespace o3g

using namespace o3g;

extern "C" int32_t o3g_clear_inner_layer(int32_t n, float* x, float* y, float* z, const o3g_surface_t* surf,
                                         float cutoff_mult, float ips, int32_t* npushed, void* stream) {
  if (n < 0 || !surf || surf->np < 1 || surf->nn < 3 || (n > 0 && (!x || !y || !z)) || !surf->x || !surf->y ||
      !surf->z || !surf->idx || !surf->nx || !surf->ny || !surf->nz) {
    set_error("o3g_clear_inner_layer: bad arguments (need n >= 0, a surface with panels, nodes and normals)");
    return O3G_ERR_INVALID_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  int* counter = nullptr;
  if (npushed) {
    *npushed = 0;
    if (n == 0) return O3G_OK;
    O3G_CUDA_TRY(o3g::dev_alloc_async((void**)&counter, sizeof(int), st));
    O3G_CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(int), st));
  }
  // the cutoff height is the reference's float product _cutoff_mult * _ips (Reflect.h:553)
  const float cut = cutoff_mult * ips;
  int32_t rc = clear_inner_layer_dev(n, x, y, z, *surf, cut, counter, st);
  if (counter) {
    int h = 0;
    if (rc == O3G_OK) {
      const cudaError_t e = cudaMemcpyAsync(&h, counter, sizeof(int), cudaMemcpyDeviceToHost, st);
      if (e != cudaSuccess) { set_error_cuda("o3g_clear_inner_layer: count copy", e); rc = O3G_ERR_CUDA; }
    }
    cudaFreeAsync(counter, st);
    const cudaError_t e = cudaStreamSynchronize(st);
    if (rc == O3G_OK && e != cudaSuccess) { set_error_cuda("o3g_clear_inner_layer", e); rc = O3G_ERR_CUDA; }
    *npushed = h;
  }
  return rc;
}
