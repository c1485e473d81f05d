// o3g_shed.cu -- Surfaces::represent_as_particles (Surfaces.h:959-1008): the vortex sheet of
// a boundary as one particle per panel, placed at the panel centroid pushed `offset` along
// the normal and carrying the panel's absolute strength ts (plus (bc1 x1 + bc2 x2) area for
// a reactive surface with boundary-condition values).  Diffusion sheds these after its
// solve_bem (Diffusion.h:187-224).  The float arithmetic is the reference's, without
// contraction: centroid = (1/3 in double) * (x0 + x1 + x2 in float), rounded to float.
// The same collocation points serve panels_affect_panels (Influence.h:1223-1243).
#include "o3g_common.cuh"

#include <algorithm>
#include <vector>

namespace o3g {

__global__ void k_represent_as_particles(int np, const float* __restrict__ nx, const float* __restrict__ ny,
                                         const float* __restrict__ nz, const uint32_t* __restrict__ idx,
                                         const float* __restrict__ area, const float* __restrict__ x1x,
                                         const float* __restrict__ x1y, const float* __restrict__ x1z,
                                         const float* __restrict__ x2x, const float* __restrict__ x2y,
                                         const float* __restrict__ x2z, const float* __restrict__ nmx,
                                         const float* __restrict__ nmy, const float* __restrict__ nmz,
                                         float offset, const float* __restrict__ tsx,
                                         const float* __restrict__ tsy, const float* __restrict__ tsz,
                                         const float* __restrict__ bc1, const float* __restrict__ bc2, float* px,
                                         float* py, float* pz, float* sx, float* sy, float* sz) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const uint32_t a = idx[3 * (size_t)i], b = idx[3 * (size_t)i + 1], c = idx[3 * (size_t)i + 2];
  const double third = 1.0 / 3.0;
  const float* node[3] = {nx, ny, nz};
  const float* nrm[3] = {nmx, nmy, nmz};
  float* pos[3] = {px, py, pz};
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const float sum = __fadd_rn(__fadd_rn(node[j][a], node[j][b]), node[j][c]);
    const float cen = __double2float_rn(__dmul_rn(third, (double)sum));
    pos[j][i] = __fadd_rn(cen, __fmul_rn(offset, nrm[j][i]));
  }
  float s[3] = {tsx[i], tsy[i], tsz[i]};
  if (bc1 && bc2) {
    const float* e1[3] = {x1x, x1y, x1z};
    const float* e2[3] = {x2x, x2y, x2z};
#pragma unroll
    for (int j = 0; j < 3; ++j)
      s[j] = __fadd_rn(s[j], __fmul_rn(__fadd_rn(__fmul_rn(bc1[i], e1[j][i]), __fmul_rn(bc2[i], e2[j][i])), area[i]));
  }
  sx[i] = s[0];
  sy[i] = s[1];
  sz[i] = s[2];
}

// collocation points of panels_affect_panels: the same centroid + offset * normal
__global__ void k_collocation(int np, const float* __restrict__ nx, const float* __restrict__ ny,
                              const float* __restrict__ nz, const uint32_t* __restrict__ idx,
                              const float* __restrict__ nmx, const float* __restrict__ nmy,
                              const float* __restrict__ nmz, float offset, float* px, float* py, float* pz) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const uint32_t a = idx[3 * (size_t)i], b = idx[3 * (size_t)i + 1], c = idx[3 * (size_t)i + 2];
  const float* node[3] = {nx, ny, nz};
  const float* nrm[3] = {nmx, nmy, nmz};
  float* pos[3] = {px, py, pz};
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const float sum = __fadd_rn(__fadd_rn(node[j][a], node[j][b]), node[j][c]);
    const float cen = __double2float_rn(__dmul_rn(1.0 / 3.0, (double)sum));
    pos[j][i] = __fadd_rn(cen, __fmul_rn(offset, nrm[j][i]));
  }
}

}  // namespace o3g

using namespace o3g;

// panels_affect_panels<float,A>, Influence.h:1223-1243: the target panels become points at
// their centroids pushed 0.0001 along the normal (represent_as_particles(0.0001, ...)), the
// source panels' velocity there is computed by panels_affect_points (velocity only), and the
// result is copied into the target panel velocities -- written, not accumulated.
extern "C" int32_t o3g_panels_affect_panels(int32_t prec, int32_t mem, int32_t maxlev, int32_t nn, const float* nx,
                                            const float* ny, const float* nz, int32_t np, const uint32_t* idx,
                                            const float* area, const float* tsx, const float* tsy,
                                            const float* tsz, const float* sss, int32_t tnn, const float* tnx,
                                            const float* tny, const float* tnz, int32_t tnp,
                                            const uint32_t* tidx, const float* tnmx, const float* tnmy,
                                            const float* tnmz, float* tu, float* tv, float* tw, void* stream) {
  if ((mem != O3G_MEM_HOST && mem != O3G_MEM_DEVICE) || tnn < 0 || tnp < 0 ||
      (tnp > 0 && (!tnx || !tny || !tnz || !tidx || !tnmx || !tnmy || !tnmz || !tu || !tv || !tw))) {
    set_error("o3g_panels_affect_panels: bad mem or target surface (nodes, idx, normals, outputs)");
    return O3G_ERR_INVALID_ARG;
  }
  if (tnp == 0) return O3G_OK;
  const float offset = (float)0.0001;   // represent_as_particles(0.0001, -1.0), Influence.h:1231
  cudaStream_t st = (cudaStream_t)stream;
  if (mem == O3G_MEM_HOST) {
    for (int j = 0; j < 3 * tnp; ++j)
      if (tidx[j] >= (uint32_t)tnn) {
        set_error("o3g_panels_affect_panels: target panel index out of range");
        return O3G_ERR_INVALID_ARG;
      }
    std::vector<float> p(3 * (size_t)tnp);
    const float* node[3] = {tnx, tny, tnz};
    const float* nrm[3] = {tnmx, tnmy, tnmz};
    for (int i = 0; i < tnp; ++i)
      for (int j = 0; j < 3; ++j) {
        const float sum = (node[j][tidx[3 * (size_t)i]] + node[j][tidx[3 * (size_t)i + 1]]) +
                          node[j][tidx[3 * (size_t)i + 2]];
        float c = (float)((1. / 3.) * sum);
        c += offset * nrm[j][i];
        p[(size_t)j * tnp + i] = c;
      }
    for (float* o : {tu, tv, tw}) std::fill(o, o + tnp, 0.0f);
    return o3g_panels_affect_points(prec, mem, maxlev, nn, nx, ny, nz, np, idx, area, tsx, tsy, tsz, sss, tnp,
                                    p.data(), p.data() + tnp, p.data() + 2 * (size_t)tnp, tu, tv, tw, nullptr,
                                    stream);
  }
  float* p = nullptr;
  O3G_CUDA_TRY(o3g::dev_alloc_async((void**)&p, 3 * (size_t)tnp * sizeof(float), st));
  k_collocation<<<(tnp + 255) / 256, 256, 0, st>>>(tnp, tnx, tny, tnz, tidx, tnmx, tnmy, tnmz, offset, p, p + tnp,
                                                   p + 2 * (size_t)tnp);
  note_launch();
  cudaError_t e = cudaGetLastError();
  for (float* o : {tu, tv, tw})
    if (e == cudaSuccess) e = cudaMemsetAsync(o, 0, (size_t)tnp * sizeof(float), st);
  int32_t rc = O3G_OK;
  if (e != cudaSuccess) {
    set_error_cuda("o3g_panels_affect_panels", e);
    rc = O3G_ERR_CUDA;
  } else {
    rc = o3g_panels_affect_points(prec, mem, maxlev, nn, nx, ny, nz, np, idx, area, tsx, tsy, tsz, sss, tnp, p,
                                  p + tnp, p + 2 * (size_t)tnp, tu, tv, tw, nullptr, stream);
  }
  cudaFreeAsync(p, st);
  return rc;
}

extern "C" int32_t o3g_represent_as_particles(const o3g_surface_t* surf, float offset, const float* tsx,
                                              const float* tsy, const float* tsz, const float* bc1,
                                              const float* bc2, float* px, float* py, float* pz, float* sx,
                                              float* sy, float* sz, void* stream) {
  if (!surf || surf->np < 0 || (surf->np > 0 && (!surf->x || !surf->y || !surf->z || !surf->idx || !surf->nx ||
                                                  !surf->ny || !surf->nz || !tsx || !tsy || !tsz || !px || !py ||
                                                  !pz || !sx || !sy || !sz)) ||
      ((bc1 != nullptr) != (bc2 != nullptr)) ||
      (bc1 && (!surf->area || !surf->x1x || !surf->x1y || !surf->x1z || !surf->x2x || !surf->x2y || !surf->x2z))) {
    set_error("o3g_represent_as_particles: bad arguments (surface with nodes, idx, normals; bc1 and bc2 together)");
    return O3G_ERR_INVALID_ARG;
  }
  const int np = surf->np;
  if (np == 0) return O3G_OK;
  cudaStream_t st = (cudaStream_t)stream;
  k_represent_as_particles<<<(np + 255) / 256, 256, 0, st>>>(
      np, surf->x, surf->y, surf->z, surf->idx, surf->area, surf->x1x, surf->x1y, surf->x1z, surf->x2x, surf->x2y,
      surf->x2z, surf->nx, surf->ny, surf->nz, offset, tsx, tsy, tsz, bc1, bc2, px, py, pz, sx, sy, sz);
  note_launch();
  O3G_CUDA_TRY(cudaGetLastError());
  return O3G_OK;
}
