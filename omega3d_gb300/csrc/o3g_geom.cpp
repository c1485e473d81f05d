// o3g_geom.cpp -- host-side surface geometry of the BEM path: the icosahedral sphere
// (GeomHelper.cpp:41-91 + IglRefine.cpp:31-77 + igl upsample), panel bases and areas
// (Surfaces.h:776-816), vortex-sheet to panel strengths (Surfaces.h:309-335) and panel
// velocities to BEM right-hand side (RHS.h:54-123).  O(N) set-up work done once per
// geometry; kept on the host with the reference's float/double arithmetic so node
// coordinates, indices, bases and areas match the reference exactly.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <unordered_map>
#include <vector>
#include <algorithm>

#include "../../include/o3dgpu.h"

extern "C" int32_t o3g_ovoid_size(int32_t levels, int32_t* num_nodes, int32_t* num_panels) {
  if (levels < 0 || levels > 10 || !num_nodes || !num_panels) return O3G_ERR_INVALID_ARG;
  *num_nodes = 10 * (1 << (2 * levels)) + 2;
  *num_panels = 20 * (1 << (2 * levels));
  return O3G_OK;
}

extern "C" int32_t o3g_generate_ovoid(int32_t levels, float rx, float ry, float rz, float* x, float* y, float* z,
                                      uint32_t* idx) {
  if (levels < 0 || levels > 10 || !x || !y || !z || !idx) return O3G_ERR_INVALID_ARG;
  // level-0 icosahedron of radius 0.5 (the 12 nodes and 20 faces of Icosahedron.h:27-63)
  const float a = 4.2532550e-01f, b = 2.6286550e-01f;
  std::vector<float> v = {a, 0, b,   0, b, a,   0, -b, a,   0, b, -a,   -a, 0, -b,   -b, a, 0,
                          0, -b, -a, -a, 0, b,  -b, -a, 0,  a, 0, -b,   b, a, 0,     b, -a, 0};
  std::vector<uint32_t> f = {0, 1, 2,   3, 4, 5,   4, 3, 6,   7, 4, 8,   9, 3, 10,  9, 6, 3,   0, 9, 10,
                             7, 2, 1,   2, 8, 11,  3, 5, 10,  10, 5, 1,  6, 9, 11,  8, 4, 6,  0, 10, 1,
                             11, 0, 2,  7, 5, 4,   7, 1, 5,   6, 11, 8,  9, 0, 11,  2, 7, 8};
  for (int lev = 0; lev < levels; ++lev) {
    const size_t nv = v.size() / 3, nf = f.size() / 3;
    // new node per edge, numbered in order of first encounter over (face, edge j =
    // (F(i,j), F(i,(j+1)%3))) -- the counter of igl's upsample (upsample.cpp:38-55)
    std::unordered_map<uint64_t, uint32_t> edge;
    edge.reserve(nf * 2);
    std::vector<uint32_t> mid(3 * nf);
    uint32_t counter = 0;
    for (size_t i = 0; i < nf; ++i)
      for (int j = 0; j < 3; ++j) {
        const uint32_t p = f[3 * i + j], q = f[3 * i + (j + 1) % 3];
        const uint64_t key = ((uint64_t)std::min(p, q) << 32) | std::max(p, q);
        auto it = edge.find(key);
        if (it == edge.end()) {
          edge.emplace(key, counter);
          mid[3 * i + j] = counter++;
        } else {
          mid[3 * i + j] = it->second;
        }
      }
    std::vector<float> nv3(3 * (nv + counter));
    std::copy(v.begin(), v.end(), nv3.begin());
    // midpoints in double, stored as float (IglRefine.cpp converts igl's double result)
    for (size_t i = 0; i < nf; ++i)
      for (int j = 0; j < 3; ++j) {
        const uint32_t p = f[3 * i + j], q = f[3 * i + (j + 1) % 3];
        const size_t m = nv + mid[3 * i + j];
        for (int d = 0; d < 3; ++d) nv3[3 * m + d] = (float)(0.5 * (double)v[3 * p + d] + 0.5 * (double)v[3 * q + d]);
      }
    // four children per face (upsample.cpp:84-101)
    std::vector<uint32_t> nf3(12 * nf);
    for (size_t i = 0; i < nf; ++i) {
      const uint32_t v0 = f[3 * i], v1 = f[3 * i + 1], v2 = f[3 * i + 2];
      const uint32_t m0 = (uint32_t)nv + mid[3 * i], m1 = (uint32_t)nv + mid[3 * i + 1],
                     m2 = (uint32_t)nv + mid[3 * i + 2];
      const uint32_t c[12] = {v0, m0, m2, v1, m1, m0, m0, m1, m2, m1, v2, m2};
      std::memcpy(&nf3[12 * i], c, sizeof(c));
    }
    // back onto the sphere of radius 0.5 (GeomHelper.cpp:57-66)
    for (size_t k = 0; k < nv3.size() / 3; ++k) {
      const float rad = std::sqrt(std::pow(nv3[3 * k], 2) + std::pow(nv3[3 * k + 1], 2) + std::pow(nv3[3 * k + 2], 2));
      const float scale = 0.5 / rad;
      nv3[3 * k] *= scale;
      nv3[3 * k + 1] *= scale;
      nv3[3 * k + 2] *= scale;
    }
    v.swap(nv3);
    f.swap(nf3);
  }
  const size_t nv = v.size() / 3;
  for (size_t k = 0; k < nv; ++k) {
    x[k] = v[3 * k] * rx;
    y[k] = v[3 * k + 1] * ry;
    z[k] = v[3 * k + 2] * rz;
  }
  std::memcpy(idx, f.data(), f.size() * sizeof(uint32_t));
  return O3G_OK;
}

extern "C" int32_t o3g_compute_bases(int32_t nn, const float* x, const float* y, const float* z, int32_t np,
                                     const uint32_t* idx, float* x1x, float* x1y, float* x1z, float* x2x, float* x2y,
                                     float* x2z, float* nx, float* ny, float* nz, float* area) {
  if (nn < 0 || np < 0) return O3G_ERR_INVALID_ARG;
  if (np > 0 && (!x || !y || !z || !idx || !x1x || !x1y || !x1z || !x2x || !x2y || !x2z || !nx || !ny || !nz || !area))
    return O3G_ERR_INVALID_ARG;
  const float* P[3] = {x, y, z};
  for (int32_t i = 0; i < np; ++i) {
    const uint32_t i0 = idx[3 * (size_t)i], i1 = idx[3 * (size_t)i + 1], i2 = idx[3 * (size_t)i + 2];
    if (i0 >= (uint32_t)nn || i1 >= (uint32_t)nn || i2 >= (uint32_t)nn) return O3G_ERR_INVALID_ARG;
    float e1[3], e2[3], n[3];
    for (int j = 0; j < 3; ++j) e1[j] = P[j][i1] - P[j][i0];
    const float base = std::sqrt(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
    for (int j = 0; j < 3; ++j) e1[j] *= (1.0 / base);
    for (int j = 0; j < 3; ++j) e2[j] = P[j][i2] - P[j][i0];
    const float dp = e2[0] * e1[0] + e2[1] * e1[1] + e2[2] * e1[2];
    for (int j = 0; j < 3; ++j) e2[j] -= dp * e1[j];
    const float height = std::sqrt(e2[0] * e2[0] + e2[1] * e2[1] + e2[2] * e2[2]);
    for (int j = 0; j < 3; ++j) e2[j] *= (1.0 / height);
    area[i] = 0.5 * base * height;
    n[0] = e1[1] * e2[2] - e1[2] * e2[1];
    n[1] = e1[2] * e2[0] - e1[0] * e2[2];
    n[2] = e1[0] * e2[1] - e1[1] * e2[0];
    x1x[i] = e1[0]; x1y[i] = e1[1]; x1z[i] = e1[2];
    x2x[i] = e2[0]; x2y[i] = e2[1]; x2z[i] = e2[2];
    nx[i] = n[0]; ny[i] = n[1]; nz[i] = n[2];
  }
  return O3G_OK;
}

extern "C" int32_t o3g_sheet_to_panel_strength(int32_t np, const float* ps0, const float* ps1, const float* x1x,
                                               const float* x1y, const float* x1z, const float* x2x, const float* x2y,
                                               const float* x2z, const float* area, float* tsx, float* tsy,
                                               float* tsz) {
  if (np < 0) return O3G_ERR_INVALID_ARG;
  if (np > 0 && (!ps0 || !ps1 || !x1x || !x1y || !x1z || !x2x || !x2y || !x2z || !area || !tsx || !tsy || !tsz))
    return O3G_ERR_INVALID_ARG;
  for (int32_t i = 0; i < np; ++i) {
    tsx[i] = (ps0[i] * x1x[i] + ps1[i] * x2x[i]) * area[i];
    tsy[i] = (ps0[i] * x1y[i] + ps1[i] * x2y[i]) * area[i];
    tsz[i] = (ps0[i] * x1z[i] + ps1[i] * x2z[i]) * area[i];
  }
  return O3G_OK;
}
