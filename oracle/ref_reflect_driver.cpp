// ref_reflect_driver.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Loop driver around the reference's own panel_point_distance (Reflect.h:56-183) and
// normalizeVec / dot_product (MathHelper.h:186-198): oracle/build_ref.sh streams
// oracle/reflect_prelude.h and the reference's Reflect.h ahead of this file.  The loop is
// clear_inner_panp2's method 1 (Reflect.h:446-600, the push used by
// Convection::advect_2nd_ralston, Convection.h:372,381,423-424), restated for flat arrays
// because Points / Surfaces cannot be built here.  Output: oracle/_ref/libo3dref_reflect.so,
// used only to pin the oracle's restatement (oracle/o3d_oracle.cpp).

namespace {

template <class S>
int ref_clear(int n, S* x, int nn, const S* nodes, int np, const uint32_t* idx, const S* norm, S cutoff_mult,
              S ips) {
  const S* nx = nodes; const S* ny = nodes + nn; const S* nz = nodes + 2 * (size_t)nn;
  const S* snx = norm; const S* sny = norm + np; const S* snz = norm + 2 * (size_t)np;
  S* tx = x; S* ty = x + n; S* tz = x + 2 * (size_t)n;
  int pushed = 0;
  const S eps = 10.0 * std::numeric_limits<S>::epsilon();
  #pragma omp parallel for reduction(+:pushed)
  for (int32_t i = 0; i < n; ++i) {
    S mindist = std::numeric_limits<S>::max();
    std::vector<ClosestReturn<S>> hits;
    for (size_t j = 0; j < (size_t)np; ++j) {
      const Int jp0 = idx[3 * j + 0], jp1 = idx[3 * j + 1], jp2 = idx[3 * j + 2];
      ClosestReturn<S> result = panel_point_distance<S>(nx[jp0], ny[jp0], nz[jp0], nx[jp1], ny[jp1], nz[jp1],
                                                        nx[jp2], ny[jp2], nz[jp2], snx[j], sny[j], snz[j],
                                                        tx[i], ty[i], tz[i]);
      if (result.distsq < mindist - eps) {
        mindist = result.distsq;
        result.jidx = j;
        hits.clear();
        hits.push_back(result);
      } else if (result.distsq < mindist + eps) {
        result.jidx = j;
        hits.push_back(result);
      }
    }
    if (hits.empty()) continue;
    std::array<S, 3> mnorm = {0.0, 0.0, 0.0};
    std::array<S, 3> mcp = {0.0, 0.0, 0.0};
    for (size_t k = 0; k < hits.size(); ++k) {
      const size_t j = hits[k].jidx;
      mnorm[0] += snx[j]; mnorm[1] += sny[j]; mnorm[2] += snz[j];
      mcp[0] += hits[k].cpx; mcp[1] += hits[k].cpy; mcp[2] += hits[k].cpz;
    }
    normalizeVec(mnorm);
    for (size_t d = 0; d < 3; ++d) mcp[d] /= (S)hits.size();
    std::array<S, 3> dx = {tx[i] - mcp[0], ty[i] - mcp[1], tz[i] - mcp[2]};
    const S dotp = dot_product(mnorm, dx) - cutoff_mult * ips;
    if (dotp < 0.0) {
      tx[i] -= dotp * mnorm[0];
      ty[i] -= dotp * mnorm[1];
      tz[i] -= dotp * mnorm[2];
      pushed++;
    }
  }
  return pushed;
}

}  // namespace

extern "C" int ref_clear_inner_layer(int prec, int n, void* x, int nn, const void* nodes, int np,
                                     const uint32_t* idx, const void* norm, double cutoff_mult, double ips) {
  if (prec == 2)
    return ref_clear<double>(n, (double*)x, nn, (const double*)nodes, np, idx, (const double*)norm, cutoff_mult, ips);
  return ref_clear<float>(n, (float*)x, nn, (const float*)nodes, np, idx, (const float*)norm, (float)cutoff_mult,
                          (float)ips);
}
