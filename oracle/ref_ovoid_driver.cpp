// TEST INFRASTRUCTURE ONLY.
//
// The C entry point around the reference's own generate_ovoid (src/GeomHelper.cpp:41-91,
// with refine_geometry from src/IglRefine.cpp and the vendored igl upsample).
// oracle/build_ref.sh streams those sources ahead of this file.

#include <algorithm>
#include <cstdint>

// generate_ovoid refines while its mean panel size, 0.35 * max(rx, ry, rz) halved after
// every level, exceeds 1.2 * ips.  An ips of 1.5x the size reached after `levels` halvings
// stops it after exactly `levels` refinements (the nearest sizes on either side differ by
// a factor of 2).  Writes nodes interleaved (x, y, z per node) and the panels' node index
// triples; returns 0, or -1 when the counts differ from 10 * 4^L + 2 and 20 * 4^L.
extern "C" int ref_generate_ovoid(int levels, float rx, float ry, float rz, float* x, uint32_t* idx) {
  if (levels < 0 || levels > 8) return -1;
  const double maxscale = std::max(rx, std::max(ry, rz));
  const float ips = (float)(0.35 * maxscale * 1.5 / (1.2 * (double)(1 << levels)));
  const ElementPacket<float> e = generate_ovoid(rx, ry, rz, ips);
  const size_t nn = (size_t)10 * ((size_t)1 << (2 * levels)) + 2;
  const size_t np = (size_t)20 * ((size_t)1 << (2 * levels));
  if (e.x.size() != 3 * nn || e.idx.size() != 3 * np) return -1;
  std::copy(e.x.begin(), e.x.end(), x);
  std::copy(e.idx.begin(), e.idx.end(), idx);
  return 0;
}
