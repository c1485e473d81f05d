// TEST INFRASTRUCTURE ONLY.
//
// Drives the reference's own VtkXmlWriter (src/VtkXmlWriter.h, with its vendored tinyxml2
// and cppcodec) through the sequence of calls that Points::write_vtk (Points.h:851-1039)
// and Surfaces::write_vtk (Surfaces.h:1301-1458) make, on the caller's arrays, so that
// files from this project's writer can be compared with the reference's byte for byte.
// oracle/build_ref.sh compiles it with those sources into oracle/_ref/libo3dref_vtk.so.
#include <array>
#include <cassert>
#include <cstdint>
#include <iostream>
#include <map>
#include <memory>
#include <numeric>
#include <string>
#include <vector>

template <class S> using Vector = std::vector<S>;

#include "VtkXmlWriter.h"

namespace {
std::array<Vector<float>, 3> soa3(int n, const float* a, const float* b, const float* c) {
  return {Vector<float>(a, a + n), Vector<float>(b, b + n), Vector<float>(c, c + n)};
}
void time_field(VtkXmlWriter& w, double t) {
  w.addElement("FieldData");
  std::map<std::string, std::string> at = {{"type", "Float64"}, {"Name", "TimeValue"}, {"NumberOfTuples", "1"}};
  w.addElement("DataArray", at);
  Vector<double> tv = {t};
  w.writeDataArray(tv);
  w.closeElement();
  w.closeElement();
}
void vec3(VtkXmlWriter& w, const char* name, const std::array<Vector<float>, 3>& a) {
  std::map<std::string, std::string> at = {{"NumberOfComponents", "3"}, {"Name", name}, {"type", "Float32"}};
  w.addElement("DataArray", at);
  Vector<float> f = w.unpackArray(a);
  w.writeDataArray(f);
  w.closeElement();
}
template <class T>
void scal(VtkXmlWriter& w, const char* name, const char* type, const Vector<T>& v) {
  std::map<std::string, std::string> at = {{"Name", name}, {"type", type}};
  w.addElement("DataArray", at);
  w.writeDataArray(v);
  w.closeElement();
}
}  // namespace

// particles (sx == NULL: field points, which carry neither strength nor radius)
extern "C" int ref_write_points_vtu(const char* path, int n, const float* x, const float* y, const float* z,
                                    const float* sx, const float* sy, const float* sz, const float* r,
                                    const float* u, const float* v, const float* w, double time) {
  const bool active = sx != nullptr;
  VtkXmlWriter wr(path, true);
  time_field(wr, time);
  {
    std::map<std::string, std::string> at = {{"NumberOfPoints", std::to_string(n)},
                                              {"NumberOfCells", std::to_string(n)}};
    wr.addElement("Piece", at);
  }
  wr.addElement("Points");
  vec3(wr, "position", soa3(n, x, y, z));
  wr.closeElement();
  wr.addElement("Cells");
  Vector<int32_t> conn(n), offs(n);
  std::iota(conn.begin(), conn.end(), 0);
  std::iota(offs.begin(), offs.end(), 1);
  scal(wr, "connectivity", "Int32", conn);
  scal(wr, "offsets", "Int32", offs);
  scal(wr, "types", "UInt8", Vector<uint8_t>(n, 1));
  wr.closeElement();
  {
    std::map<std::string, std::string> at = {{"Vectors", "velocity"}};
    if (active) at.insert({"Scalars", "radius"});
    wr.addElement("PointData", at);
  }
  if (active) {
    vec3(wr, "circulation", soa3(n, sx, sy, sz));
    scal(wr, "radius", "Float32", Vector<float>(r, r + n));
  }
  vec3(wr, "velocity", soa3(n, u, v, w));
  wr.closeElement();
  wr.closeElement();
  wr.finish();
  return 0;
}

// panels: nodes, 3 indices per panel, the vortex sheet vector per panel (tsx == NULL: an
// inert surface without cell data) and the source sheet strength (src == NULL: none)
extern "C" int ref_write_panels_vtu(const char* path, int nn, const float* x, const float* y, const float* z, int np,
                                    const uint32_t* idx, const float* tsx, const float* tsy, const float* tsz,
                                    const float* src, double time) {
  VtkXmlWriter wr(path, true);
  time_field(wr, time);
  {
    std::map<std::string, std::string> at = {{"NumberOfPoints", std::to_string(nn)},
                                              {"NumberOfCells", std::to_string(np)}};
    wr.addElement("Piece", at);
  }
  wr.addElement("Points");
  vec3(wr, "position", soa3(nn, x, y, z));
  wr.closeElement();
  wr.addElement("Cells");
  Vector<int32_t> conn(idx, idx + 3 * (size_t)np), offs(np);
  std::iota(offs.begin(), offs.end(), 1);
  for (auto& o : offs) o *= 3;
  scal(wr, "connectivity", "Int32", conn);
  scal(wr, "offsets", "Int32", offs);
  scal(wr, "types", "UInt8", Vector<uint8_t>(np, 5));
  wr.closeElement();
  if (tsx || src) {
    std::map<std::string, std::string> at;
    if (src) at.insert({"Scalars", "source sheet strength"});
    wr.addElement("CellData", at);
    if (tsx) vec3(wr, "vortex sheet strength", soa3(np, tsx, tsy, tsz));
    if (src) scal(wr, "source sheet strength", "Float32", Vector<float>(src, src + np));
    wr.closeElement();
  }
  wr.closeElement();
  wr.finish();
  return 0;
}
