// ref_splitmerge_driver.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Flat-array entry points around the reference's own split_elongated<float>
// (Split.h:44-270) and merge_close_particles<float> (Merge.h:45-218), which
// oracle/build_ref.sh streams ahead of this file together with the vendored nanoflann.
// Output: oracle/_ref/libo3dref_splitmerge.so, used only to pin the oracle's restatement
// (oracle/o3d_oracle.cpp o3o_split_elongated / o3o_merge_close_particles).

namespace {

// the reference prints progress to std::cout; silence it while it runs
struct QuietCout {
  std::streambuf* old;
  QuietCout() : old(std::cout.rdbuf(nullptr)) {}
  ~QuietCout() {
    std::cout.rdbuf(old);
    std::cout.clear();
  }
};

}  // namespace

extern "C" int ref_split_elongated(int n, int cap, float* x, float* y, float* z, float* r, float* elong, float* sx,
                                   float* sy, float* sz, int core, float overlap, float threshold) {
  if (n < 0 || cap < n) return -1;
  Vector<float> vx(x, x + n), vy(y, y + n), vz(z, z + n), vr(r, r + n), ve(elong, elong + n);
  Vector<float> vsx(sx, sx + n), vsy(sy, sy + n), vsz(sz, sz + n);
  size_t m = 0;
  {
    QuietCout q;
    m = split_elongated<float>(vx, vy, vz, vr, ve, vsx, vsy, vsz,
                               core == 0 ? CoreType::gaussian : CoreType::compactg, overlap, threshold);
  }
  if ((size_t)n + m > (size_t)cap) return -1;
  const size_t nt = (size_t)n + m;
  for (size_t i = 0; i < nt; ++i) {
    x[i] = vx[i]; y[i] = vy[i]; z[i] = vz[i]; r[i] = vr[i]; elong[i] = ve[i];
    sx[i] = vsx[i]; sy[i] = vsy[i]; sz[i] = vsz[i];
  }
  return (int)m;
}

extern "C" int ref_merge_close_particles(int n, float* x, float* y, float* z, float* sx, float* sy, float* sz,
                                         float* r, float overlap, float threshold, int adapt_radii) {
  if (n <= 0) return n < 0 ? -1 : 0;
  std::array<Vector<float>, 3> pos = {Vector<float>(x, x + n), Vector<float>(y, y + n), Vector<float>(z, z + n)};
  std::array<Vector<float>, 3> str = {Vector<float>(sx, sx + n), Vector<float>(sy, sy + n),
                                      Vector<float>(sz, sz + n)};
  Vector<float> rad(r, r + n);
  size_t removed = 0;
  {
    QuietCout q;
    removed = merge_close_particles<float>(pos, str, rad, overlap, threshold, adapt_radii != 0);
  }
  const size_t nn = rad.size();
  for (size_t i = 0; i < nn; ++i) {
    x[i] = pos[0][i]; y[i] = pos[1][i]; z[i] = pos[2][i];
    sx[i] = str[0][i]; sy[i] = str[1][i]; sz[i] = str[2][i]; r[i] = rad[i];
  }
  return (int)removed;
}
