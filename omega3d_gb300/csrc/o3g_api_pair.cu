// o3g_api_pair.cu -- extern "C" points_affect_points entry points (float and double).
#include "o3g_pair_impl.cuh"

#include <type_traits>

#include <atomic>
#include <cstdlib>
#include <cstring>

namespace o3g {

template <class I>
static int32_t dispatch_core(int core, const PtPtCall& c, const I* sx, const I* sy, const I* sz, const I* sr,
                             const I* ssx, const I* ssy, const I* ssz, const I* tx, const I* ty, const I* tz,
                             const I* tr, OutPtrs<I> out, size_t* need, char* ws);

template <>
int32_t dispatch_core<float>(int core, const PtPtCall& c, const float* sx, const float* sy, const float* sz,
                             const float* sr, const float* ssx, const float* ssy, const float* ssz,
                             const float* tx, const float* ty, const float* tz, const float* tr,
                             OutPtrs<float> out, size_t* need, char* ws) {
  switch (core) {
    case CORE_RM: return ptpt_core_f<CORE_RM>(c, sx, sy, sz, sr, ssx, ssy, ssz, tx, ty, tz, tr, out, need, ws);
    case CORE_WL: return ptpt_core_f<CORE_WL>(c, sx, sy, sz, sr, ssx, ssy, ssz, tx, ty, tz, tr, out, need, ws);
    case CORE_EXP: return ptpt_core_f<CORE_EXP>(c, sx, sy, sz, sr, ssx, ssy, ssz, tx, ty, tz, tr, out, need, ws);
    case CORE_GAUSS: return ptpt_core_f<CORE_GAUSS>(c, sx, sy, sz, sr, ssx, ssy, ssz, tx, ty, tz, tr, out, need, ws);
    case CORE_V2: return ptpt_core_f<CORE_V2>(c, sx, sy, sz, sr, ssx, ssy, ssz, tx, ty, tz, tr, out, need, ws);
    default: return O3G_ERR_INVALID_ARG;
  }
}
template <>
int32_t dispatch_core<double>(int core, const PtPtCall& c, const double* sx, const double* sy, const double* sz,
                              const double* sr, const double* ssx, const double* ssy, const double* ssz,
                              const double* tx, const double* ty, const double* tz, const double* tr,
                              OutPtrs<double> out, size_t* need, char* ws) {
  switch (core) {
    case CORE_RM: return ptpt_core_d<CORE_RM>(c, sx, sy, sz, sr, ssx, ssy, ssz, tx, ty, tz, tr, out, need, ws);
    case CORE_WL: return ptpt_core_d<CORE_WL>(c, sx, sy, sz, sr, ssx, ssy, ssz, tx, ty, tz, tr, out, need, ws);
    case CORE_EXP: return ptpt_core_d<CORE_EXP>(c, sx, sy, sz, sr, ssx, ssy, ssz, tx, ty, tz, tr, out, need, ws);
    case CORE_GAUSS: return ptpt_core_d<CORE_GAUSS>(c, sx, sy, sz, sr, ssx, ssy, ssz, tx, ty, tz, tr, out, need, ws);
    case CORE_V2: return ptpt_core_d<CORE_V2>(c, sx, sy, sz, sr, ssx, ssy, ssz, tx, ty, tz, tr, out, need, ws);
    default: return O3G_ERR_INVALID_ARG;
  }
}

template <class I>
static int32_t ptpt_entry(int core, int mode, int mem, int ns, const I* sx, const I* sy, const I* sz, const I* sr,
                          const I* ssx, const I* ssy, const I* ssz, int nt, const I* tx, const I* ty, const I* tz,
                          const I* tr, I* tu, I* tv, I* tw, I* const* tug, void* stream) {
  const int max_mode = std::is_same<I, float>::value ? O3G_PREC_ACCURATE : O3G_PREC_FP64;
  if (core < 0 || core > 4 || mode < 0 || mode > max_mode || (mem != O3G_MEM_HOST && mem != O3G_MEM_DEVICE) ||
      ns < 0 || nt < 0) {
    set_error("points_affect_points: bad core/prec/mem or negative count");
    return O3G_ERR_INVALID_ARG;
  }
  if (ns > 0 && (!sx || !sy || !sz || !sr || !ssx || !ssy || !ssz)) {
    set_error("points_affect_points: null source array");
    return O3G_ERR_INVALID_ARG;
  }
  if (nt > 0 && (!tx || !ty || !tz || !tu || !tv || !tw)) {
    set_error("points_affect_points: null target array");
    return O3G_ERR_INVALID_ARG;
  }
  const bool grads = (tug != nullptr);
  if (grads && nt > 0)
    for (int k = 0; k < 9; ++k)
      if (!tug[k]) {
        set_error("points_affect_points: null gradient component");
        return O3G_ERR_INVALID_ARG;
      }
  if (ns == 0 || nt == 0) return O3G_OK;
  DeviceFacts df;
  O3G_TRY(device_facts(&df));

  cudaStream_t st = (cudaStream_t)stream;
  const int NC = grads ? 12 : 3;
  const bool same = (ns == nt && sx == tx && sy == ty && sz == tz && sr == tr);
  PtPtCall call;
  call.mode = mode;
  call.grads = grads;
  call.ns = ns;
  call.nt = nt;
  call.same = same;
  call.st = st;

  OutPtrs<I> out;
  out.p[0] = tu; out.p[1] = tv; out.p[2] = tw;
  for (int k = 0; k < 9; ++k) out.p[3 + k] = grads ? tug[k] : nullptr;

  size_t need = 0;
  O3G_TRY(dispatch_core<I>(core, call, sx, sy, sz, sr, ssx, ssy, ssz, tx, ty, tz, tr, out, &need, nullptr));

  size_t staging = 0;
  if (mem == O3G_MEM_HOST) {
    staging += 7 * align_up((size_t)ns * sizeof(I));
    if (!same) staging += (tr ? 4 : 3) * align_up((size_t)nt * sizeof(I));
    staging += NC * align_up((size_t)nt * sizeof(I));
  }
  Workspace* ws = nullptr;
  O3G_TRY(workspace_get(st, staging + need, &ws));

  const I *dsx = sx, *dsy = sy, *dsz = sz, *dsr = sr, *dssx = ssx, *dssy = ssy, *dssz = ssz;
  const I *dtx = tx, *dty = ty, *dtz = tz, *dtr = tr;
  OutPtrs<I> dout = out;
  if (mem == O3G_MEM_HOST) {
    Carve cv(ws->base);
    const I* hs[7] = {sx, sy, sz, sr, ssx, ssy, ssz};
    const I** ds[7] = {&dsx, &dsy, &dsz, &dsr, &dssx, &dssy, &dssz};
    for (int k = 0; k < 7; ++k) {
      I* d = cv.take<I>(ns);
      O3G_CUDA_TRY(cudaMemcpyAsync(d, hs[k], (size_t)ns * sizeof(I), cudaMemcpyHostToDevice, st));
      *ds[k] = d;
    }
    if (same) {
      dtx = dsx; dty = dsy; dtz = dsz; dtr = dsr;
    } else {
      const I* ht[4] = {tx, ty, tz, tr};
      const I** dt[4] = {&dtx, &dty, &dtz, &dtr};
      for (int k = 0; k < (tr ? 4 : 3); ++k) {
        I* d = cv.take<I>(nt);
        O3G_CUDA_TRY(cudaMemcpyAsync(d, ht[k], (size_t)nt * sizeof(I), cudaMemcpyHostToDevice, st));
        *dt[k] = d;
      }
    }
    for (int c = 0; c < NC; ++c) {
      I* d = cv.take<I>(nt);
      O3G_CUDA_TRY(cudaMemcpyAsync(d, out.p[c], (size_t)nt * sizeof(I), cudaMemcpyHostToDevice, st));
      dout.p[c] = d;
    }
  }
  O3G_TRY(dispatch_core<I>(core, call, dsx, dsy, dsz, dsr, dssx, dssy, dssz, dtx, dty, dtz, dtr, dout, nullptr,
                           ws->base + staging));
  if (mem == O3G_MEM_HOST) {
    for (int c = 0; c < NC; ++c)
      O3G_CUDA_TRY(cudaMemcpyAsync(out.p[c], dout.p[c], (size_t)nt * sizeof(I), cudaMemcpyDeviceToHost, st));
    O3G_CUDA_TRY(cudaStreamSynchronize(st));
  }
  return O3G_OK;
}

}  // namespace o3g

extern "C" int32_t o3g_points_affect_points(int32_t core, int32_t prec, int32_t mem, int32_t ns, const float* sx,
                                            const float* sy, const float* sz, const float* sr, const float* ssx,
                                            const float* ssy, const float* ssz, int32_t nt, const float* tx,
                                            const float* ty, const float* tz, const float* tr, float* tu, float* tv,
                                            float* tw, float* const* tug, void* stream) {
  return o3g::ptpt_entry<float>(core, prec, mem, ns, sx, sy, sz, sr, ssx, ssy, ssz, nt, tx, ty, tz, tr, tu, tv, tw,
                                tug, stream);
}

extern "C" int32_t o3g_points_affect_points_d(int32_t core, int32_t mem, int32_t ns, const double* sx,
                                              const double* sy, const double* sz, const double* sr, const double* ssx,
                                              const double* ssy, const double* ssz, int32_t nt, const double* tx,
                                              const double* ty, const double* tz, const double* tr, double* tu,
                                              double* tv, double* tw, double* const* tug, void* stream) {
  return o3g::ptpt_entry<double>(core, o3g::MODE_FP64, mem, ns, sx, sy, sz, sr, ssx, ssy, ssz, nt, tx, ty, tz, tr,
                                 tu, tv, tw, tug, stream);
}

// ---------------------------------------------------------------------------------------
// The reference's own external-solver hook (Influence.h:33-48, called at :88-113 when the
// reference is built with EXTERNAL_VEL_SOLVE): Fortran-style by-pointer counts, source
// positions, strengths, radii, target positions (no target radius: the targets are taken as
// points, the kernel_0v_0pg form), velocity and nine gradient arrays in host memory, summed
// into (+=).  Returns the flops of the call at the reference's accounting,
// nt (12 + flops_0v_0pg ns) (Influence.h:310), or -1 on an error (o3g_last_error).
namespace {
std::atomic<int> g_ext_core{-1};
std::atomic<int> g_ext_prec{-1};

int ext_parse(const char* v, const char* const* names, int n, int dflt) {
  if (!v || !*v) return dflt;
  for (int k = 0; k < n; ++k)
    if (!strcmp(v, names[k])) return k;
  if (v[0] >= '0' && v[0] < '0' + n && v[1] == 0) return v[0] - '0';
  return dflt;
}
void ext_method(int* core, int* prec) {
  static const char* const cores[5] = {"rm", "wl", "exp", "gauss", "v2"};
  static const char* const precs[2] = {"plain", "compensated"};
  int c = g_ext_core.load(), p = g_ext_prec.load();
  if (c < 0) c = ext_parse(getenv("O3G_EXTERNAL_CORE"), cores, 5, O3G_CORE_WL);
  if (p < 0) p = ext_parse(getenv("O3G_EXTERNAL_PREC"), precs, 2, O3G_PREC_PLAIN);
  *core = c;
  *prec = p;
}
template <class I>
float ext_call(int core, int prec, const int* ns, const I* sx, const I* sy, const I* sz, const I* ssx, const I* ssy,
               const I* ssz, const I* sr, const int* nt, const I* tx, const I* ty, const I* tz, I* tu, I* tv, I* tw,
               I* g0, I* g1, I* g2, I* g3, I* g4, I* g5, I* g6, I* g7, I* g8) {
  if (!ns || !nt) {
    o3g::set_error("external_vel_solver: null count pointer");
    return -1.0f;
  }
  I* g[9] = {g0, g1, g2, g3, g4, g5, g6, g7, g8};
  int nnull = 0;
  for (int k = 0; k < 9; ++k) nnull += (g[k] == nullptr);
  if (nnull != 0 && nnull != 9) {
    o3g::set_error("external_vel_solver: some gradient arrays are null and some are not");
    return -1.0f;
  }
  const bool grads = (nnull == 0);
  int32_t st;
  if (std::is_same<I, float>::value)
    st = o3g_points_affect_points(core, prec, O3G_MEM_HOST, *ns, (const float*)sx, (const float*)sy,
                                  (const float*)sz, (const float*)sr, (const float*)ssx, (const float*)ssy,
                                  (const float*)ssz, *nt, (const float*)tx, (const float*)ty, (const float*)tz,
                                  nullptr, (float*)tu, (float*)tv, (float*)tw,
                                  grads ? (float* const*)g : nullptr, nullptr);
  else
    st = o3g_points_affect_points_d(core, O3G_MEM_HOST, *ns, (const double*)sx, (const double*)sy,
                                    (const double*)sz, (const double*)sr, (const double*)ssx, (const double*)ssy,
                                    (const double*)ssz, *nt, (const double*)tx, (const double*)ty,
                                    (const double*)tz, nullptr, (double*)tu, (double*)tv, (double*)tw,
                                    grads ? (double* const*)g : nullptr, nullptr);
  if (st != O3G_OK) return -1.0f;
  const double fpp = (double)o3g_flops_per_pair(core, grads ? 1 : 0, 0);
  return (float)((double)(*nt) * (12.0 + fpp * (double)(*ns)));
}
}  // namespace

extern "C" int32_t o3g_external_set_method(int32_t core, int32_t prec) {
  if (core < -1 || core > 4 || prec < -1 || prec > 1) {
    o3g::set_error("o3g_external_set_method: core must be -1..4 and prec -1..1");
    return O3G_ERR_INVALID_ARG;
  }
  g_ext_core.store(core);
  g_ext_prec.store(prec);
  return O3G_OK;
}

extern "C" int32_t o3g_external_get_method(int32_t* core, int32_t* prec) {
  if (!core || !prec) return O3G_ERR_INVALID_ARG;
  int c, p;
  ext_method(&c, &p);
  *core = c;
  *prec = p;
  return O3G_OK;
}

extern "C" float external_vel_solver_f_(int* ns, const float* sx, const float* sy, const float* sz, const float* ssx,
                                        const float* ssy, const float* ssz, const float* sr, int* nt, const float* tx,
                                        const float* ty, const float* tz, float* tu, float* tv, float* tw, float* tux,
                                        float* tvx, float* twx, float* tuy, float* tvy, float* twy, float* tuz,
                                        float* tvz, float* twz) {
  int core, prec;
  ext_method(&core, &prec);
  return ext_call<float>(core, prec, ns, sx, sy, sz, ssx, ssy, ssz, sr, nt, tx, ty, tz, tu, tv, tw, tux, tvx, twx,
                         tuy, tvy, twy, tuz, tvz, twz);
}

extern "C" float external_vel_solver_d_(int* ns, const double* sx, const double* sy, const double* sz,
                                        const double* ssx, const double* ssy, const double* ssz, const double* sr,
                                        int* nt, const double* tx, const double* ty, const double* tz, double* tu,
                                        double* tv, double* tw, double* tux, double* tvx, double* twx, double* tuy,
                                        double* tvy, double* twy, double* tuz, double* tvz, double* twz) {
  int core, prec;
  ext_method(&core, &prec);
  return ext_call<double>(core, O3G_PREC_FP64, ns, sx, sy, sz, ssx, ssy, ssz, sr, nt, tx, ty, tz, tu, tv, tw, tux,
                          tvx, twx, tuy, tvy, twy, tuz, tvz, twz);
}
