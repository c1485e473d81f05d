// o3g_noalloc.cu -- points_affect_points for callers that must not allocate device memory.
//
// Some host programs cannot let a library call cudaMalloc: code that runs inside a
// memory budget fixed at start-up (a solver embedded in a larger application that hands
// every byte of device memory to its own pool), real-time loops in which an allocation
// (and the device synchronisation cudaFree implies) would stall the step, and plugin
// hosts that forbid allocation after initialisation.  For them this file provides
// o3g_points_affect_points_noalloc: the same particle / field-point Biot-Savart sums as
// o3g_points_affect_points, on device-resident arrays, with all of its scratch space
// (packed source and target tiles, tile bounding boxes, per-split partial sums) taken
// from one fixed array in device global memory that is part of the library image.
//
//  * The array holds O3G_NOALLOC_SCRATCH_BYTES (64 MiB).  Every GPU on which the library
//    is loaded keeps it until the process exits.
//  * The first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (with that device current) and keeps it for that device's
//    context.  Make that first call before capturing any stream into a CUDA graph.  Each
//    later call compares the current context's unique id (cuCtxGetId) with the one the
//    address was taken in, and looks the address up again when it differs: after a
//    cudaDeviceReset the library image, and with it the array, is loaded anew.
//  * Every call uses the same array.  Calls whose work overlaps on the GPU (different
//    streams, or several host threads) race on it: issue them on one stream.
//  * Nothing in the array has to start at zero: every byte a call reads was written
//    earlier in the same call, so the contents left by the previous call do no harm.
//  * Problems too large for the array are rejected with O3G_ERR_INVALID_ARG before any
//    work is queued; the message (o3g_last_error) gives the bytes needed.
// Sources are not Morton-sorted here (the sort needs scratch proportional to N twice over).
// The Gaussian and compact-exponential cores still bound each source tile and test it
// against each warp's targets, but unsorted tiles and targets spread over the whole set,
// so the test almost never finds a far tile: nearly every pair takes the full core.
#include "o3g_pair_impl.cuh"

#include <cuda.h>

#include <cstdio>
#include <mutex>

namespace o3g {

static constexpr size_t kNoAllocBytes = (size_t)64 << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// Unique id of the calling thread's current context (0 when none is current), through the
// driver entry points the runtime hands out (no link against the driver library).
static unsigned long long current_context_id() {
  using GetCurrent = CUresult (*)(CUcontext*);
  using GetId = CUresult (*)(CUcontext, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = (GetCurrent)f;
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = (GetId)f;
    (void)cudaGetLastError();
  });
  CUcontext c = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&c) != CUDA_SUCCESS || !c || get_id(c, &id) != CUDA_SUCCESS) return 0;
  return id;
}

static int32_t noalloc_base(char** base) {
  static std::mutex mu;
  static char* addr[64] = {nullptr};
  static unsigned long long ctx[64] = {0};
  int dev = -1;
  O3G_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) {
    set_error("o3g_points_affect_points_noalloc: device index out of range");
    return O3G_ERR_NO_DEVICE;
  }
  std::lock_guard<std::mutex> lk(mu);
  const unsigned long long id = current_context_id();
  if (!addr[dev] || id == 0 || id != ctx[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      set_error_cuda("cudaGetSymbolAddress(g_noalloc_scratch)", e);
      return O3G_ERR_CUDA;
    }
    addr[dev] = (char*)p;
    ctx[dev] = current_context_id();   // the lookup made the device's context current
  }
  *base = addr[dev];
  return O3G_OK;
}

template <int C, int MODE, bool GRADS, bool HAVE_TR, int TPT>
static int32_t noalloc_run(int ns, const float* sx, const float* sy, const float* sz, const float* sr,
                           const float* ssx, const float* ssy, const float* ssz, int nt, const float* tx,
                           const float* ty, const float* tz, const float* tr, OutPtrs<float> out, bool same,
                           cudaStream_t st) {
  constexpr int NC = GRADS ? 12 : 3;
  constexpr bool ACC = (MODE == MODE_COMP);
  constexpr bool CLASSIFY = (C == CORE_GAUSS || C == CORE_EXP);
  DeviceFacts df;
  O3G_TRY(device_facts(&df));
  int nb = 0;
  O3G_TRY(occupancy_blocks((const void*)&k_pair<C, MODE, GRADS, HAVE_TR, TPT, float, float>, kBlock, &nb));
  PairPlan pl;
  plan_pair(ns, nt, TPT, nb * df.num_sms, &pl);
  const int nsp = same ? (pl.ns_pad > pl.nt_pad ? pl.ns_pad : pl.nt_pad) : pl.ns_pad;
  size_t fixed = 2 * align_up((size_t)nsp * sizeof(V4<float>));
  if (!same) fixed += align_up((size_t)pl.nt_pad * sizeof(V4<float>));
  if (CLASSIFY) fixed += 2 * align_up((size_t)pl.ntiles * 2 * sizeof(float4));
  if (fixed > kNoAllocBytes) {
    char msg[200];
    std::snprintf(msg, sizeof(msg),
                  "o3g_points_affect_points_noalloc: %zu bytes of scratch needed, the fixed array holds %zu",
                  fixed, kNoAllocBytes);
    set_error(msg);
    return O3G_ERR_INVALID_ARG;
  }
  // fewer source splits when their partial sums would not fit next to the packed tiles
  const size_t per_split = align_up((size_t)NC * (ACC ? 2 : 1) * pl.nt_pad * sizeof(float));
  if (pl.nsplit > 1 && fixed + (size_t)pl.nsplit * per_split > kNoAllocBytes) {
    long fit = (long)((kNoAllocBytes - fixed) / per_split);
    if (fit < 2) fit = 1;
    pl.tiles_per_split = (int)((pl.ntiles + fit - 1) / fit);
    pl.nsplit = (pl.ntiles + pl.tiles_per_split - 1) / pl.tiles_per_split;
  }

  char* base = nullptr;
  O3G_TRY(noalloc_base(&base));
  Carve cv(base);
  V4<float>* spos = cv.take<V4<float>>(nsp);
  V4<float>* sstr = cv.take<V4<float>>(nsp);
  V4<float>* tpos = same ? spos : cv.take<V4<float>>(pl.nt_pad);
  float4* tile_lo = CLASSIFY ? cv.take<float4>((size_t)pl.ntiles * 2) : nullptr;
  float4* tile_hi = CLASSIFY ? cv.take<float4>((size_t)pl.ntiles * 2) : nullptr;
  float* partial = pl.nsplit > 1 ? cv.take<float>((size_t)pl.nsplit * NC * (ACC ? 2 : 1) * pl.nt_pad) : nullptr;

  k_pack_src<C, float, float><<<(nsp + 255) / 256, 256, 0, st>>>(ns, nsp, sx, sy, sz, sr, ssx, ssy, ssz, nullptr,
                                                                spos, sstr);
  note_launch();
  if (!same) {
    k_pack_tgt<C, float, float><<<(pl.nt_pad + 255) / 256, 256, 0, st>>>(nt, pl.nt_pad, tx, ty, tz, tr, nullptr,
                                                                        tpos);
    note_launch();
  }
  if (CLASSIFY) {
    k_tile_bounds<float><<<pl.ntiles, kBlock, 0, st>>>(spos, ns, tile_lo, tile_hi);
    note_launch();
  }
  PairArgs<float, float> a;
  a.spos = spos; a.sstr = sstr; a.ntiles = pl.ntiles; a.tiles_per_split = pl.tiles_per_split;
  a.tpos = tpos; a.nt = nt; a.nt_pad = pl.nt_pad; a.partial = partial; a.out = out;
  a.tperm = nullptr; a.tile_lo = tile_lo; a.tile_hi = tile_hi;
  k_pair<C, MODE, GRADS, HAVE_TR, TPT, float, float><<<dim3(pl.tblocks, pl.nsplit), kBlock, 0, st>>>(a);
  note_launch();
  if (pl.nsplit > 1) {
    k_reduce<NC, ACC, float, float><<<dim3((nt + 255) / 256, NC), 256, 0, st>>>(partial, pl.nsplit, nt, pl.nt_pad,
                                                                                out, nullptr);
    note_launch();
  }
  O3G_CUDA_TRY(cudaGetLastError());
  return O3G_OK;
}

template <int C>
static int32_t noalloc_core(int mode, bool grads, bool htr, int ns, const float* sx, const float* sy, const float* sz,
                            const float* sr, const float* ssx, const float* ssy, const float* ssz, int nt,
                            const float* tx, const float* ty, const float* tz, const float* tr, OutPtrs<float> out,
                            bool same, cudaStream_t st) {
#define O3G_NA_ARGS ns, sx, sy, sz, sr, ssx, ssy, ssz, nt, tx, ty, tz, tr, out, same, st
  if (mode == MODE_PLAIN) {
    if (grads) return htr ? noalloc_run<C, MODE_PLAIN, true, true, 2>(O3G_NA_ARGS)
                          : noalloc_run<C, MODE_PLAIN, true, false, 2>(O3G_NA_ARGS);
    return htr ? noalloc_run<C, MODE_PLAIN, false, true, 4>(O3G_NA_ARGS)
               : noalloc_run<C, MODE_PLAIN, false, false, 4>(O3G_NA_ARGS);
  }
  if (grads) return htr ? noalloc_run<C, MODE_COMP, true, true, 1>(O3G_NA_ARGS)
                        : noalloc_run<C, MODE_COMP, true, false, 1>(O3G_NA_ARGS);
  return htr ? noalloc_run<C, MODE_COMP, false, true, 2>(O3G_NA_ARGS)
             : noalloc_run<C, MODE_COMP, false, false, 2>(O3G_NA_ARGS);
#undef O3G_NA_ARGS
}

}  // namespace o3g

extern "C" int32_t o3g_points_affect_points_noalloc(int32_t core, int32_t prec, int32_t ns, const float* sx,
                                                    const float* sy, const float* sz, const float* sr,
                                                    const float* ssx, const float* ssy, const float* ssz, int32_t nt,
                                                    const float* tx, const float* ty, const float* tz, const float* tr,
                                                    float* tu, float* tv, float* tw, float* const* tug,
                                                    void* stream) {
  using namespace o3g;
  if (core < 0 || core > 4 || (prec != O3G_PREC_PLAIN && prec != O3G_PREC_COMPENSATED) || ns < 0 || nt < 0) {
    set_error("o3g_points_affect_points_noalloc: core must be 0..4, prec PLAIN or COMPENSATED, counts >= 0");
    return O3G_ERR_INVALID_ARG;
  }
  if (ns > 0 && (!sx || !sy || !sz || !sr || !ssx || !ssy || !ssz)) {
    set_error("o3g_points_affect_points_noalloc: null source array");
    return O3G_ERR_INVALID_ARG;
  }
  if (nt > 0 && (!tx || !ty || !tz || !tu || !tv || !tw)) {
    set_error("o3g_points_affect_points_noalloc: null target array");
    return O3G_ERR_INVALID_ARG;
  }
  const bool grads = (tug != nullptr);
  if (grads && nt > 0)
    for (int k = 0; k < 9; ++k)
      if (!tug[k]) {
        set_error("o3g_points_affect_points_noalloc: null gradient component");
        return O3G_ERR_INVALID_ARG;
      }
  if (ns == 0 || nt == 0) return O3G_OK;
  OutPtrs<float> out;
  out.p[0] = tu; out.p[1] = tv; out.p[2] = tw;
  for (int k = 0; k < 9; ++k) out.p[3 + k] = grads ? tug[k] : nullptr;
  const bool same = (ns == nt && sx == tx && sy == ty && sz == tz && sr == tr);
  const bool htr = (tr != nullptr);
  cudaStream_t st = (cudaStream_t)stream;
  switch (core) {
    case CORE_RM: return noalloc_core<CORE_RM>(prec, grads, htr, ns, sx, sy, sz, sr, ssx, ssy, ssz, nt, tx, ty, tz, tr, out, same, st);
    case CORE_WL: return noalloc_core<CORE_WL>(prec, grads, htr, ns, sx, sy, sz, sr, ssx, ssy, ssz, nt, tx, ty, tz, tr, out, same, st);
    case CORE_EXP: return noalloc_core<CORE_EXP>(prec, grads, htr, ns, sx, sy, sz, sr, ssx, ssy, ssz, nt, tx, ty, tz, tr, out, same, st);
    case CORE_GAUSS: return noalloc_core<CORE_GAUSS>(prec, grads, htr, ns, sx, sy, sz, sr, ssx, ssy, ssz, nt, tx, ty, tz, tr, out, same, st);
    default: return noalloc_core<CORE_V2>(prec, grads, htr, ns, sx, sy, sz, sr, ssx, ssy, ssz, nt, tx, ty, tz, tr, out, same, st);
  }
}
