// o3g_batch_impl.cuh -- pair sums of many independent particle systems in ONE persistent
// launch (no counterpart in the reference, which calls points_affect_points once per
// (source collection, target collection) pair: Convection.h:144-172, Influence.h:67-551).
//
// Every system contributes sources (its particles) and targets (its particles, with their
// core radii, followed by its field points, core parameter 0 -- the field-point kernels
// kernel_0v_0pg / kernel_0v_0p are the particle kernels with tr = 0, Kernels.h:253-290).
// All systems are packed into one source array and one target array (each system padded to
// whole tiles / whole target blocks).  The host cuts the work into items
//   item = (target block, range of the system's source tiles, split index)
// sorted by cost (longest first).  A grid of resident blocks drains the item queue through
// one atomic counter; an item is swept exactly like a block of k_pair.  When a target block
// is split over several items, each writes its partial sums to its own slab and the last
// of them to arrive (one atomic per item, no waiting) adds the slabs in split order, so the
// results are deterministic whatever the arrival order.
#pragma once

#include "o3g_pair_impl.cuh"

namespace o3g {

// per system, in device memory
struct BatchSysDev {
  const float* p[7];   // particles: x, y, z, r, sx, sy, sz
  const float* f[3];   // field points: x, y, z
  float* out[12];      // particle u, v, w, ug[0..8]      (accumulated into)
  float* fout[12];     // field-point u, v, w, ug[0..8]   (accumulated into)
  int np, nf;
  int cp, ct;          // first index of the system in the concatenated source / target orders
  int soff;            // first packed source slot (a multiple of kBlock)
  int pad_;
};

template <class T>
struct BatchArgs {
  const V4<T>* spos;
  const V4<T>* sstr;
  const V4<T>* tpos;
  const int* tmap;         // packed target slot -> index within its system (-1 = padding)
  const int4* items;       // {target block, first tile, end tile, split index}
  int nitems;
  const int4* tbs;         // per target block: {system, first target slot, first partial slab or -1, nsplit}
  const BatchSysDev* sys;
  const float4* tile_lo;   // per half-tile bounds (classifying cores only)
  const float4* tile_hi;
  T* partial;              // slabs of [NP][kBlock * TPT]
  int* arrivals;           // per target block: items finished (reset by the last one)
  int* head;               // queue head (reset by the packing kernel before every launch)
  float* sink;             // when set, results are STORED here as [12][sink_ld] by target slot
  long long sink_ld;
};

template <int C, int MODE, bool GRADS, int TPT, class T>
__global__ void __launch_bounds__(kBlock) k_batch(const BatchArgs<T> a) {
  constexpr bool ACC = (MODE == MODE_COMP);
  constexpr bool CLASSIFY = (C == CORE_GAUSS || C == CORE_EXP);
  constexpr int NA = GRADS ? 15 : 3;
  constexpr int NC = GRADS ? 12 : 3;
  constexpr int NH = ACC ? NC : 1;
  constexpr int NP = ACC ? 2 * NC : NC;
  constexpr int TB = kBlock * TPT;
  static_assert(std::is_same<T, float>::value, "the batched sums are FP32 (packed pair arithmetic)");
  __shared__ float4 QB[2][5][kBlock / 2];   // staged tiles as source pairs, double-buffered
  __shared__ int s_item, s_last;
  // the Gaussian core's polynomial table, read from shared memory by the near-field pairs
  __shared__ __align__(16) float gsh[C == CORE_GAUSS && std::is_same<T, float>::value ? kGaussPolyStride * kGaussPolyN : 1];
  const float* gtab = nullptr;
  if constexpr (C == CORE_GAUSS && std::is_same<T, float>::value) {
    stage_gauss_table(gsh);   // visible after the first __syncthreads of the item loop
    gtab = gsh;
  }
  const int tid = threadIdx.x;
  // lane l of warp w handles slots wbase + 32 k (k < TPT) of the target block
  const int wbase = (tid >> 5) * (32 * TPT) + (tid & 31);

  for (;;) {
    __syncthreads();
    if (tid == 0) s_item = atomicAdd(a.head, 1);
    __syncthreads();
    const int it = s_item;
    if (it >= a.nitems) break;
    const int4 item = a.items[it];
    const int4 tb = a.tbs[item.x];
    const int tbase = tb.y + wbase;

    V4<T> tp[TPT];
    int tm[TPT];
    bool real[TPT];
    float2 tt[TPT][4];
#pragma unroll
    for (int k = 0; k < TPT; ++k) {
      tp[k] = a.tpos[tbase + 32 * k];
      tm[k] = a.tmap[tbase + 32 * k];
      real[k] = tm[k] >= 0;
      tt[k][0] = make_float2(tp[k].x, tp[k].x);
      tt[k][1] = make_float2(tp[k].y, tp[k].y);
      tt[k][2] = make_float2(tp[k].z, tp[k].z);
      tt[k][3] = make_float2(tp[k].w, tp[k].w);
    }

    float blo[3] = {0.f, 0.f, 0.f}, bhi[3] = {0.f, 0.f, 0.f}, bw = 0.f;
    bool live = true;
    if (CLASSIFY) live = warp_box<TPT, T>(tp, real, blo, bhi, bw);

    float2 acc2[TPT][NA];
#pragma unroll
    for (int k = 0; k < TPT; ++k)
#pragma unroll
      for (int c = 0; c < NA; ++c) acc2[k][c] = make_float2(0.f, 0.f);
    float hi[TPT][NH], lo[TPT][NH];
#pragma unroll
    for (int k = 0; k < TPT; ++k)
#pragma unroll
      for (int c = 0; c < NH; ++c) { hi[k][c] = 0.f; lo[k][c] = 0.f; }

    // double-buffered tiles, as in k_pair_f: one barrier per tile
    if (item.y < item.z)
      stage_pair(a.spos[(size_t)item.y * kBlock + tid], a.sstr[(size_t)item.y * kBlock + tid], QB[0], tid);
    for (int tile = item.y; tile < item.z; ++tile) {
      __syncthreads();
      const int buf = (tile - item.y) & 1;
      if (tile + 1 < item.z)
        stage_pair(a.spos[(size_t)(tile + 1) * kBlock + tid], a.sstr[(size_t)(tile + 1) * kBlock + tid],
                   QB[buf ^ 1], tid);
      const float4 (*Q)[kBlock / 2] = QB[buf];
      if constexpr (CLASSIFY) {
        if (!live) continue;
#pragma unroll 1
        for (int hf = 0; hf < kBlock / kHalf; ++hf) {
          const int u = tile * (kBlock / kHalf) + hf;
          if (half_is_far<C, true>(a.tile_lo[u], a.tile_hi[u], blo, bhi, bw))
            sweep_pairs<CORE_SING, MODE, GRADS, true, TPT, NA, NC, NH, kHalf / 2>(Q, hf * (kHalf / 2), tt, acc2, hi,
                                                                                lo, gtab);
          else
            sweep_pairs<C, MODE, GRADS, true, TPT, NA, NC, NH, kHalf / 2>(Q, hf * (kHalf / 2), tt, acc2, hi, lo,
                                                                        gtab);
        }
      } else {
        sweep_pairs<C, MODE, GRADS, true, TPT, NA, NC, NH, kBlock / 2>(Q, 0, tt, acc2, hi, lo, gtab);
      }
    }
    // the two lanes of the plain sums are added here, as the last step of the sums
    float acc[TPT][NA];
#pragma unroll
    for (int k = 0; k < TPT; ++k)
#pragma unroll
      for (int c = 0; c < NA; ++c) acc[k][c] = acc2[k][c].x + acc2[k][c].y;
    if (!ACC && GRADS) {
#pragma unroll
      for (int k = 0; k < TPT; ++k) fold_grads(acc[k]);
    }

    const BatchSysDev* S = a.sys + tb.x;
    const int nsplit = tb.w;
    if (nsplit == 1) {
#pragma unroll
      for (int k = 0; k < TPT; ++k) {
        const int g = tm[k];
        if (g < 0) continue;
        const int slot = tbase + 32 * k;
#pragma unroll
        for (int c = 0; c < NC; ++c) {
          if (a.sink) {
            a.sink[(size_t)c * a.sink_ld + slot] = ACC ? (float)((double)hi[k][c] + (double)lo[k][c]) : (float)acc[k][c];
            continue;
          }
          float* p = g < S->np ? S->out[c] + g : S->fout[c] + (g - S->np);
          if (ACC) *p = (float)((double)*p + ((double)hi[k][c] + (double)lo[k][c]));
          else     *p = *p + (float)acc[k][c];
        }
      }
      continue;
    }

    // split target block: own slab, then the last arriving item adds the slabs in order
    {
      T* base = a.partial + (size_t)(tb.z + item.w) * NP * TB;
#pragma unroll
      for (int k = 0; k < TPT; ++k) {
        const int i = wbase + 32 * k;
#pragma unroll
        for (int c = 0; c < NC; ++c) {
          if (ACC) {
            base[(size_t)c * TB + i] = hi[k][c];
            base[(size_t)(NC + c) * TB + i] = lo[k][c];
          } else {
            base[(size_t)c * TB + i] = acc[k][c];
          }
        }
      }
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) s_last = (atomicAdd(a.arrivals + item.x, 1) == nsplit - 1) ? 1 : 0;
    __syncthreads();
    if (!s_last) continue;
    __threadfence();
    const T* slabs = a.partial + (size_t)tb.z * NP * TB;
#pragma unroll
    for (int k = 0; k < TPT; ++k) {
      const int g = tm[k];
      if (g < 0) continue;
      const int i = wbase + 32 * k;
      const int slot = tbase + 32 * k;
#pragma unroll 1
      for (int c = 0; c < NC; ++c) {
        double sd = 0.0;
        T sf = T(0);
        for (int q = 0; q < nsplit; ++q) {
          const T* b = slabs + (size_t)q * NP * TB;
          if (ACC) {
            sd += (double)__ldcg(b + (size_t)c * TB + i);
            sd += (double)__ldcg(b + (size_t)(NC + c) * TB + i);
          } else {
            sf += __ldcg(b + (size_t)c * TB + i);
          }
        }
        if (a.sink) {
          a.sink[(size_t)c * a.sink_ld + slot] = ACC ? (float)sd : (float)sf;
          continue;
        }
        float* p = g < S->np ? S->out[c] + g : S->fout[c] + (g - S->np);
        if (ACC) *p = (float)((double)*p + sd);
        else     *p = *p + (float)sf;
      }
    }
    if (tid == 0) a.arrivals[item.x] = 0;
  }
}

// per-core dispatch, defined in o3g_batch_<core>.cu
template <int C> const void* batch_kernel(int mode, bool grads, int tpt);
template <int C> int32_t batch_launch(int mode, bool grads, int tpt, int grid, const BatchArgs<float>& a,
                                      cudaStream_t st);

#define O3G_DEFINE_BATCH_CORE(CORE)                                                                        \
  template <>                                                                                              \
  const void* batch_kernel<CORE>(int mode, bool grads, int tpt) {                                          \
    if (mode == MODE_PLAIN) {                                                                              \
      if (grads) {                                                                                         \
        if (tpt == 1) return (const void*)&k_batch<CORE, MODE_PLAIN, true, 1, float>;                      \
        if (tpt == 2) return (const void*)&k_batch<CORE, MODE_PLAIN, true, 2, float>;                      \
        if (tpt == 4) return (const void*)&k_batch<CORE, MODE_PLAIN, true, 4, float>;                      \
      } else {                                                                                             \
        if (tpt == 1) return (const void*)&k_batch<CORE, MODE_PLAIN, false, 1, float>;                     \
        if (tpt == 2) return (const void*)&k_batch<CORE, MODE_PLAIN, false, 2, float>;                     \
        if (tpt == 4) return (const void*)&k_batch<CORE, MODE_PLAIN, false, 4, float>;                     \
      }                                                                                                    \
    } else if (mode == MODE_COMP) {                                                                        \
      if (grads) {                                                                                         \
        if (tpt == 1) return (const void*)&k_batch<CORE, MODE_COMP, true, 1, float>;                       \
        if (tpt == 2) return (const void*)&k_batch<CORE, MODE_COMP, true, 2, float>;                       \
      } else {                                                                                             \
        if (tpt == 1) return (const void*)&k_batch<CORE, MODE_COMP, false, 1, float>;                      \
        if (tpt == 2) return (const void*)&k_batch<CORE, MODE_COMP, false, 2, float>;                      \
        if (tpt == 4) return (const void*)&k_batch<CORE, MODE_COMP, false, 4, float>;                      \
      }                                                                                                    \
    }                                                                                                      \
    return nullptr;                                                                                        \
  }                                                                                                        \
  template <>                                                                                              \
  int32_t batch_launch<CORE>(int mode, bool grads, int tpt, int grid, const BatchArgs<float>& a,           \
                             cudaStream_t st) {                                                            \
    const void* k = batch_kernel<CORE>(mode, grads, tpt);                                                  \
    if (!k) {                                                                                              \
      set_error("batched pair sums: unsupported (precision, targets per thread)");                         \
      return O3G_ERR_INVALID_ARG;                                                                          \
    }                                                                                                      \
    void* args[] = {(void*)&a};                                                                            \
    O3G_CUDA_TRY(cudaLaunchKernel(k, dim3(grid), dim3(kBlock), args, 0, st));                              \
    note_launch();                                                                                         \
    return O3G_OK;                                                                                         \
  }

}  // namespace o3g
