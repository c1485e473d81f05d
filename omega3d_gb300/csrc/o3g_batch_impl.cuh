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
  const float4* tile_lo;   // per source tile bounds (classifying cores only)
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
  __shared__ V4<T> sp[kBlock];
  __shared__ V4<T> sw[kBlock];
  __shared__ float sbox[kBlock / 32][7];
  __shared__ int s_item, s_last;
  const int tid = threadIdx.x;

  for (;;) {
    __syncthreads();
    if (tid == 0) s_item = atomicAdd(a.head, 1);
    __syncthreads();
    const int it = s_item;
    if (it >= a.nitems) break;
    const int4 item = a.items[it];
    const int4 tb = a.tbs[item.x];
    const int tbase = tb.y + tid;

    V4<T> tp[TPT];
    int tm[TPT];
#pragma unroll
    for (int k = 0; k < TPT; ++k) {
      tp[k] = a.tpos[tbase + k * kBlock];
      tm[k] = a.tmap[tbase + k * kBlock];
    }

    // bounding box and largest core parameter of the block's real targets
    float blo[3] = {0.f, 0.f, 0.f}, bhi[3] = {0.f, 0.f, 0.f}, bw = 0.f;
    if (CLASSIFY) {
      float lo3[3] = {3.0e38f, 3.0e38f, 3.0e38f}, hi3[3] = {-3.0e38f, -3.0e38f, -3.0e38f}, mw = 0.f;
#pragma unroll
      for (int k = 0; k < TPT; ++k) {
        if (tm[k] >= 0) {
          const float v[3] = {(float)tp[k].x, (float)tp[k].y, (float)tp[k].z};
#pragma unroll
          for (int d = 0; d < 3; ++d) { lo3[d] = fminf(lo3[d], v[d]); hi3[d] = fmaxf(hi3[d], v[d]); }
          mw = fmaxf(mw, (float)tp[k].w);
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          lo3[d] = fminf(lo3[d], __shfl_xor_sync(0xffffffffu, lo3[d], o));
          hi3[d] = fmaxf(hi3[d], __shfl_xor_sync(0xffffffffu, hi3[d], o));
        }
        mw = fmaxf(mw, __shfl_xor_sync(0xffffffffu, mw, o));
      }
      if ((tid & 31) == 0) {
#pragma unroll
        for (int d = 0; d < 3; ++d) { sbox[tid >> 5][d] = lo3[d]; sbox[tid >> 5][3 + d] = hi3[d]; }
        sbox[tid >> 5][6] = mw;
      }
      __syncthreads();
#pragma unroll
      for (int d = 0; d < 3; ++d) { blo[d] = 3.0e38f; bhi[d] = -3.0e38f; }
#pragma unroll
      for (int wq = 0; wq < kBlock / 32; ++wq) {
#pragma unroll
        for (int d = 0; d < 3; ++d) { blo[d] = fminf(blo[d], sbox[wq][d]); bhi[d] = fmaxf(bhi[d], sbox[wq][3 + d]); }
        bw = fmaxf(bw, sbox[wq][6]);
      }
      const float pad = 1e-6f * (fabsf(blo[0]) + fabsf(blo[1]) + fabsf(blo[2]) + fabsf(bhi[0]) + fabsf(bhi[1]) +
                                 fabsf(bhi[2]));
#pragma unroll
      for (int d = 0; d < 3; ++d) { blo[d] -= pad; bhi[d] += pad; }
      bw *= 1.000001f;
    }

    T acc[TPT][NA];
#pragma unroll
    for (int k = 0; k < TPT; ++k)
#pragma unroll
      for (int c = 0; c < NA; ++c) acc[k][c] = T(0);
    float hi[TPT][NH], lo[TPT][NH];
#pragma unroll
    for (int k = 0; k < TPT; ++k)
#pragma unroll
      for (int c = 0; c < NH; ++c) { hi[k][c] = 0.f; lo[k][c] = 0.f; }

    for (int tile = item.y; tile < item.z; ++tile) {
      __syncthreads();
      sp[tid] = a.spos[(size_t)tile * kBlock + tid];
      sw[tid] = a.sstr[(size_t)tile * kBlock + tid];
      __syncthreads();
      bool far = false;
      if (CLASSIFY) {
        const float4 slo = a.tile_lo[tile], shi = a.tile_hi[tile];
        const float gx = fmaxf(0.f, fmaxf(slo.x - bhi[0], blo[0] - shi.x));
        const float gy = fmaxf(0.f, fmaxf(slo.y - bhi[1], blo[1] - shi.y));
        const float gz = fmaxf(0.f, fmaxf(slo.z - bhi[2], blo[2] - shi.z));
        far = FarRule<C>::far(gx * gx + gy * gy + gz * gz, slo.w + bw);
      }
      if (far) sweep_tile<CORE_SING, MODE, GRADS, true, TPT, T, NA, NC, NH>(sp, sw, tp, acc, hi, lo);
      else     sweep_tile<C, MODE, GRADS, true, TPT, T, NA, NC, NH>(sp, sw, tp, acc, hi, lo);
    }
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
        const int slot = tbase + k * kBlock;
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
        const int i = tid + k * kBlock;
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
      const int i = tid + k * kBlock;
      const int slot = tbase + k * kBlock;
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
