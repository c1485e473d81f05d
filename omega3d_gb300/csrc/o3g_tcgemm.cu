// o3g_tcgemm.cu -- C -= A B on GB300's 5th-generation tensor cores (tcgen05, TF32 inputs,
// FP32 accumulation in tensor memory): the trailing updates of the BEM's blocked LU.
//
// All matrices are column-major FP32 (the BEM's layout).  A (m x k) has rows contiguous,
// so it is first copied to a K-major (row-major) scratch with k padded to whole 32-column
// slabs (zeros); B (k x n) is already K-major.  Then one persistent kernel:
//   * CTAs come in clusters of two; a cluster walks pairs of 128 x 256 tiles of C that
//     share their 256 columns (the two CTAs take the two 128-row halves), so every slab of
//     B is fetched once for both: each CTA loads 128 of its 256 rows with a TMA multicast
//     into both CTAs' shared memory.  Per 32-deep slab a CTA thus reads 16 KB of A and
//     16 KB of B from L2 for 128 x 256 outputs (a lone 128 x 128 tile reads 32 KB for half
//     as many), which keeps the TF32 operand feed below what L2 delivers;
//   * 10 warps: warp 0 issues the TMA loads, warp 1 owns the tensor memory and issues the
//     MMAs, warps 2-9 run the epilogue (two warps per 32-lane quarter of tensor memory,
//     one per 128-column half of the tile);
//   * k is swept in slabs of 32 (128 bytes of every row, the 128-byte swizzle width) through
//     a ring of kStages shared-memory stages: full/empty mbarrier pairs, TMA with
//     complete_tx on the full barrier; an empty barrier takes one tcgen05.commit from each
//     CTA of the pair (the stage is refilled by both);
//   * each slab is 4 MMAs of 128 x 256 x 8 (kind::tf32) into 256 TMEM columns; the 512
//     columns hold two accumulators, so the epilogue of one tile overlaps the MMAs of the
//     next;
//   * the epilogue never loads C: each thread writes its row of -acc (TMEM lane = row of
//     the tile) into a shared-memory chunk of 128 rows x 16 columns (two buffers for each
//     128-column half), and a TMA reduce-add (cp.reduce.async.bulk.tensor .add) adds the
//     chunk into C in L2, rounded once: the same value as C - acc.  C's base and leading
//     dimension must be 16-byte aligned (the BEM's are; the public entry point copies any
//     other C through an aligned scratch).
// Every mbarrier wait is bounded: after kWaitLimit polls it sets the error word, every
// other wait then gives up at once, the CTA still drains its copies, leaves the cluster
// together with its peer and frees its tensor memory, and the host returns
// O3G_ERR_TIMEOUT.
#include "o3g_common.cuh"

#include <cuda.h>

#include <algorithm>
#include <mutex>

namespace o3g {
namespace {

constexpr int kTM = 128, kTN = 256, kTK = 32, kStages = 4;
constexpr int kHalfN = kTN / 2;                            // B rows each CTA of a pair loads
static_assert(kHalfN == kTM, "A and B boxes share one tensor-map shape");
constexpr int kABytes = kTM * kTK * 4;                     // 16 KB
constexpr int kBBytes = kTN * kTK * 4;                     // 32 KB
constexpr int kStageBytes = kABytes + kBBytes;
constexpr int kEpiWarps = 8;
constexpr int kGemmThreads = 64 + 32 * kEpiWarps;
constexpr uint32_t kTmemCols = 2 * kTN;                    // two accumulators
constexpr unsigned long long kWaitLimit = 1ull << 26;
constexpr unsigned long long kDrainLimit = 1ull << 22;
// -acc goes through shared memory in chunks of 128 rows x 16 columns (8 KB), kCBufs buffers
// for each 128-column half of the tile, into C by TMA reduce-add
constexpr int kCCols = 16;
constexpr int kCBytes = kTM * kCCols * 4;
constexpr int kCBufs = 2;                                  // buffers per half (>= 2)
static_assert(kCBufs >= 2, "a reduce reads one buffer while the next is written");
constexpr int kChunks = kHalfN / kCCols;                   // chunks per half tile
// full[kStages], empty[kStages], tmem full[2], tmem empty[2], done
constexpr int kNumBars = 2 * kStages + 5;
constexpr size_t kGemmSmem =
    1024 + (size_t)kStages * kStageBytes + 2 * (size_t)kCBufs * kCBytes + 8 * kNumBars + 16;
static_assert(kGemmSmem <= 232448, "shared memory per CTA");

// instruction descriptor of tcgen05.mma kind::tf32: D format F32 (bits 4-5 = 1), A and B
// TF32 (bits 7-9, 10-12 = 2), both K-major (bits 15, 16 = 0), N >> 3 at bits 17-22,
// M >> 4 at bits 24-28
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kTN >> 3) << 17) |
                            ((uint32_t)(kTM >> 4) << 24);

struct GemmArgs {
  float* C;
  long long ldc;
  int m, n, nkb;
  int mpairs, ntiles;      // 128-row tile pairs, 256-column tiles
  int* err;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n"
      " .reg .pred p;\n"
      " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// false, with the error word set, after kWaitLimit polls; false at once (within 256 polls)
// when another wait already gave up
__device__ bool mbar_wait(uint32_t bar, uint32_t parity, int* err) {
  for (unsigned long long it = 0; it < kWaitLimit; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 255ull) == 255ull && *(volatile int*)err) return false;
    if (it > 64) __nanosleep(32);
  }
  atomicCAS(err, 0, O3G_ERR_TIMEOUT);
  return false;
}

// a wait on the CTA's own copies and commits, which always complete: it does not give up
// when another wait has, only after kDrainLimit polls (then it sets the error word)
__device__ bool mbar_wait_drain(uint32_t bar, uint32_t parity, int* err) {
  for (unsigned long long it = 0; it < kDrainLimit; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if (it > 64) __nanosleep(64);
  }
  atomicCAS(err, 0, O3G_ERR_TIMEOUT);
  return false;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int c0, int c1, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(bar)
      : "memory");
}

// the same box into this CTA and its cluster peer (ctaMask 0b11): data and complete_tx land
// at the same shared-memory offsets in both
__device__ __forceinline__ void tma_load_2d_pair(uint32_t dst, const CUtensorMap* map, int c0, int c1, uint32_t bar) {
  const uint16_t mask = 3;
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes.multicast::cluster"
      " [%0], [%1, {%2, %3}], [%4], %5;" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(bar), "h"(mask)
      : "memory");
}

__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
  asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// shared-memory matrix descriptor: K-major, 128-byte swizzle, rows of 128 bytes, 8-row
// groups 1024 bytes apart (SBO), start address >> 4 at bits 0-13, LBO (unused for this
// layout) 1, descriptor version 1 at bits 46-47, layout SWIZZLE_128B (2) at bits 61-63
__device__ __forceinline__ uint64_t sw128_desc(uint32_t addr) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n"
      " .reg .pred p;\n"
      " setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n"
      "}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
// one arrival on the barrier at this offset in both CTAs of the pair, once the MMAs issued
// so far have completed
__device__ __forceinline__ void mma_commit_pair(uint32_t bar) {
  const uint16_t mask = 3;
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::"r"(bar),
      "h"(mask)
      : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 16 consecutive TMEM columns of this warp's 32 lanes: thread t gets lane (base lane + t)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t* v) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
      "[%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
        "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void named_bar(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kGemmThreads)
    k_tc_gemm_sub(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                  const __grid_constant__ CUtensorMap tmC, GemmArgs g) {
  extern __shared__ unsigned char smem_raw[];
  // the 128-byte swizzle repeats every 1024 bytes: stage buffers start on 1024-byte
  // boundaries; both CTAs of a pair have the same layout (multicast writes by offset)
  const uintptr_t base = (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023;
  unsigned char* stages = reinterpret_cast<unsigned char*>(base);             // [kStages][A 16 KB | B 32 KB]
  unsigned char* cbuf = stages + (size_t)kStages * kStageBytes;                // [2 halves][2][8 KB]
  uint64_t* bars = reinterpret_cast<uint64_t*>(cbuf + 2 * (size_t)kCBufs * kCBytes);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + kNumBars);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t rank = cluster_rank();
  const int cid = blockIdx.x >> 1, ncl = gridDim.x >> 1;
  const int ntp = g.mpairs * g.ntiles;
  const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + kStages);
  const uint32_t tfull0 = smem_u32(bars + 2 * kStages), tempty0 = smem_u32(bars + 2 * kStages + 2);
  const uint32_t done = smem_u32(bars + 2 * kStages + 4);

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(full0 + 8 * s, 1);
      mbar_init(empty0 + 8 * s, 2);          // one commit from each CTA of the pair
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(tfull0 + 8 * b, 1);
      mbar_init(tempty0 + 8 * b, kEpiWarps);
    }
    mbar_init(done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  // the peer's barriers are initialised before anything is multicast into them
  cluster_sync_all();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      // TMA producer: this CTA's A tile, and its half of the pair's B tile into both CTAs
      // a box wholly outside the matrix (the odd last row tile, a half tile beyond n) is
      // replaced by the last one inside: those rows and columns of C are never written
      const int mlast = (g.m - 1) / kTM * kTM, nlast = (g.n - 1) / kHalfN * kHalfN;
      long long it = 0;
      bool ok = true;
      for (int tp = cid; tp < ntp && ok; tp += ncl) {
        const int m0 = min((2 * (tp % g.mpairs) + (int)rank) * kTM, mlast);
        const int nb = min((tp / g.mpairs) * kTN + (int)rank * kHalfN, nlast);
        for (int kb = 0; kb < g.nkb; ++kb, ++it) {
          const int s = (int)(it % kStages);
          const long long use = it / kStages;
          if (use > 0 && !mbar_wait(empty0 + 8 * s, (uint32_t)((use - 1) & 1), g.err)) {
            ok = false;
            break;
          }
          unsigned char* st = stages + (size_t)s * kStageBytes;
          mbar_expect_tx(full0 + 8 * s, kStageBytes);
          tma_load_2d(smem_u32(st), &tmA, kb * kTK, m0, full0 + 8 * s);
          tma_load_2d_pair(smem_u32(st + kABytes + (size_t)rank * (kBBytes / 2)), &tmB, kb * kTK, nb,
                           full0 + 8 * s);
        }
      }
      // before the CTA may leave: every stage's last fill has landed and both CTAs' MMAs
      // have released it (their commits arrive on this CTA's barriers); bounded
      for (long long u = it - 1; u >= 0 && u >= it - kStages; --u) {
        const int s = (int)(u % kStages);
        (void)mbar_wait_drain(full0 + 8 * s, (uint32_t)((u / kStages) & 1), g.err);
        (void)mbar_wait_drain(empty0 + 8 * s, (uint32_t)((u / kStages) & 1), g.err);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // MMA issuer
      long long it = 0;
      int t = 0;
      bool ok = true;
      for (int tp = cid; tp < ntp && ok; tp += ncl, ++t) {
        const int buf = t & 1;
        if (t >= 2 && !mbar_wait(tempty0 + 8 * buf, (uint32_t)(((t >> 1) - 1) & 1), g.err)) break;
        tc_fence_after();
        const uint32_t acc = tmem + (uint32_t)(buf * kTN);
        for (int kb = 0; kb < g.nkb; ++kb, ++it) {
          const int s = (int)(it % kStages);
          if (!mbar_wait(full0 + 8 * s, (uint32_t)((it / kStages) & 1), g.err)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t a0 = smem_u32(stages + (size_t)s * kStageBytes), b0 = a0 + kABytes;
#pragma unroll
          for (int kk = 0; kk < kTK / 8; ++kk)
            mma_tf32(acc, sw128_desc(a0 + 32u * kk), sw128_desc(b0 + 32u * kk), (kb | kk) != 0 ? 1u : 0u);
          mma_commit_pair(empty0 + 8 * s);
        }
        if (ok) mma_commit(tfull0 + 8 * buf);
      }
      // every MMA issued has completed before tensor memory is freed
      mma_commit(done);
      (void)mbar_wait_drain(done, 0u, g.err);
    }
  } else {
    // epilogue: group h (warps 2 + 4h .. 5 + 4h) owns columns 128 h .. + 127 of every tile;
    // warp w reads TMEM lanes 32 (w % 4) .. + 31 = rows of the tile.  C is never loaded
    // here: each chunk of 128 rows x 16 columns of -acc goes to a shared-memory buffer and
    // is added into C by a TMA reduce (cp.reduce.async.bulk.tensor .add: L2 performs
    // C + (-acc), rounded once, the value C - acc).  Every warp runs the same sequence of
    // named barriers whatever happens (a failed wait only turns its work off), so none
    // waits for a warp that left.
    const int q = warp & 3, h = (warp - 2) >> 2;
    const bool leader = (warp == 2 + 4 * h) && lane == 0;
    unsigned char* cb = cbuf + (size_t)h * kCBufs * kCBytes;
    const int mine = cid < ntp ? (ntp - cid + ncl - 1) / ncl : 0;   // tiles of this CTA
    bool ok = true;
    long long cc = 0;
    for (int t = 0; t < mine; ++t) {
      const int buf = t & 1;
      const int tp = cid + t * ncl;
      const int x = (2 * (tp % g.mpairs) + (int)rank) * kTM;
      const int y0 = (tp / g.mpairs) * kTN + kHalfN * h;
      ok = ok && __all_sync(0xffffffffu, mbar_wait(tfull0 + 8 * buf, (uint32_t)((t >> 1) & 1), g.err));
      tc_fence_after();
      const uint32_t tbase = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(buf * kTN + kHalfN * h);
      for (int ch = 0; ch < kChunks; ++ch, ++cc) {
        uint32_t v[16];
        tmem_ld16(tbase + (uint32_t)(kCCols * ch), v);
        if (ch + 1 == kChunks) {
          // the accumulator is read: the MMAs of the tile after next may overwrite it
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(tempty0 + 8 * buf);
        }
        // the buffer's previous reduce finished reading it before the last group barrier
        float* cs = reinterpret_cast<float*>(cb + (size_t)(cc % kCBufs) * kCBytes);   // [16 columns][128 rows]
#pragma unroll
        for (int j = 0; j < kCCols; ++j) cs[j * kTM + 32 * q + lane] = -__uint_as_float(v[j]);
        // the writes above reach the TMA reduce (async proxy) after the group's barrier;
        // before it, the leader lets the reduces issued so far finish reading their buffers
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        if (leader) asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(kCBufs - 2) : "memory");
        named_bar(1 + h, 128);
        const int y = y0 + kCCols * ch;
        if (leader && ok && x < g.m && y < g.n && *(volatile int*)g.err == 0) {
          asm volatile(
              "cp.reduce.async.bulk.tensor.2d.global.shared::cta.add.tile.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                  reinterpret_cast<uint64_t>(&tmC)),
              "r"(x), "r"(y), "r"(smem_u32(cs))
              : "memory");
          asm volatile("cp.async.bulk.commit_group;" ::: "memory");
        }
      }
    }
    if (leader) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  // neither CTA leaves while its peer may still write into its shared memory
  cluster_sync_all();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
  }
}

// At[i kp + kk] = A[kk lda + i] for kk < k, 0 for k <= kk < kp (rows i < m)
__global__ void k_transpose_pad(const float* __restrict__ A, long long lda, int m, int k, int kp,
                                float* __restrict__ At) {
  __shared__ float tile[32][33];
  const int i0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += 8) {
    const int kk = k0 + r, i = i0 + threadIdx.x;
    tile[r][threadIdx.x] = (kk < k && i < m) ? A[(size_t)kk * lda + i] : 0.f;
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += 8) {
    const int i = i0 + r, kk = k0 + threadIdx.x;
    if (i < m && kk < kp) At[(size_t)i * kp + kk] = tile[threadIdx.x][r];
  }
}

using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

int32_t encode_fn(EncodeTiled* out) {
  static EncodeTiled fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiled)f;
    (void)cudaGetLastError();
  });
  if (!fn) {
    set_error("tensor-core GEMM: cuTensorMapEncodeTiled is not available");
    return O3G_ERR_CUDA;
  }
  *out = fn;
  return O3G_OK;
}

bool aligned16(const float* base, long long stride) {
  return !(reinterpret_cast<uintptr_t>(base) & 15u) && !((stride * 4) & 15);
}

// a 2-D FP32 tensor map: `inner` contiguous elements per line, `outer` lines `stride`
// elements apart; operand boxes are 32 x 128 with the 128-byte swizzle (the default), C's
// 128 x 16 unswizzled; reads outside are zeros, writes outside are dropped
int32_t make_map(CUtensorMap* map, const float* base, long long inner, long long outer, long long stride,
                 int box_inner = kTK, int box_outer = kTM, bool swizzle = true) {
  EncodeTiled enc;
  O3G_TRY(encode_fn(&enc));
  if (!aligned16(base, stride) || inner <= 0 || outer <= 0) {
    set_error("tensor-core GEMM: operand not 16-byte aligned");
    return O3G_ERR_INVALID_ARG;
  }
  const cuuint64_t dims[2] = {(cuuint64_t)inner, (cuuint64_t)outer};
  const cuuint64_t strides[1] = {(cuuint64_t)(stride * 4)};
  const cuuint32_t box[2] = {(cuuint32_t)box_inner, (cuuint32_t)box_outer};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    char msg[96];
    std::snprintf(msg, sizeof(msg), "tensor-core GEMM: cuTensorMapEncodeTiled failed (%d)", (int)r);
    set_error(msg);
    return O3G_ERR_CUDA;
  }
  return O3G_OK;
}

}  // namespace

size_t tc_gemm_scratch_floats(int m, int k) {
  const size_t kp = (size_t)(k + kTK - 1) / kTK * kTK;
  return (size_t)((m + kTM - 1) / kTM * kTM) * kp;
}

int32_t tc_gemm_sub(int m, int n, int k, const float* A, long long lda, const float* B, long long ldb, float* C,
                    long long ldc, float* at, int* err, cudaStream_t st) {
  if (m <= 0 || n <= 0 || k <= 0) return O3G_OK;
  const int kp = (k + kTK - 1) / kTK * kTK;
  k_transpose_pad<<<dim3((m + 31) / 32, kp / 32), dim3(32, 8), 0, st>>>(A, lda, m, k, kp, at);
  note_launch();
  if (!aligned16(C, ldc)) {
    set_error("tensor-core GEMM: C not 16-byte aligned (base and leading dimension)");
    return O3G_ERR_INVALID_ARG;
  }
  CUtensorMap ta, tb, tc;
  O3G_TRY(make_map(&ta, at, kp, m, kp));
  O3G_TRY(make_map(&tb, B, k, n, ldb));
  O3G_TRY(make_map(&tc, C, m, n, ldc, kTM, kCCols, false));
  static std::once_flag attr;
  static cudaError_t attr_err = cudaSuccess;
  std::call_once(attr, [] {
    attr_err = cudaFuncSetAttribute(k_tc_gemm_sub, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGemmSmem);
  });
  O3G_CUDA_TRY(attr_err);
  const int mtiles = (m + kTM - 1) / kTM;
  GemmArgs g{C, ldc, m, n, kp / kTK, (mtiles + 1) / 2, (n + kTN - 1) / kTN, err};
  // persistent: as many pairs as can be resident at once (a GPC may leave an SM unpaired)
  static std::once_flag occ;
  static int max_pairs = 0;
  static cudaError_t occ_err = cudaSuccess;
  std::call_once(occ, [] {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(2, 1, 1);
    cfg.blockDim = dim3(kGemmThreads, 1, 1);
    cfg.dynamicSmemBytes = kGemmSmem;
    occ_err = cudaOccupancyMaxActiveClusters(&max_pairs, (const void*)k_tc_gemm_sub, &cfg);
  });
  O3G_CUDA_TRY(occ_err);
  if (max_pairs < 1) {
    set_error("tensor-core GEMM: no CTA pair can be resident");
    return O3G_ERR_CUDA;
  }
  const int pairs = std::max(1, std::min(g.mpairs * g.ntiles, max_pairs));
  k_tc_gemm_sub<<<2 * pairs, kGemmThreads, kGemmSmem, st>>>(ta, tb, tc, g);
  note_launch();
  O3G_CUDA_TRY(cudaGetLastError());
  return O3G_OK;
}

}  // namespace o3g

extern "C" int32_t o3g_gemm_tf32_sub(int32_t m, int32_t n, int32_t k, const float* A, int64_t lda, const float* B,
                                     int64_t ldb, float* C, int64_t ldc, void* stream) {
  using namespace o3g;
  if (m < 0 || n < 0 || k < 0 || (m > 0 && k > 0 && (!A || lda < m)) || (n > 0 && k > 0 && (!B || ldb < k)) ||
      (m > 0 && n > 0 && (!C || ldc < m))) {
    set_error("o3g_gemm_tf32_sub: bad sizes or pointers");
    return O3G_ERR_INVALID_ARG;
  }
  if (m == 0 || n == 0 || k == 0) return O3G_OK;
  DeviceFacts df;
  O3G_TRY(device_facts(&df));
  cudaStream_t st = (cudaStream_t)stream;
  Workspace* ws = nullptr;
  const size_t at_bytes = align_up(tc_gemm_scratch_floats(m, k) * sizeof(float));
  // the epilogue moves C by TMA, which wants a 16-byte aligned base and leading dimension:
  // any other C goes through an aligned copy
  const bool direct = aligned16(C, ldc);
  const long long cld = direct ? ldc : (m + 3) / 4 * 4;
  const size_t c_bytes = direct ? 0 : align_up((size_t)cld * n * sizeof(float));
  O3G_TRY(workspace_get(st, at_bytes + c_bytes + 256, &ws));
  float* at = reinterpret_cast<float*>(ws->base);
  float* cw = direct ? C : reinterpret_cast<float*>(ws->base + at_bytes);
  int* err = reinterpret_cast<int*>(ws->base + at_bytes + c_bytes);
  O3G_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), st));
  if (!direct)
    O3G_CUDA_TRY(cudaMemcpy2DAsync(cw, cld * sizeof(float), C, ldc * sizeof(float), (size_t)m * sizeof(float), n,
                                   cudaMemcpyDeviceToDevice, st));
  O3G_TRY(tc_gemm_sub(m, n, k, A, lda, B, ldb, cw, cld, at, err, st));
  if (!direct)
    O3G_CUDA_TRY(cudaMemcpy2DAsync(C, ldc * sizeof(float), cw, cld * sizeof(float), (size_t)m * sizeof(float), n,
                                   cudaMemcpyDeviceToDevice, st));
  int herr = 0;
  O3G_CUDA_TRY(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  O3G_CUDA_TRY(cudaStreamSynchronize(st));
  if (herr) {
    set_error("o3g_gemm_tf32_sub: a pipeline wait timed out");
    return O3G_ERR_TIMEOUT;
  }
  return O3G_OK;
}
