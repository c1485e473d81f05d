// o3g_bem.cu -- the BEM system of the boundary solve: BEM<S,I> (BEM.h:44-234).
//
// The reference holds a dense Eigen matrix and solves it with GMRES (BEM.h:182-202),
// checking ||Ax-b||/||b|| afterwards (:227-230).  Here the matrix lives on the device and
// is solved by
//   * an FP32 LU factorisation with partial pivoting (row-by-row the same pivot choice
//     as LAPACK's getrf: largest magnitude, first index on ties), panels of kNb columns:
//       - k_panel_lu: one cooperative kernel factors the whole kNb-column panel; each
//         block keeps its slab of rows in shared memory; per column every block publishes
//         its pivot candidate (the whole row, and the diagonal row if it holds it) and then
//         a tagged 64-bit key with release semantics; every block polls all keys (relaxed
//         loads issued together, then a fence), so one round of stores and polls is the
//         column's grid barrier and its exchange.
//         Each block updates the next column first, publishes its next candidate, and runs
//         the rest of the rank-1 update while the other blocks publish;
//       - k_laswp: the panel's row interchanges applied to the other columns;
//       - k_trsm_unit_lower: U12 = L11^-1 A12, one warp per column, L11 in shared memory;
//       - trailing update A22 -= L21 U12 on the tensor cores (o3g_tcgemm.cu: tcgen05, TF32
//         products, FP32 sums), two-level blocking so the big updates have k = 512;
//   * iterative refinement: residuals r = b - A x formed FP64-accurately (double-single
//     FP32 arithmetic, k_matvec_ds) from the unfactored FP32 matrix and the FP64 iterate,
//     corrections from the FP32 factors (forward/back substitution in one cooperative kernel
//     each), until ||r||/||b|| <= tol;
//   * or, without any factorisation, restarted GMRES -- the reference's own solver
//     (BEM.h:182-202) -- with FP64 Krylov vectors, classical Gram-Schmidt with one
//     reorthogonalisation, and the same FP64-accurate products (o3g_bem_solve_gmres).
// Every grid barrier and key poll here spins at most kSpinLimit rounds, then sets an error
// flag that all blocks check, so a fault in the barrier logic ends the kernel instead of
// hanging.
#include "o3g_common.cuh"


#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

namespace o3g {

constexpr int kNb = 128;              // panel width
constexpr int kNbOuter = 512;         // outer panel width: k of the big trailing updates
constexpr int kPanelThreads = 512;
constexpr int kSolveThreads = 1024;
constexpr unsigned long long kSpinLimit = 1ull << 25;

constexpr unsigned long long kTestSpinLimit = 1ull << 14;   // the wait test's limit (~1 ms)

struct Barrier {
  unsigned* count;
  int* err;
  unsigned long long limit;   // polls before giving up
  unsigned extra;             // 0; 1 in the wait test: one more arrival than blocks, never met
};

// the barrier over the handle's flag words (arrival counter, error), with the spin limit,
// or in the wait test the unreachable count and the short limit
inline Barrier make_barrier(int* flags) {
  const bool test = wait_test_on();
  return Barrier{(unsigned*)(flags + 2), flags, test ? kTestSpinLimit : kSpinLimit, test ? 1u : 0u};
}

// Grid-wide barrier on one arrival counter that only grows.  The host zeroes the counter
// before each cooperative launch (zero_barrier); the k-th barrier of the launch is passed
// when the counter reaches k * gridDim.x.  One atomic per block and acquire loads of one
// word: no reset or generation step on the critical path.  Bounded: the wait returns false
// (in every thread) once the error flag is set, by a timeout here or anywhere else.
//
// grid_arrive (thread 0, after a __syncthreads that orders the block's writes before it)
// returns the count that passes this barrier; grid_wait (every thread) waits for it.  Work
// between the two overlaps the other blocks' arrivals.  Consecutive waits must be separated
// by a __syncthreads (the result word is shared).
__device__ __forceinline__ unsigned grid_arrive(const Barrier& b) {
  __threadfence();
  const unsigned arrived = atomicAdd(b.count, 1u) + 1u;
  return (arrived + gridDim.x - 1u) / gridDim.x * gridDim.x + b.extra;
}

__device__ bool grid_wait(const Barrier& b, unsigned target) {
  __shared__ int ok;
  if (threadIdx.x == 0) {
    unsigned long long it = 0;
    for (;;) {
      unsigned c;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(c) : "l"(b.count) : "memory");
      if (c >= target) break;
      if ((it & 63ull) == 63ull && *(volatile int*)b.err) break;
      if (++it > b.limit) {
        atomicExch(b.err, 1);
        break;
      }
    }
    __threadfence();
    ok = (*(volatile int*)b.err == 0);
  }
  __syncthreads();
  return ok != 0;
}

__device__ bool grid_sync(const Barrier& b) {
  __syncthreads();
  unsigned target = 0;
  if (threadIdx.x == 0) target = grid_arrive(b);
  return grid_wait(b, target);
}

// zeroes the arrival counter of make_barrier(flags) before a cooperative launch
inline cudaError_t zero_barrier(int* flags, cudaStream_t st) { return cudaMemsetAsync(flags + 2, 0, sizeof(int), st); }

// global -> shared copy of a column-major rows x cols block (leading dimension ld), with 8
// loads in flight per thread before the stores (a plain load->store loop is latency-bound)
__device__ __forceinline__ void stage_in(float* __restrict__ dst, int ldd, const float* __restrict__ src, long long ld,
                                         int rows, int cols) {
  const int total = rows * cols;
  for (int e0 = threadIdx.x; e0 < total; e0 += 8 * blockDim.x) {
    float v[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int e = e0 + q * blockDim.x;
      v[q] = e < total ? __ldg(src + (size_t)(e / rows) * ld + (e % rows)) : 0.f;
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int e = e0 + q * blockDim.x;
      if (e < total) dst[(size_t)(e / rows) * ldd + (e % rows)] = v[q];
    }
  }
}
__device__ __forceinline__ void stage_out(float* __restrict__ dst, long long ld, const float* __restrict__ src, int lds,
                                          int rows, int cols) {
  const int total = rows * cols;
  for (int e = threadIdx.x; e < total; e += blockDim.x) dst[(size_t)(e / rows) * ld + (e % rows)] = src[(size_t)(e / rows) * lds + (e % rows)];
}

struct PanelArgs {
  float* A;
  long long ld;
  int n, k0, jb, R;        // matrix order, first panel column, panel width, rows per block
  int* piv;                // absolute pivot row of each column
  unsigned long long* keys;  // [2][G] tagged pivot candidates (panel_key)
  unsigned long long* crows; // [2][G][jb] candidate rows, tagged words (panel_word)
  unsigned long long* drow;  // [2][jb] diagonal rows, tagged words
  int* singular;           // first singular column + 1, or 0
  unsigned tag0;           // tag of column 0 of this panel (nonzero; see panel_key)
  Barrier bar;             // error word, poll limit and the wait test's offset
};

// A block's pivot candidate for one panel column as one 64-bit word:
//   bits 42-63  tag = (tag0 + column) mod 2^22: which launch and column the word is for;
//   bits 10-41  |value| bits + 1 (0: no finite candidate);
//   bits 0-9    the candidate's row offset inside the block's slab (R <= 1023).
// The rows themselves travel as 64-bit words too (panel_word): the value's bits and the
// full 32-bit tag.  Every word names its column, so no store needs to be ordered before
// another: readers poll the keys, then read the winner's row and re-read any word whose
// tag is not yet the column's.  One round of relaxed stores and polls is the grid barrier
// and the exchange.  The host zeroes keys and rows before each factorisation and numbers
// the panels from 1, so no word is ever mistaken for a later column's.
__device__ __forceinline__ unsigned long long panel_key(unsigned tag, float v, int rowoff) {
  const unsigned long long vk = v >= 0.f ? (unsigned long long)__float_as_uint(v) + 1ull : 0ull;
  return ((unsigned long long)(tag & 0x3FFFFFu) << 42) | (vk << 10) | (unsigned long long)rowoff;
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
constexpr int kMaxKeysPerLane = 8;   // up to 256 panel blocks
__device__ __forceinline__ void st_relaxed_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long panel_word(unsigned tag, float v) {
  return ((unsigned long long)tag << 32) | (unsigned long long)__float_as_uint(v);
}

__device__ __forceinline__ void argmax_merge(float& v, int& i, float ov, int oi) {
  if (ov > v || (ov == v && oi < i)) { v = ov; i = oi; }
}

// The block's candidate for panel column jc: the block argmax of (best, bi), then warp 0
// writes the whole candidate row and its key, and warp 1 the diagonal row k0 + jc if this
// block holds it; no barrier after (every word is tagged).  Rows go out in their state
// after column jc - 1's elimination: in the slab that update is still pending for the
// columns beyond jc, so warps 0 and 1 apply it to their row here (the same fmaf as the
// rest of the slab) and write it back; the other rows get it in the caller's loop, which
// skips the two returned rows (-1: none).
__device__ __forceinline__ void panel_publish(const PanelArgs& a, float* slab, const float* prow, int jc,
                                              bool pending, float best, int bi, float* rv, int* ri, int r0, int nr,
                                              int& done_cand, int& done_diag) {
  const int G = gridDim.x, b = blockIdx.x, jb = a.jb, R = a.R, par = jc & 1;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const unsigned tag = a.tag0 + (unsigned)jc;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    argmax_merge(best, bi, __shfl_xor_sync(0xffffffffu, best, o), __shfl_xor_sync(0xffffffffu, bi, o));
  if (lane == 0) { rv[warp] = best; ri[warp] = bi; }
  __syncthreads();
  // the block's candidate, found by every warp alike
  float v = lane < kPanelThreads / 32 ? rv[lane] : -1.f;
  int i = lane < kPanelThreads / 32 ? ri[lane] : 0x7fffffff;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    argmax_merge(v, i, __shfl_xor_sync(0xffffffffu, v, o), __shfl_xor_sync(0xffffffffu, i, o));
  const int c = a.k0 + jc;
  const bool has_cand = v >= 0.f;
  const bool has_diag = c >= r0 && c < r0 + nr;
  done_cand = has_cand ? i - r0 : -1;
  done_diag = (has_diag && !(has_cand && i == c)) ? c - r0 : -1;
  // one warp per published row: the update applied and written back, the words out to
  // dst (and to dst2 when the candidate is the diagonal row itself)
  auto put_row = [&](unsigned long long* dst, unsigned long long* dst2, int rr) {
    const float l = pending ? slab[(size_t)(jc - 1) * R + rr] : 0.f;
    for (int jj = lane; jj < jb; jj += 32) {
      float x = slab[(size_t)jj * R + rr];
      if (pending && jj > jc) {
        x = fmaf(-l, prow[jj], x);
        slab[(size_t)jj * R + rr] = x;
      }
      st_relaxed_u64(dst + jj, panel_word(tag, x));
      if (dst2) st_relaxed_u64(dst2 + jj, panel_word(tag, x));
    }
  };
  if (warp == 0) {
    if (has_cand)
      put_row(a.crows + ((size_t)par * G + b) * jb, (has_diag && i == c) ? a.drow + par * jb : nullptr, i - r0);
    if (lane == 0) st_relaxed_u64(a.keys + (size_t)par * G + b, panel_key(tag, v, has_cand ? i - r0 : 0));
  } else if (warp == 1 && done_diag >= 0) {
    put_row(a.drow + par * jb, nullptr, c - r0);
  }
}

// Warp 0: waits (bounded) until every block's key for column j is out, then the pivot
// (largest |value|, first row on ties; the same answer in every block), the pivot row into
// prow and, when this block holds the pivot row, the diagonal row into dsw.  Returns the
// pivot row (absolute), or -1 after a timeout or another block's error.
__device__ int panel_collect(const PanelArgs& a, int j, float* prow, float* dsw, int r0, int nr) {
  const int G = gridDim.x, jb = a.jb, par = j & 1, lane = threadIdx.x & 31;
  const int c = a.k0 + j;
  const unsigned tag = (a.tag0 + (unsigned)j + a.bar.extra) & 0x3FFFFFu;
  float v = -1.f;
  int i = 0x7fffffff, ow = -1;
  // this lane's keys (G <= 32 kMaxKeysPerLane blocks), polled together with relaxed loads
  unsigned long long k[kMaxKeysPerLane];
  unsigned pending = 0;
#pragma unroll
  for (int q = 0; q < kMaxKeysPerLane; ++q)
    if (lane + 32 * q < G) pending |= 1u << q;
  bool ok = true;
  for (unsigned long long it = 0; pending; ++it) {
#pragma unroll
    for (int q = 0; q < kMaxKeysPerLane; ++q)
      if (pending & (1u << q)) k[q] = ld_relaxed_u64(a.keys + (size_t)par * G + lane + 32 * q);
#pragma unroll
    for (int q = 0; q < kMaxKeysPerLane; ++q)
      if ((pending & (1u << q)) && (unsigned)(k[q] >> 42) == tag) pending &= ~(1u << q);
    if (!pending) break;
    if ((it & 63ull) == 63ull && *(volatile int*)a.bar.err) { ok = false; break; }
    if (it > a.bar.limit) {
      atomicExch(a.bar.err, 1);
      ok = false;
      break;
    }
  }
  if (__any_sync(0xffffffffu, !ok)) return -1;
#pragma unroll
  for (int q = 0; q < kMaxKeysPerLane; ++q) {
    const int g = lane + 32 * q;
    if (g >= G) break;
    const unsigned vk = (unsigned)(k[q] >> 10);
    if (vk != 0u) {
      const float gv = __uint_as_float(vk - 1u);
      const int gi = a.k0 + g * a.R + (int)(k[q] & 1023ull);
      if (gv > v || (gv == v && gi < i)) { v = gv; i = gi; ow = g; }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float ov = __shfl_xor_sync(0xffffffffu, v, o);
    const int oi = __shfl_xor_sync(0xffffffffu, i, o);
    const int oo = __shfl_xor_sync(0xffffffffu, ow, o);
    if (ov > v || (ov == v && oi < i)) { v = ov; i = oi; ow = oo; }
  }
  if (!(v >= 0.f) || i < c || i >= a.n || ow < 0) {   // no finite candidate (a NaN column): keep the row
    i = c;
    ow = -1;
    v = 0.f;
  }
  // the rows: every word read until it carries this column's tag (the stores are not
  // ordered with the key's); bounded like the keys
  const unsigned wtag = a.tag0 + (unsigned)j + a.bar.extra;
  const bool mine = i >= r0 && i < r0 + nr && i != c;
  const unsigned long long* src = ow >= 0 ? a.crows + ((size_t)par * G + ow) * jb : a.drow + par * jb;
  // this lane's words of a row (jb <= 128: at most 4), loaded together, stale ones again
  auto fetch = [&](const unsigned long long* p, float* out) -> bool {
    constexpr int kW = kNb / 32;
    unsigned long long w[kW];
    unsigned stale = 0;
#pragma unroll
    for (int q = 0; q < kW; ++q)
      if (lane + 32 * q < jb) stale |= 1u << q;
    for (unsigned long long it = 0; stale; ++it) {
#pragma unroll
      for (int q = 0; q < kW; ++q)
        if (stale & (1u << q)) w[q] = ld_relaxed_u64(p + lane + 32 * q);
#pragma unroll
      for (int q = 0; q < kW; ++q)
        if ((stale & (1u << q)) && (unsigned)(w[q] >> 32) == wtag) stale &= ~(1u << q);
      if (!stale) break;
      if (it > a.bar.limit || ((it & 63ull) == 63ull && *(volatile int*)a.bar.err)) {
        atomicExch(a.bar.err, 1);
        return false;
      }
    }
#pragma unroll
    for (int q = 0; q < kW; ++q)
      if (lane + 32 * q < jb) out[lane + 32 * q] = __uint_as_float((unsigned)w[q]);
    return true;
  };
  ok = fetch(src, prow);
  if (ok && mine) ok = fetch(a.drow + par * jb, dsw);
  if (__any_sync(0xffffffffu, !ok)) return -1;
  if (lane == 0 && blockIdx.x == 0) {
    a.piv[c] = i;
    if (!(v > 0.f) && *a.singular == 0) *a.singular = c + 1;
  }
  return i;
}

// Partial-pivoting LU of the panel's jb columns, rows k0..n-1 spread over the blocks (R rows
// each, kept in shared memory).  Per column: every block publishes its candidate (its key
// last, with release semantics), then polls all blocks' keys; every block finds the same
// pivot, swaps, forms its multipliers and updates the next column first -- enough for the
// next candidate, which is published at once -- and only then updates the rest of its
// rows, while the other blocks publish.
__global__ void __launch_bounds__(kPanelThreads) k_panel_lu(PanelArgs a) {
  extern __shared__ float smem[];
  const int jb = a.jb, R = a.R;
  const int warp = threadIdx.x >> 5;
  float* slab = smem;                       // [jb][R]
  float* prow = smem + (size_t)jb * R;      // [jb] pivot row
  float* dsw = prow + jb;                   // [jb] diagonal row, for the swap
  __shared__ float rv[kPanelThreads / 32];
  __shared__ int ri[kPanelThreads / 32];
  __shared__ int sg_row;
  const int r0 = a.k0 + blockIdx.x * R;
  const int nr = max(0, min(a.n, r0 + R) - r0);
  if (nr > 0) stage_in(slab, R, a.A + (size_t)a.k0 * a.ld + r0, a.ld, nr, jb);
  __syncthreads();
  {
    float best = -1.f;
    int bi = 0x7fffffff;
    for (int r = threadIdx.x; r < nr; r += blockDim.x) argmax_merge(best, bi, fabsf(slab[r]), r0 + r);
    int dc, dd;
    panel_publish(a, slab, prow, 0, false, best, bi, rv, ri, r0, nr, dc, dd);
  }
  for (int j = 0; j < jb; ++j) {
    const int c = a.k0 + j;
    if (warp == 0) {
      const int pi = panel_collect(a, j, prow, dsw, r0, nr);
      if ((threadIdx.x & 31) == 0) sg_row = pi;
    }
    __syncthreads();
    const int prow_i = sg_row;
    if (prow_i < 0) return;
    if (prow_i != c) {
      if (c >= r0 && c < r0 + nr)
        for (int jj = threadIdx.x; jj < jb; jj += blockDim.x) slab[(size_t)jj * R + (c - r0)] = prow[jj];
      if (prow_i >= r0 && prow_i < r0 + nr)
        for (int jj = threadIdx.x; jj < jb; jj += blockDim.x) slab[(size_t)jj * R + (prow_i - r0)] = dsw[jj];
      __syncthreads();
    }
    // multipliers and the next column, with the next column's local argmax on the fly
    const float p = prow[j];
    const bool nxt = (j + 1 < jb);
    float best = -1.f;
    int bi = 0x7fffffff;
    for (int r = threadIdx.x; r < nr; r += blockDim.x) {
      if (r0 + r <= c) continue;
      float* row = slab + r;
      if (p != 0.f) {
        const float l = row[(size_t)j * R] / p;
        row[(size_t)j * R] = l;
        if (nxt) row[(size_t)(j + 1) * R] = fmaf(-l, prow[j + 1], row[(size_t)(j + 1) * R]);
      }
      if (nxt) argmax_merge(best, bi, fabsf(row[(size_t)(j + 1) * R]), r0 + r);
    }
    if (!nxt) break;
    int done_cand, done_diag;
    panel_publish(a, slab, prow, j + 1, p != 0.f, best, bi, rv, ri, r0, nr, done_cand, done_diag);
    // the rest of the rank-1 update (the published rows have theirs), eight loads in flight
    // per thread
    if (p != 0.f) {
      for (int r = threadIdx.x; r < nr; r += blockDim.x) {
        if (r0 + r <= c || r == done_cand || r == done_diag) continue;
        float* row = slab + r;
        const float l = row[(size_t)j * R];
        int jj = j + 2;
        for (; jj + 8 <= jb; jj += 8) {
          float v[8], q[8];
#pragma unroll
          for (int t = 0; t < 8; ++t) {
            v[t] = row[(size_t)(jj + t) * R];
            q[t] = prow[jj + t];
          }
#pragma unroll
          for (int t = 0; t < 8; ++t) row[(size_t)(jj + t) * R] = fmaf(-l, q[t], v[t]);
        }
        for (; jj < jb; ++jj) row[(size_t)jj * R] = fmaf(-l, prow[jj], row[(size_t)jj * R]);
      }
    }
    __syncthreads();
  }
  __syncthreads();
  if (nr > 0) stage_out(a.A + (size_t)a.k0 * a.ld + r0, a.ld, slab, R, nr, jb);
}

// row interchanges p0..p1-1 (piv) applied to the columns [c0, c1) outside [s0, s1).  Each
// block first composes the interchanges into one permutation of the rows they touch (the
// np rows [p0, p1) and the distinct pivot rows below p1): slot s holds row rowof[s], and
// after all interchanges the value of slot perm[s] ends up in slot s.  Then one warp per
// column gathers the touched values and scatters them permuted: two parallel passes per
// column instead of a chain of dependent loads.
// dynamic shared memory for np interchanges: 8 warps' segments of 2 np floats, then pv,
// slot_of (np ints each), rowof, perm (2 np ints each)
inline size_t laswp_smem(int np_) { return (size_t)(8 * 2 * np_ + 6 * np_) * 4; }
__global__ void __launch_bounds__(256) k_laswp(float* A, long long ld, int n, int p0, int p1, const int* piv, int c0,
                                               int c1, int s0, int s1) {
  extern __shared__ float lsw[];
  const int np_ = p1 - p0;
  float* segs = lsw;                                         // [8][2 np]
  int* pv = reinterpret_cast<int*>(segs + 8 * 2 * np_);      // [np]
  int* slot_of = pv + np_;                                   // [np]: slot of pivot row pv[e]
  int* rowof = slot_of + np_;                                // [2 np]
  int* perm = rowof + 2 * np_;                               // [2 np]
  __shared__ int nslots;
  for (int e = threadIdx.x; e < np_; e += blockDim.x) pv[e] = piv[p0 + e];
  __syncthreads();
  // the first interchange naming each pivot row below p1 (the same row can be named twice)
  for (int e = threadIdx.x; e < np_; e += blockDim.x) {
    const int p = pv[e];
    int first = e;
    if (p >= p1 && p < n)
      for (int f = 0; f < e; ++f)
        if (pv[f] == p) { first = f; break; }
    slot_of[e] = first;   // provisional: the first occurrence's index
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int ns = np_;
    for (int e = 0; e < np_; ++e) rowof[e] = p0 + e;
    for (int e = 0; e < np_; ++e) {
      const int p = pv[e];
      if (p < p1 || p >= n) {
        slot_of[e] = (p >= p0 && p < p1) ? p - p0 : -1;
      } else if (slot_of[e] == e) {
        rowof[ns] = p;
        slot_of[e] = ns++;
      } else {
        slot_of[e] = slot_of[slot_of[e]];   // the earlier occurrence's slot (already final)
      }
    }
    for (int q = 0; q < ns; ++q) perm[q] = q;
    for (int e = 0; e < np_; ++e) {
      const int p = pv[e];
      if (p == p0 + e || p < p0 + e || p >= n) continue;
      const int s2 = slot_of[e];
      const int t = perm[e];
      perm[e] = perm[s2];
      perm[s2] = t;
    }
    nslots = ns;
  }
  __syncthreads();
  const int ns = nslots;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int skip = (s1 > s0) ? (s1 - s0) : 0;
  const int ncol = c1 - c0 - skip;
  for (int t = blockIdx.x * 8 + warp; t < ncol; t += gridDim.x * 8) {
    int col = c0 + t;
    if (skip && col >= s0) col += skip;
    float* a = A + (size_t)col * ld;
    float* seg = segs + (size_t)warp * 2 * np_;
    for (int q = lane; q < ns; q += 32) seg[q] = a[rowof[perm[q]]];
    __syncwarp();
    for (int q = lane; q < ns; q += 32) a[rowof[q]] = seg[q];
    __syncwarp();
  }
}

// B = L^-1 B for a unit lower jb x jb L (column-major at Lp, leading dimension ldl) and the
// ncols columns of B (jb rows at Bp, leading dimension ldb): one warp per column of B, L in
// shared memory
__global__ void __launch_bounds__(256) k_trsm_unit_lower(const float* Lp, long long ldl, int jb, float* Bp,
                                                         long long ldb, int ncols) {
  extern __shared__ float L[];   // [jb][jb] column-major
  stage_in(L, jb, Lp, ldl, jb, jb);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int cidx = blockIdx.x * (blockDim.x / 32) + warp; cidx < ncols; cidx += gridDim.x * (blockDim.x / 32)) {
    float* col = Bp + (size_t)cidx * ldb;
    float x[kNb / 32];
#pragma unroll
    for (int q = 0; q < kNb / 32; ++q) x[q] = (q * 32 + lane < jb) ? col[q * 32 + lane] : 0.f;
    for (int i = 0; i < jb; ++i) {
      const float xi = __shfl_sync(0xffffffffu, x[i >> 5], i & 31);
#pragma unroll
      for (int q = 0; q < kNb / 32; ++q) {
        const int m = q * 32 + lane;
        if (m > i && m < jb) x[q] = fmaf(-L[(size_t)i * jb + m], xi, x[q]);
      }
    }
#pragma unroll
    for (int q = 0; q < kNb / 32; ++q)
      if (q * 32 + lane < jb) col[q * 32 + lane] = x[q];
  }
}

// identity into a jb x jb column-major block
__global__ void k_eye(float* E, int jb) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < jb * jb) E[e] = (e % jb == e / jb) ? 1.f : 0.f;
}

// C[:, j] = L T[:, j] for j < ncols in FP32: L jb x jb (leading dimension jb, jb <= kNb), T
// jb x ncols (leading dimension jb), C with leading dimension ldc.  L stays in shared memory;
// T goes through it 64 columns at a time, transposed (k-major, rows padded to 68 floats so
// the transposing stores spread over the banks).  Thread (tr, tc) of 16 x 16 owns rows
// 8 tr .. 8 tr + 7 and columns 4 tc .. 4 tc + 3 of the 128 x 64 block: per k two 16-byte
// loads of L and one of T feed 32 FMAs, summed in k order.
constexpr int kLeftCols = 64;
constexpr int kLeftLd = kLeftCols + 4;
__global__ void __launch_bounds__(256) k_left_gemm(const float* __restrict__ L, int jb, const float* __restrict__ T,
                                                   int ncols, float* __restrict__ C, long long ldc) {
  extern __shared__ float4 lsm4[];
  float* Ls = reinterpret_cast<float*>(lsm4);   // [k][kNb], zero beyond jb
  float* Ts = Ls + (size_t)kNb * kNb;            // [k][kLeftLd]
  // staging: 8 loads in flight per thread before their stores (a load -> store loop waits
  // out the full memory latency at every element)
  for (int e0 = threadIdx.x; e0 < kNb * kNb; e0 += 8 * blockDim.x) {
    float v[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int e = e0 + q * blockDim.x, kk = e / kNb, r = e % kNb;
      v[q] = (e < kNb * kNb && kk < jb && r < jb) ? __ldg(L + (size_t)kk * jb + r) : 0.f;
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int e = e0 + q * blockDim.x;
      if (e < kNb * kNb) Ls[e] = v[q];
    }
  }
  const int tr = threadIdx.x & 15, tc = threadIdx.x >> 4;
  for (int c0 = blockIdx.x * kLeftCols; c0 < ncols; c0 += gridDim.x * kLeftCols) {
    const int nc = min(kLeftCols, ncols - c0);
    __syncthreads();
    for (int e0 = threadIdx.x; e0 < kLeftCols * jb; e0 += 8 * blockDim.x) {
      float v[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int e = e0 + q * blockDim.x, c = e / jb, kk = e % jb;
        v[q] = (e < kLeftCols * jb && c < nc) ? __ldg(T + (size_t)(c0 + c) * jb + kk) : 0.f;
      }
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int e = e0 + q * blockDim.x, c = e / jb, kk = e % jb;
        if (e < kLeftCols * jb) Ts[(size_t)kk * kLeftLd + c] = v[q];
      }
    }
    __syncthreads();
    float acc[8][4];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[i][c] = 0.f;
#pragma unroll 4
    for (int kk = 0; kk < jb; ++kk) {
      const float4 a0 = *reinterpret_cast<const float4*>(Ls + (size_t)kk * kNb + 8 * tr);
      const float4 a1 = *reinterpret_cast<const float4*>(Ls + (size_t)kk * kNb + 8 * tr + 4);
      const float4 b = *reinterpret_cast<const float4*>(Ts + (size_t)kk * kLeftLd + 4 * tc);
      const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      const float bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[i][c] = fmaf(av[i], bv[c], acc[i][c]);
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int col = 4 * tc + c;
      if (col < nc)
#pragma unroll
        for (int i = 0; i < 8; ++i)
          if (8 * tr + i < jb) C[(size_t)(c0 + col) * ldc + 8 * tr + i] = acc[i][c];
    }
  }
}

// ------------------------------------------------------------------------------------
// solves with the factors: y = P b (gather), L y = y (unit lower), U x = y (upper)
__global__ void k_permute_to_float(const double* r, const int* perm, float* y, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = (float)r[perm[i]];
}

// sum_m col[m*ld] * yd[m] for m < jb; the full-width case is unrolled so every load of the
// row is in flight at once (the loop is latency-bound otherwise)
__device__ __forceinline__ float panel_dot(const float* __restrict__ col, long long ld, const float* yd, int jb) {
  if (jb == kNb) {
    float s[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int m = 0; m < kNb; ++m) s[m & 7] = fmaf(__ldg(col + (size_t)m * ld), yd[m], s[m & 7]);
    return ((s[0] + s[1]) + (s[2] + s[3])) + ((s[4] + s[5]) + (s[6] + s[7]));
  }
  float s = 0.f;
  for (int m = 0; m < jb; ++m) s = fmaf(col[(size_t)m * ld], yd[m], s);
  return s;
}

// Inverses of the diagonal kNb x kNb blocks of the factors, one block per CUDA block:
// Linv (unit lower) and Uinv (upper) column-major at dinv + kb*2*kNb*kNb (+kNb*kNb).
// Columns of the identity are solved by one warp each (forward / back substitution).
__global__ void __launch_bounds__(256) k_diag_inverses(const float* __restrict__ LU, long long ld, int n,
                                                       float* __restrict__ dinv) {
  extern __shared__ float D[];   // [jb][jb] diagonal block
  const int kb = blockIdx.x, k0 = kb * kNb, jb = min(kNb, n - k0);
  stage_in(D, jb, LU + (size_t)k0 * ld + k0, ld, jb, jb);
  __syncthreads();
  float* Li = dinv + (size_t)kb * 2 * kNb * kNb;
  float* Ui = Li + (size_t)kNb * kNb;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int c = warp; c < jb; c += blockDim.x / 32) {
    float x[kNb / 32];
    // L x = e_c
#pragma unroll
    for (int q = 0; q < kNb / 32; ++q) x[q] = (q * 32 + lane == c) ? 1.f : 0.f;
    for (int i = c; i < jb; ++i) {
      const float xi = __shfl_sync(0xffffffffu, x[i >> 5], i & 31);
#pragma unroll
      for (int q = 0; q < kNb / 32; ++q) {
        const int m = q * 32 + lane;
        if (m > i && m < jb) x[q] = fmaf(-D[(size_t)i * jb + m], xi, x[q]);
      }
    }
#pragma unroll
    for (int q = 0; q < kNb / 32; ++q) {
      const int m = q * 32 + lane;
      if (m < kNb) Li[(size_t)c * kNb + m] = m < jb ? x[q] : 0.f;
    }
    // U x = e_c
#pragma unroll
    for (int q = 0; q < kNb / 32; ++q) x[q] = (q * 32 + lane == c) ? 1.f : 0.f;
    for (int i = c; i >= 0; --i) {
      if ((i & 31) == lane) x[i >> 5] = x[i >> 5] / D[(size_t)i * jb + i];
      const float xi = __shfl_sync(0xffffffffu, x[i >> 5], i & 31);
#pragma unroll
      for (int q = 0; q < kNb / 32; ++q) {
        const int m = q * 32 + lane;
        if (m < i) x[q] = fmaf(-D[(size_t)i * jb + m], xi, x[q]);
      }
    }
#pragma unroll
    for (int q = 0; q < kNb / 32; ++q) {
      const int m = q * 32 + lane;
      if (m < kNb) Ui[(size_t)c * kNb + m] = m < jb ? x[q] : 0.f;
    }
  }
}

// yd = Dinv y[k0 : k0+jb] (Dinv kNb x kNb column-major) by the whole block
__device__ __forceinline__ void diag_apply(const float* __restrict__ Dinv, const float* y, int jb, float* yin,
                                           float* part, float* yd) {
  if (threadIdx.x < jb) yin[threadIdx.x] = y[threadIdx.x];
  __syncthreads();
  constexpr int kQ = kSolveThreads / kNb;   // 8 column chunks
  const int m = threadIdx.x % kNb, q = threadIdx.x / kNb;
  float s = 0.f;
  if (m < jb) {
    for (int k = q * (kNb / kQ); k < (q + 1) * (kNb / kQ); ++k)
      if (k < jb) s = fmaf(__ldg(Dinv + (size_t)k * kNb + m), yin[k], s);
  }
  part[q * kNb + m] = s;
  __syncthreads();
  if (threadIdx.x < jb) {
    float t = 0.f;
#pragma unroll
    for (int qq = 0; qq < kQ; ++qq) t += part[qq * kNb + threadIdx.x];
    yd[threadIdx.x] = t;
  }
  __syncthreads();
}

// y[i] -= sum_m M(i, k0+m) yd[m] for the rows [i0, i1) of this block: the 128 columns are
// split in 4 chunks of 32 so every thread of the block has loads in flight (one row per
// thread leaves most threads idle and each row latency-bound); partials meet in `part`
__device__ __forceinline__ void update_rows(const float* __restrict__ LU, long long ld, int k0, int jb, int i0, int i1,
                                            const float* yd, float* y, float* part) {
  const int nr = i1 - i0;
  if (nr <= 0) return;
  if (jb != kNb) {
    for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) y[i] -= panel_dot(LU + (size_t)k0 * ld + i, ld, yd, jb);
    return;
  }
  constexpr int kChunks = 4, kW = kNb / kChunks;
  for (int r0 = 0; r0 < nr; r0 += kSolveThreads / kChunks) {
    const int rows = min(kSolveThreads / kChunks, nr - r0);
    const int q = threadIdx.x / (kSolveThreads / kChunks), r = threadIdx.x % (kSolveThreads / kChunks);
    if (r < rows) {
      const float* col = LU + (size_t)(k0 + q * kW) * ld + i0 + r0 + r;
      float s[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int m = 0; m < kW; ++m) s[m & 3] = fmaf(__ldg(col + (size_t)m * ld), yd[q * kW + m], s[m & 3]);
      part[q * (kSolveThreads / kChunks) + r] = (s[0] + s[1]) + (s[2] + s[3]);
    }
    __syncthreads();
    if (threadIdx.x < rows) {
      const int rr = threadIdx.x;
      float t = 0.f;
#pragma unroll
      for (int qq = 0; qq < kChunks; ++qq) t += part[qq * (kSolveThreads / kChunks) + rr];
      y[i0 + r0 + rr] -= t;
    }
    __syncthreads();
  }
}

struct TrsvArgs {
  const float* LU;
  const float* dinv;
  long long ld;
  int n;
  float* y;     // right-hand side, overwritten by the partial updates
  float* out;   // the solution: each segment, once final (never read by the kernel)
  Barrier bar;
};

// forward substitution with the unit lower factor: per block column, every block applies
// the block's inverse to the (final) y segment, then updates its share of the rows below;
// block 0 stores the solved segment in `out`, which no block reads, so it cannot overtake
// another block still reading that segment of y
__global__ void __launch_bounds__(kSolveThreads) k_trsv_lower(TrsvArgs a) {
  __shared__ float yd[kNb], yin[kNb];
  __shared__ float part[kSolveThreads];
  const int G = gridDim.x;
  for (int k0 = 0; k0 < a.n; k0 += kNb) {
    const int jb = min(kNb, a.n - k0);
    diag_apply(a.dinv + (size_t)(k0 / kNb) * 2 * kNb * kNb, a.y + k0, jb, yin, part, yd);
    const int rest = a.n - k0 - jb;
    const int chunk = (rest + G - 1) / G;
    const int i0 = k0 + jb + blockIdx.x * chunk, i1 = min(a.n, i0 + chunk);
    update_rows(a.LU, a.ld, k0, jb, i0, i1, yd, a.y, part);
    if (blockIdx.x == 0 && threadIdx.x < jb) a.out[k0 + threadIdx.x] = yd[threadIdx.x];
    if (!grid_sync(a.bar)) return;
  }
}

// back substitution with the upper factor
__global__ void __launch_bounds__(kSolveThreads) k_trsv_upper(TrsvArgs a) {
  __shared__ float yd[kNb], yin[kNb];
  __shared__ float part[kSolveThreads];
  const int G = gridDim.x;
  const int nblk = (a.n + kNb - 1) / kNb;
  for (int kb = nblk - 1; kb >= 0; --kb) {
    const int k0 = kb * kNb, jb = min(kNb, a.n - k0);
    diag_apply(a.dinv + (size_t)kb * 2 * kNb * kNb + (size_t)kNb * kNb, a.y + k0, jb, yin, part, yd);
    const int chunk = (k0 + G - 1) / G;
    const int i0 = blockIdx.x * chunk, i1 = min(k0, i0 + chunk);
    update_rows(a.LU, a.ld, k0, jb, i0, i1, yd, a.y, part);
    if (blockIdx.x == 0 && threadIdx.x < jb) a.out[k0 + threadIdx.x] = yd[threadIdx.x];
    if (!grid_sync(a.bar)) return;
  }
}

__global__ void k_axpy_f2d(double* x, const float* d, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] += (double)d[i];
}
__global__ void k_f2d(const float* s, double* d, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) d[i] = (double)s[i];
}
__global__ void k_d2f(const double* s, float* d, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) d[i] = (float)s[i];
}

// ---- FP64-accurate products of the FP32 matrix without the FP64 pipe --------------------
// x (double) is split into xh + xl (floats, ~48 significant bits together).  Each product
// a * xh is formed error-free (p + e, e = fma(a, xh, -p)), a * xl in one fma, and the row
// sum is carried as a double-single pair (hi, lo) with Knuth's two-sum, renormalised every
// 8 columns.  About 10 FP32 instructions per matrix element: the kernel streams the matrix
// at HBM speed, where the same sum on the FP64 pipe is limited by its rate.
constexpr int kMvChunk = 1024;   // columns per block (blockIdx.y)

__global__ void k_split_f64(const double* __restrict__ x, float* xh, float* xl, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double v = x[i];
  const float h = (float)v;
  xh[i] = h;
  xl[i] = (float)(v - (double)h);
}

__device__ __forceinline__ void ds_add_product(float a, float h, float l, float& hi, float& lo) {
  const float p = __fmul_rn(a, h);
  const float e = fmaf(a, h, -p);
  const float s = __fadd_rn(hi, p);
  const float bb = __fsub_rn(s, hi);
  const float t = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  hi = s;
  lo = fmaf(a, l, __fadd_rn(lo, __fadd_rn(t, e)));
}

// part[cb][i] = sum over the columns of chunk cb of A[i, j] x[j]
__global__ void __launch_bounds__(256) k_matvec_ds(const float* __restrict__ A, long long ld, int n,
                                                   const float* __restrict__ xh, const float* __restrict__ xl,
                                                   double* __restrict__ part) {
  __shared__ float sh[kMvChunk], sl[kMvChunk];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int cb = blockIdx.y;
  const int j0 = cb * kMvChunk, m = min(n - j0, kMvChunk);
  for (int k = threadIdx.x; k < m; k += blockDim.x) { sh[k] = xh[j0 + k]; sl[k] = xl[j0 + k]; }
  __syncthreads();
  if (i >= n) return;
  const float* a = A + (size_t)j0 * ld + i;
  float hi = 0.f, lo = 0.f;
  int k = 0;
  for (; k + 8 <= m; k += 8) {
    float av[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) av[q] = __ldg(a + (size_t)(k + q) * ld);
#pragma unroll
    for (int q = 0; q < 8; ++q) ds_add_product(av[q], sh[k + q], sl[k + q], hi, lo);
    // renormalise: move the bulk of lo into hi (Dekker's fast two-sum, |hi| >= |lo|)
    const float s2 = __fadd_rn(hi, lo);
    lo = __fsub_rn(lo, __fsub_rn(s2, hi));
    hi = s2;
  }
  for (; k < m; ++k) ds_add_product(__ldg(a + (size_t)k * ld), sh[k], sl[k], hi, lo);
  part[(size_t)cb * n + i] = (double)hi + (double)lo;
}

// y = b - sum_cb part (b != null) or y = sum_cb part; per-block sums of y^2 into nrm
__global__ void k_matvec_finish(const double* __restrict__ part, int ncb, int n, const double* __restrict__ b,
                                double* __restrict__ y, double* __restrict__ nrm) {
  __shared__ double s1[8];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double yy = 0.0;
  if (i < n) {
    double s = 0.0;
    for (int k = 0; k < ncb; ++k) s += part[(size_t)k * n + i];
    const double v = b ? b[i] - s : s;
    y[i] = v;
    yy = v * v;
  }
  for (int o = 16; o > 0; o >>= 1) yy += __shfl_xor_sync(0xffffffffu, yy, o);
  if ((threadIdx.x & 31) == 0) s1[threadIdx.x >> 5] = yy;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a1 = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) a1 += s1[w];
    if (nrm) nrm[blockIdx.x] = a1;
  }
}

// finalize_vels of the panel velocities (u = fs + u/(4 pi) in double, ElementBase.h:187-193
// via Surfaces.h:877-887) followed by vels_to_rhs_panels (RHS.h:92-110)
__global__ void k_vels_to_rhs(int np, int nunk, double fx, double fy, double fz, float* pu, float* pv, float* pw,
                              const float* __restrict__ x1x, const float* __restrict__ x1y,
                              const float* __restrict__ x1z, const float* __restrict__ x2x,
                              const float* __restrict__ x2y, const float* __restrict__ x2z,
                              const float* __restrict__ nx, const float* __restrict__ ny,
                              const float* __restrict__ nz, float* rhs) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const double factor = 0.25 / 3.14159265358979323846;
  const float u = (float)(fx + (double)pu[i] * factor);
  const float v = (float)(fy + (double)pv[i] * factor);
  const float w = (float)(fz + (double)pw[i] * factor);
  pu[i] = u;
  pv[i] = v;
  pw[i] = w;
  if (nunk == 1) {
    rhs[i] = -(__fadd_rn(__fadd_rn(__fmul_rn(u, nx[i]), __fmul_rn(v, ny[i])), __fmul_rn(w, nz[i])));
    return;
  }
  rhs[(size_t)nunk * i] = -(__fadd_rn(__fadd_rn(__fmul_rn(u, x1x[i]), __fmul_rn(v, x1y[i])), __fmul_rn(w, x1z[i])));
  rhs[(size_t)nunk * i + 1] = -(__fadd_rn(__fadd_rn(__fmul_rn(u, x2x[i]), __fmul_rn(v, x2y[i])), __fmul_rn(w, x2z[i])));
  if (nunk == 3)
    rhs[(size_t)nunk * i + 2] = -(__fadd_rn(__fadd_rn(__fmul_rn(u, nx[i]), __fmul_rn(v, ny[i])), __fmul_rn(w, nz[i])));
}

}  // namespace o3g

extern "C" int32_t o3g_panel_vels_to_rhs(int32_t np, int32_t nunk, const double* fs, float* pu, float* pv, float* pw,
                                         const o3g_surface_t* surf, float* rhs, void* stream) {
  using namespace o3g;
  if (np < 0 || nunk < 1 || nunk > 3 || !surf || surf->np != np || !fs) {
    set_error("o3g_panel_vels_to_rhs: bad sizes or null arguments");
    return O3G_ERR_INVALID_ARG;
  }
  if (np == 0) return O3G_OK;
  if (!pu || !pv || !pw || !rhs || !surf->x1x || !surf->x2x || (nunk != 2 && !surf->nx)) {
    set_error("o3g_panel_vels_to_rhs: null array");
    return O3G_ERR_INVALID_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  k_vels_to_rhs<<<(np + 255) / 256, 256, 0, st>>>(np, nunk, fs[0], fs[1], fs[2], pu, pv, pw, surf->x1x, surf->x1y,
                                                 surf->x1z, surf->x2x, surf->x2y, surf->x2z, surf->nx, surf->ny,
                                                 surf->nz, rhs);
  note_launch();
  O3G_CUDA_TRY(cudaGetLastError());
  return O3G_OK;
}

// ======================================================================================
struct o3g_bem {
  int device = -1;
  int n = 0;
  long long ld = 0;
  float* A = nullptr;     // assembled matrix (kept for residuals)
  float* LU = nullptr;    // factors
  int* piv = nullptr;     // per-column pivot rows
  int* perm = nullptr;    // composed row permutation: (P b)[i] = b[perm[i]]
  float* dinv = nullptr;  // inverses of the diagonal blocks of L and U
  char* scratch = nullptr;
  size_t scratch_bytes = 0;
  int* flags = nullptr;   // [0] barrier error, [1] singular column + 1, [2] barrier arrivals,
                          // [4] tensor-core update error
  float* tcw = nullptr;   // K-major copies of the update's left operand (n x 512)
  bool factored = false;
  int panel_blocks = 0, solve_blocks = 0;
  int bs = 1;             // unknowns per panel: GMRES preconditions with the bs x bs diagonal blocks
};

using namespace o3g;

extern "C" int32_t o3g_bem_size(const o3g_bem_t* h, int64_t* n) {
  if (!h || !n) return O3G_ERR_INVALID_ARG;
  *n = h->n;
  return O3G_OK;
}

static int32_t bem_check(o3g_bem_t* h) {
  if (!h || !h->A) {
    set_error("o3g_bem: null or destroyed handle");
    return O3G_ERR_INVALID_ARG;
  }
  int dev = -1;
  O3G_CUDA_TRY(cudaGetDevice(&dev));
  if (dev != h->device) {
    set_error("o3g_bem: handle belongs to another device");
    return O3G_ERR_STATE;
  }
  return O3G_OK;
}

extern "C" int32_t o3g_bem_create(int64_t n, o3g_bem_t** out) {
  if (!out || n <= 0 || n > (int64_t)200000) {
    set_error("o3g_bem_create: n must be in 1..200000");
    return O3G_ERR_INVALID_ARG;
  }
  *out = nullptr;
  DeviceFacts df;
  O3G_TRY(device_facts(&df));
  o3g_bem_t* h = new o3g_bem_t();
  h->device = df.device;
  h->n = (int)n;
  h->ld = (n + 31) / 32 * 32;
  const size_t mat = (size_t)h->ld * n * sizeof(float);
  cudaError_t e = o3g::dev_alloc((void**)&h->A, mat);
  if (e == cudaSuccess) e = o3g::dev_alloc((void**)&h->LU, mat);
  if (e == cudaSuccess) e = o3g::dev_alloc((void**)&h->piv, n * sizeof(int));
  if (e == cudaSuccess) e = o3g::dev_alloc((void**)&h->perm, n * sizeof(int));
  if (e == cudaSuccess) e = o3g::dev_alloc((void**)&h->flags, 64 * sizeof(int));
  if (e == cudaSuccess) e = o3g::dev_alloc((void**)&h->dinv, (size_t)((n + kNb - 1) / kNb) * 2 * kNb * kNb * sizeof(float));
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    set_error_cuda("o3g_bem_create: cudaMalloc", e);
    cudaFree(h->A); cudaFree(h->LU); cudaFree(h->piv); cudaFree(h->perm); cudaFree(h->flags); cudaFree(h->dinv);
    delete h;
    return O3G_ERR_ALLOC;
  }
  cudaMemset(h->A, 0, mat);
  *out = h;
  return O3G_OK;
}

extern "C" int32_t o3g_bem_destroy(o3g_bem_t* h) {
  if (!h) return O3G_OK;
  cudaDeviceSynchronize();
  cudaFree(h->A); cudaFree(h->LU); cudaFree(h->piv); cudaFree(h->perm); cudaFree(h->flags); cudaFree(h->scratch);
  cudaFree(h->dinv);
  cudaFree(h->tcw);
  h->A = nullptr;
  delete h;
  return O3G_OK;
}

extern "C" int32_t o3g_bem_matrix(o3g_bem_t* h, float** A, int64_t* ld) {
  O3G_TRY(bem_check(h));
  if (!A || !ld) return O3G_ERR_INVALID_ARG;
  *A = h->A;
  *ld = h->ld;
  h->factored = false;
  return O3G_OK;
}

extern "C" int32_t o3g_bem_set_unknowns_per_panel(o3g_bem_t* h, int32_t bs) {
  O3G_TRY(bem_check(h));
  if (bs < 1 || bs > 3 || h->n % bs != 0) {
    set_error("o3g_bem_set_unknowns_per_panel: bs must be 1..3 and divide n");
    return O3G_ERR_INVALID_ARG;
  }
  h->bs = bs;
  return O3G_OK;
}

extern "C" int32_t o3g_bem_set_block(o3g_bem_t* h, int64_t rstart, int64_t nrows, int64_t cstart, int64_t ncols,
                                     const float* blk, int32_t mem, void* stream) {
  O3G_TRY(bem_check(h));
  if (rstart < 0 || cstart < 0 || nrows < 0 || ncols < 0 || rstart + nrows > h->n || cstart + ncols > h->n ||
      (!blk && nrows * ncols > 0) || (mem != O3G_MEM_HOST && mem != O3G_MEM_DEVICE)) {
    set_error("o3g_bem_set_block: block outside the matrix or bad arguments");
    return O3G_ERR_INVALID_ARG;
  }
  if (nrows == 0 || ncols == 0) return O3G_OK;
  cudaStream_t st = (cudaStream_t)stream;
  O3G_CUDA_TRY(cudaMemcpy2DAsync(h->A + cstart * h->ld + rstart, h->ld * sizeof(float), blk, nrows * sizeof(float),
                                 nrows * sizeof(float), ncols,
                                 mem == O3G_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, st));
  if (mem == O3G_MEM_HOST) O3G_CUDA_TRY(cudaStreamSynchronize(st));
  h->factored = false;
  return O3G_OK;
}

static int32_t bem_scratch(o3g_bem_t* h, size_t bytes) {
  if (h->scratch_bytes >= bytes) return O3G_OK;
  O3G_CUDA_TRY(cudaDeviceSynchronize());
  cudaFree(h->scratch);
  h->scratch = nullptr;
  h->scratch_bytes = 0;
  cudaError_t e = o3g::dev_alloc((void**)&h->scratch, bytes);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    set_error_cuda("o3g_bem: scratch", e);
    return O3G_ERR_ALLOC;
  }
  h->scratch_bytes = bytes;
  return O3G_OK;
}

extern "C" int32_t o3g_bem_factor(o3g_bem_t* h, void* stream) {
  O3G_TRY(bem_check(h));
  cudaStream_t st = (cudaStream_t)stream;
  const int n = h->n;
  const long long ld = h->ld;
  DeviceFacts df;
  O3G_TRY(device_facts(&df));
  // panel kernel: co-resident blocks, each keeping R rows x kNb columns in shared memory
  int per_sm = 0, optin = 0;
  O3G_CUDA_TRY(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, df.device));
  cudaFuncAttributes fa;
  O3G_CUDA_TRY(cudaFuncGetAttributes(&fa, k_panel_lu));
  const size_t max_smem = (size_t)optin - fa.sharedSizeBytes;
  O3G_CUDA_TRY(cudaFuncSetAttribute(k_panel_lu, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem));
  int G = std::min(df.num_sms, 32 * kMaxKeysPerLane);
  int R = (n + G - 1) / G;
  size_t smem = ((size_t)kNb * R + 2 * kNb + 32) * sizeof(float);
  if (smem > max_smem) {
    set_error("o3g_bem_factor: matrix too large for the panel kernel's shared memory");
    return O3G_ERR_INVALID_ARG;
  }
  O3G_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_panel_lu, kPanelThreads, smem));
  if (per_sm < 1) {
    set_error("o3g_bem_factor: panel kernel cannot be resident");
    return O3G_ERR_INVALID_ARG;
  }
  const size_t cand = align_up((2 * (size_t)G + 2 * (size_t)G * kNb + 2 * (size_t)kNb) * sizeof(unsigned long long));
  O3G_TRY(bem_scratch(h, cand + align_up((size_t)kNb * kNb * 4) + align_up((size_t)kNb * n * 4) + (1 << 20)));
  Carve cv(h->scratch);
  // keys and tagged rows back to back, zeroed together once per factorisation
  const size_t xwords = 2 * (size_t)G + 2 * (size_t)G * kNb + 2 * (size_t)kNb;
  unsigned long long* keys = cv.take<unsigned long long>(xwords);
  unsigned long long* crows = keys + 2 * (size_t)G;
  unsigned long long* drow = crows + 2 * (size_t)G * kNb;
  O3G_CUDA_TRY(cudaMemsetAsync(h->flags, 0, 64 * sizeof(int), st));
  O3G_CUDA_TRY(cudaMemsetAsync(keys, 0, xwords * sizeof(unsigned long long), st));
  O3G_CUDA_TRY(cudaMemcpy2DAsync(h->LU, ld * sizeof(float), h->A, ld * sizeof(float), n * sizeof(float), n,
                                 cudaMemcpyDeviceToDevice, st));
  KernelTimer& tm = thread_timer();
  tm.begin(st);
  const size_t tsm = (size_t)kNb * kNb * sizeof(float);
  O3G_CUDA_TRY(cudaFuncSetAttribute(k_trsm_unit_lower, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsm));
  O3G_CUDA_TRY(cudaFuncSetAttribute(k_laswp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)laswp_smem(kNbOuter)));
  // C = C - A B on the tensor cores (o3g_tcgemm.cu: tcgen05, TF32 products, FP32 sums; all
  // operands column-major in LU); the error word of its pipeline waits is flags[4]
  if (!h->tcw) {
    const cudaError_t e = o3g::dev_alloc((void**)&h->tcw, tc_gemm_scratch_floats(n, kNbOuter) * sizeof(float));
    if (e != cudaSuccess) {
      (void)cudaGetLastError();
      h->tcw = nullptr;
      set_error_cuda("o3g_bem_factor: tensor-core scratch", e);
      return O3G_ERR_ALLOC;
    }
  }
  auto gemm = [&](int m, int nn, int kk, const float* Am, const float* Bm, float* Cm) -> int32_t {
    return tc_gemm_sub(m, nn, kk, Am, ld, Bm, ld, Cm, ld, h->tcw, h->flags + 4, st);
  };
  auto trsm = [&](int k0, int jb, int c0, int ncols) {
    if (ncols <= 0) return;
    int tb = (ncols + 7) / 8;
    if (tb > 4 * df.num_sms) tb = 4 * df.num_sms;
    k_trsm_unit_lower<<<tb, 256, (size_t)jb * jb * sizeof(float), st>>>(h->LU + (size_t)k0 * ld + k0, ld, jb,
                                                                         h->LU + (size_t)c0 * ld + k0, ld, ncols);
    note_launch();
  };
  // the same solve for a wide right-hand side: Linv = L11^-1 once (TRSM on the identity),
  // then B <- Linv B as an FP32 product (k_left_gemm) through a scratch copy
  float* linv = cv.take<float>((size_t)kNb * kNb);
  const size_t lsm_bytes = ((size_t)kNb * kNb + (size_t)kNb * kLeftLd) * sizeof(float);
  O3G_CUDA_TRY(cudaFuncSetAttribute(k_left_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lsm_bytes));
  float* tmp = cv.take<float>((size_t)kNb * n);
  auto trsm_wide = [&](int k0, int jb, int c0, int ncols) -> int32_t {
    if (ncols <= 0) return O3G_OK;
    k_eye<<<(jb * jb + 255) / 256, 256, 0, st>>>(linv, jb);
    k_trsm_unit_lower<<<(jb + 7) / 8, 256, (size_t)jb * jb * sizeof(float), st>>>(h->LU + (size_t)k0 * ld + k0, ld,
                                                                                 jb, linv, jb, jb);
    note_launch(2);
    float* B = h->LU + (size_t)c0 * ld + k0;
    O3G_CUDA_TRY(cudaMemcpy2DAsync(tmp, (size_t)jb * sizeof(float), B, ld * sizeof(float), (size_t)jb * sizeof(float),
                                   ncols, cudaMemcpyDeviceToDevice, st));
    const int lb = std::min((ncols + kLeftCols - 1) / kLeftCols, 2 * df.num_sms);
    k_left_gemm<<<lb, 256, lsm_bytes, st>>>(linv, jb, tmp, ncols, B, ld);
    note_launch();
    return O3G_OK;
  };
  auto laswp = [&](int p0, int p1, int c0, int c1, int s0, int s1) {
    const int cnt = (c1 - c0) - (s1 > s0 ? s1 - s0 : 0);
    if (cnt <= 0) return;
    const int lb = std::min((cnt + 7) / 8, 8 * df.num_sms);
    k_laswp<<<lb, 256, laswp_smem(p1 - p0), st>>>(h->LU, ld, n, p0, p1, h->piv, c0, c1, s0, s1);
    note_launch();
  };
  auto at = [&](int r, int c) { return h->LU + (size_t)c * ld + r; };
  // two-level right-looking LU: kNb-column panels inside kNbOuter-column outer panels; the
  // big trailing update of each outer panel has k = kNbOuter
  for (int K0 = 0; K0 < n; K0 += kNbOuter) {
    const int KB = std::min(kNbOuter, n - K0), K1 = K0 + KB;
    for (int k0 = K0; k0 < K1; k0 += kNb) {
      const int jb = std::min(kNb, K1 - k0);
      const int m = n - k0;
      int g = G;
      int r = (m + g - 1) / g;
      if (r < 32) {   // short panels: fewer blocks
        g = (m + 31) / 32;
        r = (m + g - 1) / g;
      }
      PanelArgs pa;
      pa.A = h->LU; pa.ld = ld; pa.n = n; pa.k0 = k0; pa.jb = jb; pa.R = r;
      pa.piv = h->piv; pa.keys = keys; pa.crows = crows; pa.drow = drow;
      pa.singular = h->flags + 1;
      pa.tag0 = (unsigned)(k0 / kNb + 1) << 7;   // panels numbered from 1: zeroed keys never match
      pa.bar = make_barrier(h->flags);
      void* args[] = {&pa};
      const size_t sm = ((size_t)jb * r + 2 * jb + 32) * sizeof(float);
      O3G_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)k_panel_lu, dim3(g), dim3(kPanelThreads), args, sm, st));
      note_launch();
      // interchanges inside the outer panel; the other columns get them once per outer panel
      laswp(k0, k0 + jb, K0, K1, k0, k0 + jb);
      if (k0 + jb < K1) {
        trsm(k0, jb, k0 + jb, K1 - k0 - jb);
        O3G_TRY(gemm(n - k0 - jb, K1 - k0 - jb, jb, at(k0 + jb, k0), at(k0, k0 + jb), at(k0 + jb, k0 + jb)));
      }
    }
    laswp(K0, K1, 0, n, K0, K1);
    if (K1 < n) {
      // U12 = L11^-1 A12 for the KB x KB unit lower L11, block by block
      for (int k0 = K0; k0 < K1; k0 += kNb) {
        const int jb = std::min(kNb, K1 - k0);
        O3G_TRY(trsm_wide(k0, jb, K1, n - K1));
        if (k0 + jb < K1) O3G_TRY(gemm(K1 - k0 - jb, n - K1, jb, at(k0 + jb, k0), at(k0, K1), at(k0 + jb, K1)));
      }
      O3G_TRY(gemm(n - K1, n - K1, KB, at(K1, K0), at(K0, K1), at(K1, K1)));
    }
  }
  {
    const size_t dsm = (size_t)kNb * kNb * sizeof(float);
    O3G_CUDA_TRY(cudaFuncSetAttribute(k_diag_inverses, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dsm));
    k_diag_inverses<<<(n + kNb - 1) / kNb, 256, dsm, st>>>(h->LU, ld, n, h->dinv);
    note_launch();
  }
  tm.end(st);
  O3G_CUDA_TRY(cudaGetLastError());
  int fl[5] = {0, 0, 0, 0, 0};
  O3G_CUDA_TRY(cudaMemcpyAsync(fl, h->flags, 5 * sizeof(int), cudaMemcpyDeviceToHost, st));
  std::vector<int> piv(n);
  O3G_CUDA_TRY(cudaMemcpyAsync(piv.data(), h->piv, n * sizeof(int), cudaMemcpyDeviceToHost, st));
  O3G_CUDA_TRY(cudaStreamSynchronize(st));
  if (fl[0]) {
    set_error("o3g_bem_factor: a grid barrier timed out");
    return O3G_ERR_TIMEOUT;
  }
  if (fl[4]) {
    set_error("o3g_bem_factor: a wait of the tensor-core update timed out");
    return O3G_ERR_TIMEOUT;
  }
  // compose the interchanges into one gather permutation
  std::vector<int> perm(n);
  for (int i = 0; i < n; ++i) perm[i] = i;
  for (int i = 0; i < n; ++i) {
    const int p = piv[i];
    if (p < 0 || p >= n) {
      set_error("o3g_bem_factor: pivot index out of range");
      return O3G_ERR_CUDA;
    }
    std::swap(perm[i], perm[p]);
  }
  O3G_CUDA_TRY(cudaMemcpyAsync(h->perm, perm.data(), n * sizeof(int), cudaMemcpyHostToDevice, st));
  O3G_CUDA_TRY(cudaStreamSynchronize(st));
  if (fl[1]) {
    char msg[128];
    std::snprintf(msg, sizeof(msg), "o3g_bem_factor: zero pivot in column %d", fl[1] - 1);
    set_error(msg);
    return O3G_ERR_SINGULAR;
  }
  h->factored = true;
  return O3G_OK;
}

extern "C" int32_t o3g_bem_solve(o3g_bem_t* h, const float* b, float* x, double* x64, int32_t mem, double tol,
                                 int32_t max_iter, int32_t* iters, double* relres, void* stream) {
  O3G_TRY(bem_check(h));
  if (!h->factored) {
    set_error("o3g_bem_solve: factor the matrix first (o3g_bem_factor)");
    return O3G_ERR_STATE;
  }
  if (!b || (mem != O3G_MEM_HOST && mem != O3G_MEM_DEVICE) || max_iter < 1 || !(tol >= 0.0)) {
    set_error("o3g_bem_solve: bad arguments");
    return O3G_ERR_INVALID_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const int n = h->n;
  const long long ld = h->ld;
  DeviceFacts df;
  O3G_TRY(device_facts(&df));
  const int ncb = (n + kMvChunk - 1) / kMvChunk;
  const int nrb = (n + 255) / 256;
  const size_t need = align_up((size_t)n * 8) * 3 + align_up((size_t)n * 4) * 5 + align_up((size_t)ncb * n * 8) +
                      align_up((size_t)nrb * 16);
  O3G_TRY(bem_scratch(h, need));
  Carve cv(h->scratch);
  double* bd = cv.take<double>(n);
  double* xd = cv.take<double>(n);
  double* rd = cv.take<double>(n);
  float* bf = cv.take<float>(n);
  float* y = cv.take<float>(n);
  float* xf = cv.take<float>(n);
  float* xh = cv.take<float>(n);
  float* xl = cv.take<float>(n);
  double* part = cv.take<double>((size_t)ncb * n);
  double* nrm = cv.take<double>(2 * (size_t)nrb);
  O3G_CUDA_TRY(cudaMemcpyAsync(bf, b, (size_t)n * 4, mem == O3G_MEM_HOST ? cudaMemcpyHostToDevice
                                                                           : cudaMemcpyDeviceToDevice, st));
  k_f2d<<<nrb, 256, 0, st>>>(bf, bd, n);
  O3G_CUDA_TRY(cudaMemsetAsync(xd, 0, (size_t)n * 8, st));
  O3G_CUDA_TRY(cudaMemcpyAsync(rd, bd, (size_t)n * 8, cudaMemcpyDeviceToDevice, st));
  O3G_CUDA_TRY(cudaMemsetAsync(h->flags, 0, 4 * sizeof(int), st));
  // cooperative solve kernels: one block per SM
  int G = df.num_sms;
  int per_sm = 0;
  const size_t dsm = 0;
  O3G_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trsv_lower, kSolveThreads, dsm));
  if (per_sm < 1) return O3G_ERR_CUDA;
  // L w = P r (y -> w; xh is free between the products), then U y = w (w -> y)
  TrsvArgs ta, tb;
  ta.LU = h->LU; ta.dinv = h->dinv; ta.ld = ld; ta.n = n; ta.y = y; ta.out = xh;
  ta.bar = make_barrier(h->flags);
  tb = ta;
  tb.y = xh; tb.out = y;
  void* targs[] = {&ta};
  void* tbargs[] = {&tb};
  std::vector<double> hn((size_t)nrb);
  double rel = 1.0, bnorm = 0.0;
  int it = 0;
  KernelTimer& tm = thread_timer();
  tm.begin(st);
  for (it = 0; it <= max_iter; ++it) {
    // r = b - A x in FP64-accurate double-single arithmetic (r = b at x = 0)
    if (it > 0) {
      k_split_f64<<<nrb, 256, 0, st>>>(xd, xh, xl, n);
      k_matvec_ds<<<dim3(nrb, ncb), 256, 0, st>>>(h->A, ld, n, xh, xl, part);
      note_launch(2);
    }
    k_matvec_finish<<<nrb, 256, 0, st>>>(part, it > 0 ? ncb : 0, n, bd, rd, nrm);
    note_launch();
    O3G_CUDA_TRY(cudaMemcpyAsync(hn.data(), nrm, (size_t)nrb * 8, cudaMemcpyDeviceToHost, st));
    O3G_CUDA_TRY(cudaStreamSynchronize(st));
    double rr = 0.0;
    for (int k = 0; k < nrb; ++k) rr += hn[k];
    if (it == 0) bnorm = std::sqrt(rr);
    rel = bnorm > 0.0 ? std::sqrt(rr) / bnorm : std::sqrt(rr);
    if (rel <= tol || it == max_iter) break;
    k_permute_to_float<<<nrb, 256, 0, st>>>(rd, h->perm, y, n);
    O3G_CUDA_TRY(zero_barrier(h->flags, st));
    O3G_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)k_trsv_lower, dim3(G), dim3(kSolveThreads), targs, dsm, st));
    O3G_CUDA_TRY(zero_barrier(h->flags, st));
    O3G_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)k_trsv_upper, dim3(G), dim3(kSolveThreads), tbargs, dsm, st));
    k_axpy_f2d<<<nrb, 256, 0, st>>>(xd, y, n);
    note_launch(4);
  }
  tm.end(st);
  int fl = 0;
  O3G_CUDA_TRY(cudaMemcpyAsync(&fl, h->flags, sizeof(int), cudaMemcpyDeviceToHost, st));
  k_d2f<<<nrb, 256, 0, st>>>(xd, xf, n);
  note_launch();
  if (x)
    O3G_CUDA_TRY(cudaMemcpyAsync(x, xf, (size_t)n * 4, mem == O3G_MEM_HOST ? cudaMemcpyDeviceToHost
                                                                            : cudaMemcpyDeviceToDevice, st));
  if (x64)
    O3G_CUDA_TRY(cudaMemcpyAsync(x64, xd, (size_t)n * 8, mem == O3G_MEM_HOST ? cudaMemcpyDeviceToHost
                                                                              : cudaMemcpyDeviceToDevice, st));
  O3G_CUDA_TRY(cudaStreamSynchronize(st));
  if (iters) *iters = it;
  if (relres) *relres = rel;
  if (fl) {
    set_error("o3g_bem_solve: a grid barrier timed out");
    return O3G_ERR_TIMEOUT;
  }
  if (!(rel <= tol)) {
    char msg[160];
    std::snprintf(msg, sizeof(msg), "o3g_bem_solve: relative residual %.3e after %d refinements (tol %.1e)", rel, it,
                  tol);
    set_error(msg);
    return O3G_ERR_NOT_CONVERGED;
  }
  return O3G_OK;
}

// ---- the Krylov bases' FP64 operations (Gram-Schmidt, norms, updates), sums in a fixed order
namespace o3g {
constexpr int kKrylovRows = 4096;   // rows per block of the reductions

// part[b kc + j] = sum over the rows [b R, b R + R) of V[j n + i] w[i], j < kc
__global__ void __launch_bounds__(256) k_kry_dots(const double* __restrict__ V, int n, int kc,
                                                  const double* __restrict__ w, double* __restrict__ part) {
  __shared__ double red[8];
  const int r0 = blockIdx.x * kKrylovRows, r1 = min(n, r0 + kKrylovRows);
  for (int j = 0; j < kc; ++j) {
    double s = 0.0;
    for (int i = r0 + threadIdx.x; i < r1; i += blockDim.x) s = fma(V[(size_t)j * n + i], w[i], s);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double a = 0.0;
      for (int q = 0; q < (int)(blockDim.x >> 5); ++q) a += red[q];
      part[(size_t)blockIdx.x * kc + j] = a;
    }
    __syncthreads();
  }
}

// h[j] = sum over the nb blocks, in block order, of part[b kc + j]
__global__ void k_kry_sum(const double* __restrict__ part, int nb, int kc, double* __restrict__ h) {
  for (int j = threadIdx.x; j < kc; j += blockDim.x) {
    double a = 0.0;
    for (int b = 0; b < nb; ++b) a += part[(size_t)b * kc + j];
    h[j] = a;
  }
}

// y[i] += alpha sum_j V[j n + i] h[j], kc <= 512
__global__ void __launch_bounds__(256) k_kry_update(const double* __restrict__ V, int n, int kc,
                                                    const double* __restrict__ h, double alpha, double* y) {
  __shared__ double hs[512];
  for (int j = threadIdx.x; j < kc; j += blockDim.x) hs[j] = h[j];
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int j = 0; j < kc; ++j) s = fma(V[(size_t)j * n + i], hs[j], s);
  y[i] = fma(alpha, s, y[i]);
}

__global__ void k_kry_scale(double* w, int n, double s) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) w[i] *= s;
}

// Block-Jacobi preconditioner of GMRES: the inverses (FP64) of the BS x BS diagonal blocks
// of A, one per panel (the panel's self-influence, Coefficients.h:414-436, when the blocks
// are surfaces on themselves).  A block that is singular or not finite gets the identity.
// Minv[p] is row-major.  BS is a template argument so the blocks stay in registers.
template <int BS>
__global__ void k_block_inv(const float* __restrict__ A, long long ld, int nb, double* __restrict__ Minv) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nb) return;
  double a[3][3] = {{1.0, 0.0, 0.0}, {0.0, 1.0, 0.0}, {0.0, 0.0, 1.0}};
  const size_t o = (size_t)p * BS;
#pragma unroll
  for (int r = 0; r < BS; ++r)
#pragma unroll
    for (int c = 0; c < BS; ++c) a[r][c] = (double)A[(o + c) * ld + o + r];
  double inv[3][3] = {{1.0, 0.0, 0.0}, {0.0, 1.0, 0.0}, {0.0, 0.0, 1.0}};
  // cofactors of the 3 x 3 (a 2 x 2 block sits in the leading corner of an identity, so
  // the same formula serves)
  const double c00 = a[1][1] * a[2][2] - a[1][2] * a[2][1];
  const double c01 = a[1][2] * a[2][0] - a[1][0] * a[2][2];
  const double c02 = a[1][0] * a[2][1] - a[1][1] * a[2][0];
  const double det = a[0][0] * c00 + a[0][1] * c01 + a[0][2] * c02;
  if (det != 0.0 && isfinite(det)) {
    const double id = 1.0 / det;
    inv[0][0] = c00 * id;
    inv[1][0] = c01 * id;
    inv[2][0] = c02 * id;
    inv[0][1] = (a[0][2] * a[2][1] - a[0][1] * a[2][2]) * id;
    inv[1][1] = (a[0][0] * a[2][2] - a[0][2] * a[2][0]) * id;
    inv[2][1] = (a[0][1] * a[2][0] - a[0][0] * a[2][1]) * id;
    inv[0][2] = (a[0][1] * a[1][2] - a[0][2] * a[1][1]) * id;
    inv[1][2] = (a[0][2] * a[1][0] - a[0][0] * a[1][2]) * id;
    inv[2][2] = (a[0][0] * a[1][1] - a[0][1] * a[1][0]) * id;
  }
#pragma unroll
  for (int r = 0; r < BS; ++r)
#pragma unroll
    for (int c = 0; c < BS; ++c) Minv[(size_t)p * BS * BS + r * BS + c] = inv[r][c];
}
// out = M^-1 in (acc = 0) or out += M^-1 in (acc = 1)
template <int BS>
__global__ void k_block_apply(const double* __restrict__ Minv, int nb, const double* __restrict__ in,
                              double* __restrict__ out, int acc) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nb) return;
  const double* x = in + (size_t)p * BS;
  double* y = out + (size_t)p * BS;
  const double* M = Minv + (size_t)p * BS * BS;
  double v[BS];
#pragma unroll
  for (int c = 0; c < BS; ++c) v[c] = x[c];
#pragma unroll
  for (int r = 0; r < BS; ++r) {
    double t = 0.0;
#pragma unroll
    for (int c = 0; c < BS; ++c) t += M[r * BS + c] * v[c];
    y[r] = acc ? y[r] + t : t;
  }
}
// launches for the unknowns per panel (2 or 3)
static void block_inv(const float* A, long long ld, int nb, int bs, double* Minv, cudaStream_t st) {
  const int g = (nb + 255) / 256;
  if (bs == 2) k_block_inv<2><<<g, 256, 0, st>>>(A, ld, nb, Minv);
  else         k_block_inv<3><<<g, 256, 0, st>>>(A, ld, nb, Minv);
  note_launch();
}
static void block_apply(const double* Minv, int nb, int bs, const double* in, double* out, int acc,
                        cudaStream_t st) {
  const int g = (nb + 255) / 256;
  if (bs == 2) k_block_apply<2><<<g, 256, 0, st>>>(Minv, nb, in, out, acc);
  else         k_block_apply<3><<<g, 256, 0, st>>>(Minv, nb, in, out, acc);
  note_launch();
}

namespace {
// one classical Gram-Schmidt pass: hp = V^T w (kc columns), w -= V hp
void gs_pass(const double* V, int n, int kc, double* w, double* hp, double* part, cudaStream_t st) {
  const int nb = (n + kKrylovRows - 1) / kKrylovRows;
  k_kry_dots<<<nb, 256, 0, st>>>(V, n, kc, w, part);
  k_kry_sum<<<1, 256, 0, st>>>(part, nb, kc, hp);
  k_kry_update<<<(n + 255) / 256, 256, 0, st>>>(V, n, kc, hp, -1.0, w);
  note_launch(3);
}
// per-block partial sums of w^2 into part (nb of them), summed on the host in order
void norm_partials(const double* w, int n, double* part, cudaStream_t st) {
  k_kry_dots<<<(n + kKrylovRows - 1) / kKrylovRows, 256, 0, st>>>(w, n, 1, w, part);
  note_launch();
}
double host_sum(const std::vector<double>& v) {
  double a = 0.0;
  for (double x : v) a += x;
  return a;
}
}  // namespace
}  // namespace o3g

// ---- GMRES: the reference's solver (Eigen GMRES, BEM.h:182-202) ----------------------------
// Restarted GMRES(m) on the unfactored FP32 matrix: FP64 Krylov vectors, classical
// Gram-Schmidt with one reorthogonalisation (k_kry_dots / k_kry_update on the n x (k+1)
// basis, sums in a fixed order), Givens
// rotations of the small Hessenberg matrix on the host, FP64-accurate matrix products
// (k_matvec_ds).  The true residual ||b - A x|| / ||b|| (BEM.h:227-230) is recomputed at
// every restart and decides convergence.  The vortex-sheet rows of the matrix have a zero
// diagonal (Coefficients.h:414-436), where a Jacobi preconditioner is the identity; with the
// unknowns per panel set (o3g_bem_set_unknowns_per_panel) GMRES is right-preconditioned by
// the inverses of the panels' diagonal blocks (A M^-1 u = b, x = M^-1 u), which keeps the
// residual the system's own.
extern "C" int32_t o3g_bem_solve_gmres(o3g_bem_t* h, const float* b, float* x, double* x64, int32_t mem, double tol,
                                       int32_t max_iter, int32_t restart, int32_t* iters, double* relres,
                                       void* stream) {
  O3G_TRY(bem_check(h));
  if (!b || (mem != O3G_MEM_HOST && mem != O3G_MEM_DEVICE) || max_iter < 1 || restart < 1 || restart > 500 ||
      !(tol >= 0.0)) {
    set_error("o3g_bem_solve_gmres: bad arguments (max_iter >= 1, restart 1..500, tol >= 0)");
    return O3G_ERR_INVALID_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  const int n = h->n;
  const long long ld = h->ld;
  const int m = std::min(restart, max_iter);
  const int ncb = (n + kMvChunk - 1) / kMvChunk;
  const int nrb = (n + 255) / 256;
  const int nkb = (n + kKrylovRows - 1) / kKrylovRows;
  const int bs = h->bs, npb = n / bs;
  const bool pre = bs > 1;
  const size_t need = align_up((size_t)(m + 1) * n * 8) + 2 * align_up((size_t)n * 8) + 4 * align_up((size_t)n * 4) +
                      align_up((size_t)ncb * n * 8) + align_up((size_t)nrb * 8) + align_up((size_t)2 * (m + 1) * 8) +
                      2 * align_up((size_t)nkb * (m + 1) * 8) + align_up((size_t)n * bs * 8) + align_up((size_t)n * 8);
  O3G_TRY(bem_scratch(h, need));
  Carve cv(h->scratch);
  double* V = cv.take<double>((size_t)(m + 1) * n);
  double* bd = cv.take<double>(n);
  double* xd = cv.take<double>(n);
  double* Minv = cv.take<double>((size_t)n * bs);   // the diagonal blocks' inverses (pre)
  double* zd = cv.take<double>(n);                  // M^-1 v, and V y before M^-1 (pre)
  if (pre) block_inv(h->A, ld, npb, bs, Minv, st);
  float* bf = cv.take<float>(n);
  float* xf = cv.take<float>(n);
  float* xh = cv.take<float>(n);
  float* xl = cv.take<float>(n);
  double* part = cv.take<double>((size_t)ncb * n);
  double* nrm = cv.take<double>(nrb);
  double* hd = cv.take<double>(2 * (size_t)(m + 1));
  double* kpart = cv.take<double>((size_t)nkb * (m + 1));
  double* npart = cv.take<double>((size_t)nkb * (m + 1));
  std::vector<double> hnp((size_t)nkb);
  O3G_CUDA_TRY(cudaMemcpyAsync(bf, b, (size_t)n * 4, mem == O3G_MEM_HOST ? cudaMemcpyHostToDevice
                                                                           : cudaMemcpyDeviceToDevice, st));
  k_f2d<<<nrb, 256, 0, st>>>(bf, bd, n);
  note_launch();
  O3G_CUDA_TRY(cudaMemsetAsync(xd, 0, (size_t)n * 8, st));
  std::vector<double> hn((size_t)nrb);
  // y = b - A xin (bin given) or y = A xin; the squared norm of y when asked (synchronises)
  auto matvec = [&](const double* xin, const double* bin, double* yout, double* norm2) -> int32_t {
    int nc = 0;
    if (xin) {
      k_split_f64<<<nrb, 256, 0, st>>>(xin, xh, xl, n);
      k_matvec_ds<<<dim3(nrb, ncb), 256, 0, st>>>(h->A, ld, n, xh, xl, part);
      note_launch(2);
      nc = ncb;
    }
    k_matvec_finish<<<nrb, 256, 0, st>>>(part, nc, n, bin, yout, nrm);
    note_launch();
    O3G_CUDA_TRY(cudaGetLastError());
    if (norm2) {
      O3G_CUDA_TRY(cudaMemcpyAsync(hn.data(), nrm, (size_t)nrb * 8, cudaMemcpyDeviceToHost, st));
      O3G_CUDA_TRY(cudaStreamSynchronize(st));
      double s2 = 0.0;
      for (int k = 0; k < nrb; ++k) s2 += hn[k];
      *norm2 = s2;
    }
    return O3G_OK;
  };
  double bb = 0.0;
  O3G_TRY(matvec(nullptr, bd, V, &bb));           // V0 = b, ||b||^2
  const double bnorm = std::sqrt(bb);
  int total = 0;
  double rel = 0.0;
  KernelTimer& tm = thread_timer();
  tm.begin(st);
  if (bnorm > 0.0) {
    std::vector<double> H((size_t)(m + 1) * m, 0.0), cs(m), sn(m), g(m + 1), y(m), hc(2 * (size_t)(m + 1));
    auto Hat = [&](int i, int k) -> double& { return H[(size_t)k * (m + 1) + i]; };
    for (;;) {
      double rr = 0.0;
      O3G_TRY(matvec(total > 0 ? xd : nullptr, bd, V, &rr));   // V0 = r = b - A x
      rel = std::sqrt(rr) / bnorm;
      if (rel <= tol || total >= max_iter) break;
      const double beta = std::sqrt(rr);
      k_kry_scale<<<nrb, 256, 0, st>>>(V, n, 1.0 / beta);
      note_launch();
      std::fill(g.begin(), g.end(), 0.0);
      g[0] = beta;
      int k = 0;
      for (; k < m && total < max_iter;) {
        double* vk = V + (size_t)k * n;
        double* w = V + (size_t)(k + 1) * n;
        if (pre) {
          // right preconditioning: w = A M^-1 v_k, so the residual stays the system's own
          block_apply(Minv, npb, bs, vk, zd, 0, st);
          O3G_TRY(matvec(zd, nullptr, w, nullptr));
        } else {
          O3G_TRY(matvec(vk, nullptr, w, nullptr));
        }
        // classical Gram-Schmidt, twice
        for (int pass = 0; pass < 2; ++pass) gs_pass(V, n, k + 1, w, hd + (size_t)pass * (m + 1), kpart, st);
        norm_partials(w, n, npart, st);
        O3G_CUDA_TRY(cudaMemcpyAsync(hc.data(), hd, 2 * (size_t)(m + 1) * 8, cudaMemcpyDeviceToHost, st));
        O3G_CUDA_TRY(cudaMemcpyAsync(hnp.data(), npart, (size_t)nkb * 8, cudaMemcpyDeviceToHost, st));
        O3G_CUDA_TRY(cudaStreamSynchronize(st));
        const double wn = std::sqrt(host_sum(hnp));
        for (int i = 0; i <= k; ++i) Hat(i, k) = hc[i] + hc[(size_t)(m + 1) + i];
        Hat(k + 1, k) = wn;
        if (wn > 0.0) {
          k_kry_scale<<<nrb, 256, 0, st>>>(w, n, 1.0 / wn);
          note_launch();
        }
        // previous rotations, then a new one that zeroes H(k+1, k)
        for (int i = 0; i < k; ++i) {
          const double a = Hat(i, k), c = Hat(i + 1, k);
          Hat(i, k) = cs[i] * a + sn[i] * c;
          Hat(i + 1, k) = -sn[i] * a + cs[i] * c;
        }
        const double dd = std::hypot(Hat(k, k), Hat(k + 1, k));
        cs[k] = dd > 0.0 ? Hat(k, k) / dd : 1.0;
        sn[k] = dd > 0.0 ? Hat(k + 1, k) / dd : 0.0;
        Hat(k, k) = dd;
        Hat(k + 1, k) = 0.0;
        g[k + 1] = -sn[k] * g[k];
        g[k] = cs[k] * g[k];
        ++k;
        ++total;
        if (std::fabs(g[k]) <= 0.5 * tol * bnorm || wn == 0.0) break;
      }
      // x += V y with H(0:k, 0:k) y = g(0:k)
      for (int i = k - 1; i >= 0; --i) {
        double sacc = g[i];
        for (int j = i + 1; j < k; ++j) sacc -= Hat(i, j) * y[j];
        y[i] = Hat(i, i) != 0.0 ? sacc / Hat(i, i) : 0.0;
      }
      O3G_CUDA_TRY(cudaMemcpyAsync(hd, y.data(), (size_t)k * 8, cudaMemcpyHostToDevice, st));
      if (pre) {
        // x += M^-1 (V y)
        O3G_CUDA_TRY(cudaMemsetAsync(zd, 0, (size_t)n * 8, st));
        k_kry_update<<<nrb, 256, 0, st>>>(V, n, k, hd, 1.0, zd);
        note_launch();
        block_apply(Minv, npb, bs, zd, xd, 1, st);
      } else {
        k_kry_update<<<nrb, 256, 0, st>>>(V, n, k, hd, 1.0, xd);
        note_launch();
      }
    }
  }
  tm.end(st);
  k_d2f<<<nrb, 256, 0, st>>>(xd, xf, n);
  note_launch();
  if (x)
    O3G_CUDA_TRY(cudaMemcpyAsync(x, xf, (size_t)n * 4, mem == O3G_MEM_HOST ? cudaMemcpyDeviceToHost
                                                                            : cudaMemcpyDeviceToDevice, st));
  if (x64)
    O3G_CUDA_TRY(cudaMemcpyAsync(x64, xd, (size_t)n * 8, mem == O3G_MEM_HOST ? cudaMemcpyDeviceToHost
                                                                              : cudaMemcpyDeviceToDevice, st));
  O3G_CUDA_TRY(cudaStreamSynchronize(st));
  if (iters) *iters = total;
  if (relres) *relres = rel;
  if (!(rel <= tol)) {
    char msg[160];
    std::snprintf(msg, sizeof(msg), "o3g_bem_solve_gmres: relative residual %.3e after %d iterations (tol %.1e)", rel,
                  total, tol);
    set_error(msg);
    return O3G_ERR_NOT_CONVERGED;
  }
  return O3G_OK;
}

// =====================================================================================
// Several right-hand sides per pass over the matrix.  Each refinement sweep and each
// GMRES iteration of one right-hand side streams the n^2 FP32 matrix once (6.7 GB at
// n = 40,960): the products, the triangular solves and the Krylov steps below serve up to
// kMaxRhs right-hand sides with that one pass.  BEM::solve takes one b (BEM.h:200-203); the
// reference solves again per RK stage (Convection.h:197) and per diffusion step
// (Diffusion.h:184-187), and these entry points let a caller hand all of them over at once.
namespace o3g {

constexpr int kMaxRhs = 8;
constexpr int kMvChunkM = 512;   // columns per block of the multi-vector product

struct DIn { const double* p[kMaxRhs]; };
struct DOut { double* p[kMaxRhs]; };

// xh/xl[c][.] = the float split of src.p[c] (K vectors of n)
__global__ void k_split_f64_multi(DIn src, float* xh, float* xl, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
  if (i >= n) return;
  const double v = src.p[c][i];
  const float h = (float)v;
  xh[(size_t)c * n + i] = h;
  xl[(size_t)c * n + i] = (float)(v - (double)h);
}

// part[cb][c][i] = sum over the columns of chunk cb of A[i, j] x_c[j], double-single as in
// k_matvec_ds: every matrix element is loaded once for the K vectors.  With K vectors the
// sums cost K times the FP32 instructions of one, so they run in packed FP32 (FFMA2,
// FADD2, FMUL2; each lane rounds like the scalar instruction): columns j and j + 1 of the
// chunk ride in the two lanes, each lane carrying its own double-single sum, added in
// double at the end.  Differences are formed as fused multiply-adds with -1 (exact
// negation), so the two-sum needs no negated operands: shared memory holds x_h, -x_h and
// x_l of each column pair.
__device__ __forceinline__ void ds_add_product2(float2 a, float2 h, float2 hn, float2 l, float2& hi, float2& lo) {
  const float2 m1 = make_float2(-1.f, -1.f);
  const float2 pn = __fmul2_rn(a, hn);                      // -p, p = a h rounded
  const float2 e = __ffma2_rn(a, h, pn);                    // a h - p, exact
  const float2 sum = __ffma2_rn(pn, m1, hi);                // hi + p
  const float2 bb = __ffma2_rn(hi, m1, sum);                // sum - hi
  const float2 t2 = __ffma2_rn(__ffma2_rn(bb, m1, sum), m1, hi);   // hi - (sum - bb)
  const float2 t = __ffma2_rn(__fadd2_rn(pn, bb), m1, t2);  // t2 + (p - bb)
  hi = sum;
  lo = __ffma2_rn(a, l, __fadd2_rn(lo, __fadd2_rn(t, e)));
}

template <int K>
__global__ void __launch_bounds__(256) k_matvec_ds_multi(const float* __restrict__ A, long long ld, int n,
                                                         const float* __restrict__ xh, const float* __restrict__ xl,
                                                         double* __restrict__ part) {
  constexpr int M2 = kMvChunkM / 2;
  __shared__ float2 sh[K][M2], shn[K][M2], sl[K][M2];   // column pairs (x_h, -x_h, x_l)
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int cb = blockIdx.y;
  const int j0 = cb * kMvChunkM, m = min(n - j0, kMvChunkM);
#pragma unroll
  for (int c = 0; c < K; ++c)
    for (int k = threadIdx.x; k < M2; k += blockDim.x) {
      // a column beyond the chunk gets x = 0 (and its matrix element 0 below)
      const float h0 = 2 * k < m ? xh[(size_t)c * n + j0 + 2 * k] : 0.f;
      const float h1 = 2 * k + 1 < m ? xh[(size_t)c * n + j0 + 2 * k + 1] : 0.f;
      const float l0 = 2 * k < m ? xl[(size_t)c * n + j0 + 2 * k] : 0.f;
      const float l1 = 2 * k + 1 < m ? xl[(size_t)c * n + j0 + 2 * k + 1] : 0.f;
      sh[c][k] = make_float2(h0, h1);
      shn[c][k] = make_float2(-h0, -h1);
      sl[c][k] = make_float2(l0, l1);
    }
  __syncthreads();
  if (i >= n) return;
  const float* a = A + (size_t)j0 * ld + i;
  float2 hi[K], lo[K];
#pragma unroll
  for (int c = 0; c < K; ++c) { hi[c] = make_float2(0.f, 0.f); lo[c] = make_float2(0.f, 0.f); }
  const float2 m1 = make_float2(-1.f, -1.f);
  int k = 0;
  for (; k + 8 <= m; k += 8) {
    float2 av[4];
#pragma unroll
    for (int q = 0; q < 4; ++q)
      av[q] = make_float2(__ldg(a + (size_t)(k + 2 * q) * ld), __ldg(a + (size_t)(k + 2 * q + 1) * ld));
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
      for (int c = 0; c < K; ++c)
        ds_add_product2(av[q], sh[c][k / 2 + q], shn[c][k / 2 + q], sl[c][k / 2 + q], hi[c], lo[c]);
    // renormalise: move the bulk of lo into hi (Dekker's fast two-sum, |hi| >= |lo|)
#pragma unroll
    for (int c = 0; c < K; ++c) {
      const float2 s2 = __fadd2_rn(hi[c], lo[c]);
      lo[c] = __ffma2_rn(__ffma2_rn(hi[c], m1, s2), m1, lo[c]);
      hi[c] = s2;
    }
  }
  for (; k < m; k += 2) {   // the chunk's last columns (m is even except at the matrix edge)
    const float2 av = make_float2(__ldg(a + (size_t)k * ld), k + 1 < m ? __ldg(a + (size_t)(k + 1) * ld) : 0.f);
#pragma unroll
    for (int c = 0; c < K; ++c) ds_add_product2(av, sh[c][k / 2], shn[c][k / 2], sl[c][k / 2], hi[c], lo[c]);
  }
#pragma unroll
  for (int c = 0; c < K; ++c)
    part[((size_t)cb * K + c) * n + i] = ((double)hi[c].x + (double)lo[c].x) + ((double)hi[c].y + (double)lo[c].y);
}

// y_c = b_c - sum_cb part (b given) or y_c = sum_cb part, c = blockIdx.y < K; per-block sums
// of y_c^2 into nrm[c][blockIdx.x]
__global__ void k_matvec_finish_multi(const double* __restrict__ part, int ncb, int K, int n, DIn b, DOut y,
                                      double* __restrict__ nrm) {
  __shared__ double s1[8];
  const int i = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
  double yy = 0.0;
  if (i < n) {
    double s = 0.0;
    for (int k = 0; k < ncb; ++k) s += part[((size_t)k * K + c) * n + i];
    const double v = b.p[c] ? b.p[c][i] - s : s;
    y.p[c][i] = v;
    yy = v * v;
  }
  for (int o = 16; o > 0; o >>= 1) yy += __shfl_xor_sync(0xffffffffu, yy, o);
  if ((threadIdx.x & 31) == 0) s1[threadIdx.x >> 5] = yy;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a1 = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) a1 += s1[w];
    nrm[(size_t)c * gridDim.x + blockIdx.x] = a1;
  }
}

// y[c][i] = r[c][perm[i]] for the columns in `mask`, 0 for the others (no correction)
__global__ void k_permute_to_float_multi(const double* r, const int* perm, float* y, int n, unsigned mask) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
  if (i < n) y[(size_t)c * n + i] = ((mask >> c) & 1u) ? (float)r[(size_t)c * n + perm[i]] : 0.f;
}

template <int K>
__device__ __forceinline__ void diag_apply_multi(const float* __restrict__ Dinv, const float* y, int n, int jb,
                                                 float (*yin)[kNb], float* part, float (*yd)[kNb]) {
  for (int e = threadIdx.x; e < K * jb; e += blockDim.x) yin[e / jb][e % jb] = y[(size_t)(e / jb) * n + e % jb];
  __syncthreads();
  constexpr int kQ = kSolveThreads / kNb;
  const int m = threadIdx.x % kNb, q = threadIdx.x / kNb;
  float s[K];
#pragma unroll
  for (int c = 0; c < K; ++c) s[c] = 0.f;
  if (m < jb) {
    for (int k = q * (kNb / kQ); k < (q + 1) * (kNb / kQ); ++k)
      if (k < jb) {
        const float d = __ldg(Dinv + (size_t)k * kNb + m);
#pragma unroll
        for (int c = 0; c < K; ++c) s[c] = fmaf(d, yin[c][k], s[c]);
      }
  }
#pragma unroll
  for (int c = 0; c < K; ++c) part[(c * kQ + q) * kNb + m] = s[c];
  __syncthreads();
  for (int e = threadIdx.x; e < K * jb; e += blockDim.x) {
    const int c = e / jb, tt = e % jb;
    float v = 0.f;
#pragma unroll
    for (int qq = 0; qq < kQ; ++qq) v += part[(c * kQ + qq) * kNb + tt];
    yd[c][tt] = v;
  }
  __syncthreads();
}

template <int K>
__device__ __forceinline__ void update_rows_multi(const float* __restrict__ LU, long long ld, int n, int k0, int jb,
                                                  int i0, int i1, float (*yd)[kNb], float* y, float* part) {
  const int nr = i1 - i0;
  if (nr <= 0) return;
  if (jb != kNb) {
    for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
      float s[K];
#pragma unroll
      for (int c = 0; c < K; ++c) s[c] = 0.f;
      for (int m = 0; m < jb; ++m) {
        const float a = LU[(size_t)(k0 + m) * ld + i];
#pragma unroll
        for (int c = 0; c < K; ++c) s[c] = fmaf(a, yd[c][m], s[c]);
      }
#pragma unroll
      for (int c = 0; c < K; ++c) y[(size_t)c * n + i] -= s[c];
    }
    return;
  }
  constexpr int kChunks = 4, kW = kNb / kChunks, kRows = kSolveThreads / kChunks;
  for (int r0 = 0; r0 < nr; r0 += kRows) {
    const int rows = min(kRows, nr - r0);
    const int q = threadIdx.x / kRows, r = threadIdx.x % kRows;
    if (r < rows) {
      const float* col = LU + (size_t)(k0 + q * kW) * ld + i0 + r0 + r;
      float s[K];
#pragma unroll
      for (int c = 0; c < K; ++c) s[c] = 0.f;
#pragma unroll 8
      for (int m = 0; m < kW; ++m) {
        const float a = __ldg(col + (size_t)m * ld);
#pragma unroll
        for (int c = 0; c < K; ++c) s[c] = fmaf(a, yd[c][q * kW + m], s[c]);
      }
#pragma unroll
      for (int c = 0; c < K; ++c) part[(c * kChunks + q) * kRows + r] = s[c];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < K * rows; e += blockDim.x) {
      const int c = e / rows, rr = e % rows;
      float v = 0.f;
#pragma unroll
      for (int qq = 0; qq < kChunks; ++qq) v += part[(c * kChunks + qq) * kRows + rr];
      y[(size_t)c * n + i0 + r0 + rr] -= v;
    }
    __syncthreads();
  }
}

// L w = y and U x = w for K right-hand sides (y, out: K vectors of n, column c at c n)
template <int K>
__global__ void __launch_bounds__(kSolveThreads) k_trsv_lower_multi(TrsvArgs a) {
  __shared__ float yd[K][kNb], yin[K][kNb];
  __shared__ float part[K * kSolveThreads];
  const int G = gridDim.x;
  for (int k0 = 0; k0 < a.n; k0 += kNb) {
    const int jb = min(kNb, a.n - k0);
    diag_apply_multi<K>(a.dinv + (size_t)(k0 / kNb) * 2 * kNb * kNb, a.y + k0, a.n, jb, yin, part, yd);
    const int rest = a.n - k0 - jb;
    const int chunk = (rest + G - 1) / G;
    const int i0 = k0 + jb + blockIdx.x * chunk, i1 = min(a.n, i0 + chunk);
    update_rows_multi<K>(a.LU, a.ld, a.n, k0, jb, i0, i1, yd, a.y, part);
    if (blockIdx.x == 0)
      for (int e = threadIdx.x; e < K * jb; e += blockDim.x) a.out[(size_t)(e / jb) * a.n + k0 + e % jb] = yd[e / jb][e % jb];
    if (!grid_sync(a.bar)) return;
  }
}

template <int K>
__global__ void __launch_bounds__(kSolveThreads) k_trsv_upper_multi(TrsvArgs a) {
  __shared__ float yd[K][kNb], yin[K][kNb];
  __shared__ float part[K * kSolveThreads];
  const int G = gridDim.x;
  const int nblk = (a.n + kNb - 1) / kNb;
  for (int kb = nblk - 1; kb >= 0; --kb) {
    const int k0 = kb * kNb, jb = min(kNb, a.n - k0);
    diag_apply_multi<K>(a.dinv + (size_t)kb * 2 * kNb * kNb + (size_t)kNb * kNb, a.y + k0, a.n, jb, yin, part, yd);
    const int chunk = (k0 + G - 1) / G;
    const int i0 = blockIdx.x * chunk, i1 = min(k0, i0 + chunk);
    update_rows_multi<K>(a.LU, a.ld, a.n, k0, jb, i0, i1, yd, a.y, part);
    if (blockIdx.x == 0)
      for (int e = threadIdx.x; e < K * jb; e += blockDim.x) a.out[(size_t)(e / jb) * a.n + k0 + e % jb] = yd[e / jb][e % jb];
    if (!grid_sync(a.bar)) return;
  }
}

// the products b_c - A x_c (b given) or A x_c for K vectors in one pass over A, with the
// squared norms of the results on the host (synchronises) when norm2 is given
static int32_t matvec_multi(o3g_bem_t* h, int K, const DIn& x, const DIn& b, const DOut& y, float* xh, float* xl,
                            double* part, double* nrm, std::vector<double>* norm2, cudaStream_t st) {
  const int n = h->n;
  const int nrb = (n + 255) / 256;
  const int ncb = (n + kMvChunkM - 1) / kMvChunkM;
  int nc = 0;
  if (x.p[0] && K == 1) {
    // one vector: the single-vector product (HBM-bound already, 1024-column chunks)
    k_split_f64_multi<<<dim3(nrb, 1), 256, 0, st>>>(x, xh, xl, n);
    const int ncb1 = (n + kMvChunk - 1) / kMvChunk;
    k_matvec_ds<<<dim3(nrb, ncb1), 256, 0, st>>>(h->A, h->ld, n, xh, xl, part);
    note_launch(2);
    nc = ncb1;
  } else if (x.p[0]) {
    k_split_f64_multi<<<dim3(nrb, K), 256, 0, st>>>(x, xh, xl, n);
    const dim3 g(nrb, ncb);
    switch (K) {
      case 2: k_matvec_ds_multi<2><<<g, 256, 0, st>>>(h->A, h->ld, n, xh, xl, part); break;
      case 3: k_matvec_ds_multi<3><<<g, 256, 0, st>>>(h->A, h->ld, n, xh, xl, part); break;
      case 4: k_matvec_ds_multi<4><<<g, 256, 0, st>>>(h->A, h->ld, n, xh, xl, part); break;
      case 5: k_matvec_ds_multi<5><<<g, 256, 0, st>>>(h->A, h->ld, n, xh, xl, part); break;
      case 6: k_matvec_ds_multi<6><<<g, 256, 0, st>>>(h->A, h->ld, n, xh, xl, part); break;
      case 7: k_matvec_ds_multi<7><<<g, 256, 0, st>>>(h->A, h->ld, n, xh, xl, part); break;
      default: k_matvec_ds_multi<8><<<g, 256, 0, st>>>(h->A, h->ld, n, xh, xl, part); break;
    }
    note_launch(2);
    nc = ncb;
  }
  k_matvec_finish_multi<<<dim3(nrb, K), 256, 0, st>>>(part, nc, K, n, b, y, nrm);
  note_launch();
  O3G_CUDA_TRY(cudaGetLastError());
  if (norm2) {
    std::vector<double> hn((size_t)K * nrb);
    O3G_CUDA_TRY(cudaMemcpyAsync(hn.data(), nrm, hn.size() * 8, cudaMemcpyDeviceToHost, st));
    O3G_CUDA_TRY(cudaStreamSynchronize(st));
    norm2->assign(K, 0.0);
    for (int c = 0; c < K; ++c)
      for (int k = 0; k < nrb; ++k) (*norm2)[c] += hn[(size_t)c * nrb + k];
  }
  return O3G_OK;
}

template <int K>
static int32_t launch_trsv_multi(const TrsvArgs& lower, const TrsvArgs& upper, int G, cudaStream_t st) {
  TrsvArgs a = lower, b = upper;
  void* aa[] = {&a};
  void* bb[] = {&b};
  int* flags = reinterpret_cast<int*>(a.bar.err);
  O3G_CUDA_TRY(zero_barrier(flags, st));
  O3G_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)k_trsv_lower_multi<K>, dim3(G), dim3(kSolveThreads), aa, 0,
                                           st));
  O3G_CUDA_TRY(zero_barrier(flags, st));
  O3G_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)k_trsv_upper_multi<K>, dim3(G), dim3(kSolveThreads), bb, 0,
                                           st));
  note_launch(2);
  return O3G_OK;
}

static int32_t trsv_multi(int K, const TrsvArgs& lower, const TrsvArgs& upper, int G, cudaStream_t st) {
  switch (K) {
    case 1: return launch_trsv_multi<1>(lower, upper, G, st);
    case 2: return launch_trsv_multi<2>(lower, upper, G, st);
    case 3: return launch_trsv_multi<3>(lower, upper, G, st);
    case 4: return launch_trsv_multi<4>(lower, upper, G, st);
    case 5: return launch_trsv_multi<5>(lower, upper, G, st);
    case 6: return launch_trsv_multi<6>(lower, upper, G, st);
    case 7: return launch_trsv_multi<7>(lower, upper, G, st);
    default: return launch_trsv_multi<8>(lower, upper, G, st);
  }
}

// blocks per SM of the K-vector solve kernels (their shared memory grows with K)
static int32_t trsv_multi_grid(int K, int num_sms, int* G) {
  int per_sm = 0;
  cudaError_t e;
  switch (K) {
    case 1: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trsv_lower_multi<1>, kSolveThreads, 0); break;
    case 2: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trsv_lower_multi<2>, kSolveThreads, 0); break;
    case 3: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trsv_lower_multi<3>, kSolveThreads, 0); break;
    case 4: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trsv_lower_multi<4>, kSolveThreads, 0); break;
    case 5: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trsv_lower_multi<5>, kSolveThreads, 0); break;
    case 6: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trsv_lower_multi<6>, kSolveThreads, 0); break;
    case 7: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trsv_lower_multi<7>, kSolveThreads, 0); break;
    default: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trsv_lower_multi<8>, kSolveThreads, 0); break;
  }
  O3G_CUDA_TRY(e);
  if (per_sm < 1) {
    set_error("o3g_bem_solve_many: the solve kernel does not fit on an SM");
    return O3G_ERR_CUDA;
  }
  *G = num_sms;   // one block per SM, as the single-vector solve
  return O3G_OK;
}

}  // namespace o3g

static int32_t many_args(o3g_bem_t* h, int32_t nrhs, const float* B, int32_t mem, double tol, int32_t max_iter,
                         const char* who) {
  O3G_TRY(bem_check(h));
  if (nrhs < 0 || (nrhs > 0 && !B) || (mem != O3G_MEM_HOST && mem != O3G_MEM_DEVICE) || max_iter < 1 ||
      !(tol >= 0.0)) {
    char msg[160];
    std::snprintf(msg, sizeof(msg), "%s: bad arguments (nrhs >= 0, B given, mem HOST or DEVICE, max_iter >= 1, tol >= 0)",
                  who);
    set_error(msg);
    return O3G_ERR_INVALID_ARG;
  }
  return O3G_OK;
}

extern "C" int32_t o3g_bem_solve_many(o3g_bem_t* h, int32_t nrhs, const float* B, float* X, double* X64, int32_t mem,
                                      double tol, int32_t max_iter, int32_t* iters, double* relres, void* stream) {
  O3G_TRY(many_args(h, nrhs, B, mem, tol, max_iter, "o3g_bem_solve_many"));
  if (!h->factored) {
    set_error("o3g_bem_solve_many: factor the matrix first (o3g_bem_factor)");
    return O3G_ERR_STATE;
  }
  if (nrhs == 0) return O3G_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const int n = h->n;
  const long long ld = h->ld;
  DeviceFacts df;
  O3G_TRY(device_facts(&df));
  const int KM = std::min(nrhs, kMaxRhs);
  const int ncb = (n + kMvChunkM - 1) / kMvChunkM;
  const int nrb = (n + 255) / 256;
  const size_t kn = (size_t)KM * n;
  const size_t need = 3 * align_up(kn * 8) + 5 * align_up(kn * 4) + align_up((size_t)ncb * kn * 8) +
                      align_up((size_t)KM * nrb * 8);
  O3G_TRY(bem_scratch(h, need));
  Carve cv(h->scratch);
  double* bd = cv.take<double>(kn);
  double* xd = cv.take<double>(kn);
  double* rd = cv.take<double>(kn);
  float* bf = cv.take<float>(kn);
  float* y = cv.take<float>(kn);
  float* w = cv.take<float>(kn);
  float* xh = cv.take<float>(kn);
  float* xl = cv.take<float>(kn);
  double* part = cv.take<double>((size_t)ncb * kn);
  double* nrm = cv.take<double>((size_t)KM * nrb);
  const cudaMemcpyKind h2d = mem == O3G_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  const cudaMemcpyKind d2h = mem == O3G_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  bool timed_out = false, all_converged = true;
  KernelTimer& tm = thread_timer();
  tm.begin(st);
  for (int g0 = 0; g0 < nrhs; g0 += kMaxRhs) {
    const int K = std::min(kMaxRhs, nrhs - g0);
    const size_t knn = (size_t)K * n;
    O3G_CUDA_TRY(cudaMemcpyAsync(bf, B + (size_t)g0 * n, knn * 4, h2d, st));
    k_f2d<<<(unsigned)((knn + 255) / 256), 256, 0, st>>>(bf, bd, (int)knn);
    note_launch();
    O3G_CUDA_TRY(cudaMemsetAsync(xd, 0, knn * 8, st));
    O3G_CUDA_TRY(cudaMemsetAsync(h->flags, 0, 4 * sizeof(int), st));
    DIn xin{}, bin{};
    DOut rout{};
    for (int c = 0; c < K; ++c) {
      xin.p[c] = xd + (size_t)c * n;
      bin.p[c] = bd + (size_t)c * n;
      rout.p[c] = rd + (size_t)c * n;
    }
    DIn none{};
    int G = 0;
    O3G_TRY(trsv_multi_grid(K, df.num_sms, &G));
    TrsvArgs lo, up;
    lo.LU = h->LU; lo.dinv = h->dinv; lo.ld = ld; lo.n = n; lo.y = y; lo.out = w;
    lo.bar = make_barrier(h->flags);
    up = lo;
    up.y = w; up.out = y;
    std::vector<double> rr, bnorm(K, 0.0), rel(K, 1.0);
    unsigned active = (1u << K) - 1u;
    std::vector<int> it_of(K, max_iter);
    for (int it = 0; it <= max_iter; ++it) {
      O3G_TRY(matvec_multi(h, K, it > 0 ? xin : none, bin, rout, xh, xl, part, nrm, &rr, st));
      for (int c = 0; c < K; ++c) {
        if (it == 0) bnorm[c] = std::sqrt(rr[c]);
        if (!((active >> c) & 1u)) continue;
        rel[c] = bnorm[c] > 0.0 ? std::sqrt(rr[c]) / bnorm[c] : std::sqrt(rr[c]);
        if (rel[c] <= tol || it == max_iter) {
          active &= ~(1u << c);
          it_of[c] = it;
        }
      }
      if (!active) break;
      k_permute_to_float_multi<<<dim3(nrb, K), 256, 0, st>>>(rd, h->perm, y, n, active);
      note_launch();
      O3G_TRY(trsv_multi(K, lo, up, G, st));
      k_axpy_f2d<<<(unsigned)((knn + 255) / 256), 256, 0, st>>>(xd, y, (int)knn);
      note_launch();
    }
    int fl = 0;
    O3G_CUDA_TRY(cudaMemcpyAsync(&fl, h->flags, sizeof(int), cudaMemcpyDeviceToHost, st));
    k_d2f<<<(unsigned)((knn + 255) / 256), 256, 0, st>>>(xd, bf, (int)knn);
    note_launch();
    if (X) O3G_CUDA_TRY(cudaMemcpyAsync(X + (size_t)g0 * n, bf, knn * 4, d2h, st));
    if (X64) O3G_CUDA_TRY(cudaMemcpyAsync(X64 + (size_t)g0 * n, xd, knn * 8, d2h, st));
    O3G_CUDA_TRY(cudaStreamSynchronize(st));
    for (int c = 0; c < K; ++c) {
      if (iters) iters[g0 + c] = it_of[c];
      if (relres) relres[g0 + c] = rel[c];
      if (!(rel[c] <= tol)) all_converged = false;
    }
    if (fl) {
      timed_out = true;
      break;
    }
  }
  tm.end(st);
  if (timed_out) {
    set_error("o3g_bem_solve_many: a grid barrier timed out");
    return O3G_ERR_TIMEOUT;
  }
  if (!all_converged) {
    set_error("o3g_bem_solve_many: some right-hand sides did not reach the tolerance (see relres)");
    return O3G_ERR_NOT_CONVERGED;
  }
  return O3G_OK;
}

// GMRES(restart) for several right-hand sides in lockstep: each keeps its own Krylov basis,
// Hessenberg matrix and restarts (the single-vector algorithm of o3g_bem_solve_gmres), and
// every iteration applies A to all of their current vectors in one pass over the matrix.
extern "C" int32_t o3g_bem_solve_gmres_many(o3g_bem_t* h, int32_t nrhs, const float* B, float* X, double* X64,
                                            int32_t mem, double tol, int32_t max_iter, int32_t restart,
                                            int32_t* iters, double* relres, void* stream) {
  O3G_TRY(many_args(h, nrhs, B, mem, tol, max_iter, "o3g_bem_solve_gmres_many"));
  if (restart < 1 || restart > 500) {
    set_error("o3g_bem_solve_gmres_many: restart must be 1..500");
    return O3G_ERR_INVALID_ARG;
  }
  if (nrhs == 0) return O3G_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const int n = h->n;
  const int m = std::min(restart, max_iter);
  const int KM = std::min(nrhs, kMaxRhs);
  const int ncb = (n + kMvChunkM - 1) / kMvChunkM;
  const int nrb = (n + 255) / 256;
  const size_t kn = (size_t)KM * n;
  const int nkb = (n + kKrylovRows - 1) / kKrylovRows;
  const int bs = h->bs, npb = n / bs;
  const bool pre = bs > 1;   // right-preconditioned by the diagonal blocks, as o3g_bem_solve_gmres
  const size_t need = align_up(kn * (m + 1) * 8) + 2 * align_up(kn * 8) + 3 * align_up(kn * 4) +
                      align_up((size_t)ncb * kn * 8) + align_up((size_t)KM * nrb * 8) +
                      align_up((size_t)KM * 2 * (m + 1) * 8) + 2 * align_up((size_t)nkb * (m + 1) * 8) +
                      align_up((size_t)n * bs * 8) + align_up(kn * 8);
  O3G_TRY(bem_scratch(h, need));
  Carve cv(h->scratch);
  double* V = cv.take<double>(kn * (m + 1));     // basis of column c at V + c (m+1) n
  double* bd = cv.take<double>(kn);
  double* xd = cv.take<double>(kn);
  float* bf = cv.take<float>(kn);
  float* xh = cv.take<float>(kn);
  float* xl = cv.take<float>(kn);
  double* part = cv.take<double>((size_t)ncb * kn);
  double* nrm = cv.take<double>((size_t)KM * nrb);
  double* hd = cv.take<double>((size_t)KM * 2 * (m + 1));
  double* kpart = cv.take<double>((size_t)nkb * (m + 1));
  double* npart = cv.take<double>((size_t)nkb * (m + 1));
  double* Minv = cv.take<double>((size_t)n * bs);
  double* zb = cv.take<double>(kn);   // per column: M^-1 v, and V y before M^-1
  std::vector<double> hnp((size_t)nkb);
  if (pre) block_inv(h->A, h->ld, npb, bs, Minv, st);
  const cudaMemcpyKind h2d = mem == O3G_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  const cudaMemcpyKind d2h = mem == O3G_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  bool all_converged = true;
  KernelTimer& tm = thread_timer();
  tm.begin(st);
  struct Rhs {
    std::vector<double> H, cs, sn, g, y;
    double bnorm = 0.0, rel = 1.0;
    int k = 0, total = 0;
    bool done = false, fresh = true;   // fresh: a cycle starts (residual, basis reset) next
  };
  for (int g0 = 0; g0 < nrhs; g0 += kMaxRhs) {
    const int K = std::min(kMaxRhs, nrhs - g0);
    const size_t knn = (size_t)K * n;
    O3G_CUDA_TRY(cudaMemcpyAsync(bf, B + (size_t)g0 * n, knn * 4, h2d, st));
    k_f2d<<<(unsigned)((knn + 255) / 256), 256, 0, st>>>(bf, bd, (int)knn);
    note_launch();
    O3G_CUDA_TRY(cudaMemsetAsync(xd, 0, knn * 8, st));
    std::vector<Rhs> R(K);
    auto Vc = [&](int c, int k) { return V + ((size_t)c * (m + 1) + k) * n; };
    for (int c = 0; c < K; ++c) {
      R[c].H.assign((size_t)(m + 1) * m, 0.0);
      R[c].cs.assign(m, 0.0);
      R[c].sn.assign(m, 0.0);
      R[c].g.assign(m + 1, 0.0);
      R[c].y.assign(m, 0.0);
    }
    // ||b_c||
    {
      DIn none{}, bin{};
      DOut vout{};
      for (int c = 0; c < K; ++c) {
        bin.p[c] = bd + (size_t)c * n;
        vout.p[c] = Vc(c, 0);
      }
      std::vector<double> bb;
      O3G_TRY(matvec_multi(h, K, none, bin, vout, xh, xl, part, nrm, &bb, st));
      for (int c = 0; c < K; ++c) {
        R[c].bnorm = std::sqrt(bb[c]);
        if (R[c].bnorm == 0.0) { R[c].done = true; R[c].rel = 0.0; }
      }
    }
    for (;;) {
      // columns starting a cycle: r = b - A x into their V_0, in one pass (x = 0 on the
      // first cycle: r = b, no product)
      std::vector<int> fr;
      for (int c = 0; c < K; ++c)
        if (!R[c].done && R[c].fresh) fr.push_back(c);
      if (!fr.empty()) {
        DIn xin{}, bin{};
        DOut vout{};
        bool any_x = false;
        for (int q = 0; q < (int)fr.size(); ++q) {
          const int c = fr[q];
          xin.p[q] = xd + (size_t)c * n;
          bin.p[q] = bd + (size_t)c * n;
          vout.p[q] = Vc(c, 0);
          any_x = any_x || R[c].total > 0;
        }
        if (!any_x) xin = DIn{};
        std::vector<double> rr;
        O3G_TRY(matvec_multi(h, (int)fr.size(), xin, bin, vout, xh, xl, part, nrm, &rr, st));
        for (int q = 0; q < (int)fr.size(); ++q) {
          Rhs& s = R[fr[q]];
          s.rel = std::sqrt(rr[q]) / s.bnorm;
          if (s.rel <= tol || s.total >= max_iter) {
            s.done = true;
            continue;
          }
          const double beta = std::sqrt(rr[q]);
          k_kry_scale<<<nrb, 256, 0, st>>>(Vc(fr[q], 0), n, 1.0 / beta);
          note_launch();
          std::fill(s.g.begin(), s.g.end(), 0.0);
          s.g[0] = beta;
          s.k = 0;
          s.fresh = false;
        }
      }
      std::vector<int> act;
      for (int c = 0; c < K; ++c)
        if (!R[c].done) act.push_back(c);
      if (act.empty()) break;
      // w_c = A v_{c,k} for every active column, one pass
      {
        DIn xin{}, none{};
        DOut wout{};
        for (int q = 0; q < (int)act.size(); ++q) {
          xin.p[q] = Vc(act[q], R[act[q]].k);
          wout.p[q] = Vc(act[q], R[act[q]].k + 1);
          if (pre) {
            block_apply(Minv, npb, bs, xin.p[q], zb + (size_t)q * n, 0, st);
            xin.p[q] = zb + (size_t)q * n;
          }
        }
        O3G_TRY(matvec_multi(h, (int)act.size(), xin, none, wout, xh, xl, part, nrm, nullptr, st));
      }
      for (int c : act) {
        Rhs& s = R[c];
        const int k = s.k;
        double* Vb = Vc(c, 0);
        double* w = Vc(c, k + 1);
        double* hc_d = hd + (size_t)c * 2 * (m + 1);
        for (int pass = 0; pass < 2; ++pass) gs_pass(Vb, n, k + 1, w, hc_d + (size_t)pass * (m + 1), kpart, st);
        norm_partials(w, n, npart, st);
        std::vector<double> hc(2 * (size_t)(m + 1));
        O3G_CUDA_TRY(cudaMemcpyAsync(hc.data(), hc_d, hc.size() * 8, cudaMemcpyDeviceToHost, st));
        O3G_CUDA_TRY(cudaMemcpyAsync(hnp.data(), npart, (size_t)nkb * 8, cudaMemcpyDeviceToHost, st));
        O3G_CUDA_TRY(cudaStreamSynchronize(st));
        const double wn = std::sqrt(host_sum(hnp));
        auto Hat = [&](int i, int kk) -> double& { return s.H[(size_t)kk * (m + 1) + i]; };
        for (int i = 0; i <= k; ++i) Hat(i, k) = hc[i] + hc[(size_t)(m + 1) + i];
        Hat(k + 1, k) = wn;
        if (wn > 0.0) {
          k_kry_scale<<<nrb, 256, 0, st>>>(w, n, 1.0 / wn);
          note_launch();
        }
        for (int i = 0; i < k; ++i) {
          const double a = Hat(i, k), cc = Hat(i + 1, k);
          Hat(i, k) = s.cs[i] * a + s.sn[i] * cc;
          Hat(i + 1, k) = -s.sn[i] * a + s.cs[i] * cc;
        }
        const double dd = std::hypot(Hat(k, k), Hat(k + 1, k));
        s.cs[k] = dd > 0.0 ? Hat(k, k) / dd : 1.0;
        s.sn[k] = dd > 0.0 ? Hat(k + 1, k) / dd : 0.0;
        Hat(k, k) = dd;
        Hat(k + 1, k) = 0.0;
        s.g[k + 1] = -s.sn[k] * s.g[k];
        s.g[k] = s.cs[k] * s.g[k];
        s.k = k + 1;
        ++s.total;
        if (s.k == m || s.total >= max_iter || std::fabs(s.g[s.k]) <= 0.5 * tol * s.bnorm || wn == 0.0) {
          // end of the cycle: x += V y with H(0:k, 0:k) y = g(0:k)
          const int kk = s.k;
          for (int i = kk - 1; i >= 0; --i) {
            double sacc = s.g[i];
            for (int j = i + 1; j < kk; ++j) sacc -= Hat(i, j) * s.y[j];
            s.y[i] = Hat(i, i) != 0.0 ? sacc / Hat(i, i) : 0.0;
          }
          O3G_CUDA_TRY(cudaMemcpyAsync(hc_d, s.y.data(), (size_t)kk * 8, cudaMemcpyHostToDevice, st));
          if (pre) {
            double* z = zb + (size_t)c * n;
            O3G_CUDA_TRY(cudaMemsetAsync(z, 0, (size_t)n * 8, st));
            k_kry_update<<<nrb, 256, 0, st>>>(Vb, n, kk, hc_d, 1.0, z);
            note_launch();
            block_apply(Minv, npb, bs, z, xd + (size_t)c * n, 1, st);
          } else {
            k_kry_update<<<nrb, 256, 0, st>>>(Vb, n, kk, hc_d, 1.0, xd + (size_t)c * n);
            note_launch();
          }
          s.fresh = true;
        }
      }
    }
    k_d2f<<<(unsigned)((knn + 255) / 256), 256, 0, st>>>(xd, bf, (int)knn);
    note_launch();
    if (X) O3G_CUDA_TRY(cudaMemcpyAsync(X + (size_t)g0 * n, bf, knn * 4, d2h, st));
    if (X64) O3G_CUDA_TRY(cudaMemcpyAsync(X64 + (size_t)g0 * n, xd, knn * 8, d2h, st));
    O3G_CUDA_TRY(cudaStreamSynchronize(st));
    for (int c = 0; c < K; ++c) {
      if (iters) iters[g0 + c] = R[c].total;
      if (relres) relres[g0 + c] = R[c].rel;
      if (!(R[c].rel <= tol)) all_converged = false;
    }
  }
  tm.end(st);
  if (!all_converged) {
    set_error("o3g_bem_solve_gmres_many: some right-hand sides did not reach the tolerance (see relres)");
    return O3G_ERR_NOT_CONVERGED;
  }
  return O3G_OK;
}
