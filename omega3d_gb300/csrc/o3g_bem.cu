// o3g_bem.cu -- the BEM system of the boundary solve: BEM<S,I> (BEM.h:44-234).
//
// The reference holds a dense Eigen matrix and solves it with GMRES (BEM.h:182-202),
// checking ||Ax-b||/||b|| afterwards (:227-230).  Here the matrix lives on the device and
// is solved by
//   * an FP32 LU factorisation with partial pivoting (row-by-row the same pivot choice
//     as LAPACK's getrf: largest magnitude, first index on ties), panels of kNb columns:
//       - k_panel_lu: one cooperative kernel factors the whole kNb-column panel; each
//         block keeps its slab of rows in shared memory; per column every block publishes
//         its local pivot candidate (value, row, the whole row) and, for the block holding
//         the diagonal row, that row; one bounded grid barrier later every block knows the
//         pivot and both rows to swap, so a column costs one barrier;
//       - k_laswp: the panel's row interchanges applied to the other columns;
//       - k_trsm_unit_lower: U12 = L11^-1 A12, one warp per column, L11 in shared memory;
//       - trailing update A22 -= L21 U12 as a TF32 tensor-core GEMM (cuBLAS, a plain GEMM);
//   * iterative refinement: residuals r = b - A x formed in FP64 from the unfactored FP32
//     matrix and the FP64 iterate, corrections from the FP32 factors (forward/back
//     substitution in one cooperative kernel each), until ||r||/||b|| <= tol.
// Every grid barrier here spins at most kSpinLimit rounds, then sets an error flag that all
// blocks check, so a fault in the barrier logic ends the kernel instead of hanging.
#include "o3g_common.cuh"

#include <cublas_v2.h>

#include <cmath>
#include <cstdio>
#include <vector>

namespace o3g {

constexpr int kNb = 128;              // panel width
constexpr int kPanelThreads = 256;
constexpr int kSolveThreads = 256;
constexpr unsigned long long kSpinLimit = 1ull << 25;

struct Barrier {
  unsigned* count;
  unsigned* gen;
  int* err;
};

// grid-wide barrier with a bounded spin; returns false (in every thread) once the error
// flag is set, by a timeout here or anywhere else
__device__ bool grid_sync(const Barrier& b) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* gen = b.gen;
    const unsigned g = *gen;
    __threadfence();
    const unsigned arrived = atomicAdd(b.count, 1u) + 1u;
    if (arrived == gridDim.x) {
      atomicExch(b.count, 0u);
      __threadfence();
      atomicAdd(b.gen, 1u);
    } else {
      unsigned long long it = 0;
      while (*gen == g) {
        if (*(volatile int*)b.err) break;
        if (++it > kSpinLimit) {
          atomicExch(b.err, 1);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    ok = (*(volatile int*)b.err == 0);
  }
  __syncthreads();
  return ok != 0;
}

struct PanelArgs {
  float* A;
  long long ld;
  int n, k0, jb, R;        // matrix order, first panel column, panel width, rows per block
  int* piv;                // absolute pivot row of each column
  float* cval;             // [2][G] candidate |value|
  int* crow;               // [2][G] candidate row
  float* crows;            // [2][G][jb] candidate rows
  float* drow;             // [2][jb] diagonal rows
  int* singular;           // first singular column + 1, or 0
  Barrier bar;
};

__global__ void __launch_bounds__(kPanelThreads) k_panel_lu(PanelArgs a) {
  extern __shared__ float smem[];
  const int G = gridDim.x, b = blockIdx.x, jb = a.jb, R = a.R;
  float* slab = smem;                       // [jb][R]
  float* prow = smem + (size_t)jb * R;      // [jb] pivot row
  __shared__ float rv[kPanelThreads / 32];
  __shared__ int ri[kPanelThreads / 32];
  __shared__ int sg_row, sg_owner;
  __shared__ float sg_val;
  const int r0 = a.k0 + b * R;
  const int nr = max(0, min(a.n, r0 + R) - r0);
  for (int j = 0; j < jb; ++j)
    for (int r = threadIdx.x; r < nr; r += blockDim.x) slab[(size_t)j * R + r] = a.A[(size_t)(a.k0 + j) * a.ld + r0 + r];
  __syncthreads();
  for (int j = 0; j < jb; ++j) {
    const int c = a.k0 + j, par = j & 1;
    // local argmax of |a(i, c)| over my rows i >= c (first index on ties)
    float best = -1.f;
    int bi = 0x7fffffff;
    for (int r = threadIdx.x; r < nr; r += blockDim.x) {
      if (r0 + r < c) continue;
      const float v = fabsf(slab[(size_t)j * R + r]);
      if (v > best || (v == best && r0 + r < bi)) { best = v; bi = r0 + r; }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const float ov = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
    }
    if ((threadIdx.x & 31) == 0) { rv[threadIdx.x >> 5] = best; ri[threadIdx.x >> 5] = bi; }
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int w = 1; w < kPanelThreads / 32; ++w)
        if (rv[w] > rv[0] || (rv[w] == rv[0] && ri[w] < ri[0])) { rv[0] = rv[w]; ri[0] = ri[w]; }
      a.cval[par * G + b] = rv[0];
      a.crow[par * G + b] = ri[0];
    }
    __syncthreads();
    const int lrow = ri[0];
    if (rv[0] >= 0.f)
      for (int jj = threadIdx.x; jj < jb; jj += blockDim.x)
        a.crows[((size_t)par * G + b) * jb + jj] = slab[(size_t)jj * R + (lrow - r0)];
    if (c >= r0 && c < r0 + nr)
      for (int jj = threadIdx.x; jj < jb; jj += blockDim.x) a.drow[par * jb + jj] = slab[(size_t)jj * R + (c - r0)];
    if (!grid_sync(a.bar)) return;
    // global pivot: every block scans all candidates (same answer everywhere)
    best = -1.f;
    bi = 0x7fffffff;
    int bo = 0;
    for (int g = threadIdx.x; g < G; g += blockDim.x) {
      const float v = a.cval[par * G + g];
      const int i = a.crow[par * G + g];
      if (v > best || (v == best && i < bi)) { best = v; bi = i; bo = g; }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const float ov = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      const int oo = __shfl_xor_sync(0xffffffffu, bo, o);
      if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; bo = oo; }
    }
    if ((threadIdx.x & 31) == 0) { rv[threadIdx.x >> 5] = best; ri[threadIdx.x >> 5] = bi; smem[(size_t)jb * R + jb + (threadIdx.x >> 5)] = __int_as_float(bo); }
    __syncthreads();
    if (threadIdx.x == 0) {
      float v = rv[0];
      int i = ri[0], ow = __float_as_int(smem[(size_t)jb * R + jb]);
      for (int w = 1; w < kPanelThreads / 32; ++w)
        if (rv[w] > v || (rv[w] == v && ri[w] < i)) { v = rv[w]; i = ri[w]; ow = __float_as_int(smem[(size_t)jb * R + jb + w]); }
      if (!(v >= 0.f) || i < c || i >= a.n) {   // no finite candidate (a NaN column): keep the row
        i = c;
        ow = -1;
        v = 0.f;
      }
      sg_val = v;
      sg_row = i;
      sg_owner = ow;
      if (b == 0) a.piv[c] = i;
      if (b == 0 && !(v > 0.f) && *a.singular == 0) *a.singular = c + 1;
    }
    __syncthreads();
    const int prow_i = sg_row;
    for (int jj = threadIdx.x; jj < jb; jj += blockDim.x)
      prow[jj] = sg_owner >= 0 ? a.crows[((size_t)par * G + sg_owner) * jb + jj] : a.drow[par * jb + jj];
    __syncthreads();
    if (prow_i != c) {
      if (c >= r0 && c < r0 + nr)
        for (int jj = threadIdx.x; jj < jb; jj += blockDim.x) slab[(size_t)jj * R + (c - r0)] = prow[jj];
      if (prow_i >= r0 && prow_i < r0 + nr)
        for (int jj = threadIdx.x; jj < jb; jj += blockDim.x)
          slab[(size_t)jj * R + (prow_i - r0)] = a.drow[par * jb + jj];
    }
    __syncthreads();
    const float p = prow[j];
    if (p != 0.f) {
      for (int r = threadIdx.x; r < nr; r += blockDim.x) {
        if (r0 + r <= c) continue;
        const float l = slab[(size_t)j * R + r] / p;
        slab[(size_t)j * R + r] = l;
        for (int jj = j + 1; jj < jb; ++jj) slab[(size_t)jj * R + r] = fmaf(-l, prow[jj], slab[(size_t)jj * R + r]);
      }
    }
    __syncthreads();
  }
  for (int j = 0; j < jb; ++j)
    for (int r = threadIdx.x; r < nr; r += blockDim.x) a.A[(size_t)(a.k0 + j) * a.ld + r0 + r] = slab[(size_t)j * R + r];
}

// row interchanges k0..k0+jb-1 applied to the columns outside the panel
__global__ void k_laswp(float* A, long long ld, int n, int k0, int jb, const int* piv) {
  int col = blockIdx.x * blockDim.x + threadIdx.x;
  const int nother = n - jb;
  if (col >= nother) return;
  if (col >= k0) col += jb;
  float* a = A + (size_t)col * ld;
  for (int i = k0; i < k0 + jb; ++i) {
    const int p = piv[i];
    if (p != i && p > i && p < n) {
      const float t = a[i];
      a[i] = a[p];
      a[p] = t;
    }
  }
}

// U12 = L11^-1 A12: one warp per column of A12, L11 (unit lower, jb x jb) in shared memory
__global__ void __launch_bounds__(256) k_trsm_unit_lower(float* A, long long ld, int n, int k0, int jb) {
  extern __shared__ float L[];   // [jb][jb] column-major
  for (int e = threadIdx.x; e < jb * jb; e += blockDim.x) {
    const int i = e % jb, j = e / jb;
    L[e] = A[(size_t)(k0 + j) * ld + k0 + i];
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ncols = n - k0 - jb;
  for (int cidx = blockIdx.x * (blockDim.x / 32) + warp; cidx < ncols; cidx += gridDim.x * (blockDim.x / 32)) {
    float* col = A + (size_t)(k0 + jb + cidx) * ld + k0;
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

// ------------------------------------------------------------------------------------
// solves with the factors: y = P b (gather), L y = y (unit lower), U x = y (upper)
__global__ void k_permute_to_float(const double* r, const int* perm, float* y, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = (float)r[perm[i]];
}

struct TrsvArgs {
  const float* LU;
  long long ld;
  int n;
  float* y;
  Barrier bar;
};

// forward substitution with the unit lower factor: per block column, every block solves the
// diagonal block redundantly (from L2), then updates its share of the rows below
__global__ void __launch_bounds__(kSolveThreads) k_trsv_lower(TrsvArgs a) {
  __shared__ float yd[kNb];
  const int G = gridDim.x;
  for (int k0 = 0; k0 < a.n; k0 += kNb) {
    const int jb = min(kNb, a.n - k0);
    if (threadIdx.x < 32) {
      float x[kNb / 32];
#pragma unroll
      for (int q = 0; q < kNb / 32; ++q) {
        const int m = q * 32 + threadIdx.x;
        x[q] = m < jb ? a.y[k0 + m] : 0.f;
      }
      for (int i = 0; i < jb; ++i) {
        const float xi = __shfl_sync(0xffffffffu, x[i >> 5], i & 31);
        const float* Lc = a.LU + (size_t)(k0 + i) * a.ld + k0;
#pragma unroll
        for (int q = 0; q < kNb / 32; ++q) {
          const int m = q * 32 + threadIdx.x;
          if (m > i && m < jb) x[q] = fmaf(-Lc[m], xi, x[q]);
        }
      }
#pragma unroll
      for (int q = 0; q < kNb / 32; ++q) {
        const int m = q * 32 + threadIdx.x;
        if (m < jb) yd[m] = x[q];
      }
    }
    __syncthreads();
    // rows below the block: y[i] -= sum_m L(i, k0+m) yd[m]
    const int rest = a.n - k0 - jb;
    const int chunk = (rest + G - 1) / G;
    const int i0 = k0 + jb + blockIdx.x * chunk, i1 = min(a.n, i0 + chunk);
    for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
      float s = 0.f;
      for (int m = 0; m < jb; ++m) s = fmaf(a.LU[(size_t)(k0 + m) * a.ld + i], yd[m], s);
      a.y[i] -= s;
    }
    if (blockIdx.x == 0 && threadIdx.x < jb) a.y[k0 + threadIdx.x] = yd[threadIdx.x];
    if (!grid_sync(a.bar)) return;
  }
}

// back substitution with the upper factor (non-unit diagonal)
__global__ void __launch_bounds__(kSolveThreads) k_trsv_upper(TrsvArgs a) {
  __shared__ float yd[kNb];
  const int G = gridDim.x;
  const int nblk = (a.n + kNb - 1) / kNb;
  for (int kb = nblk - 1; kb >= 0; --kb) {
    const int k0 = kb * kNb, jb = min(kNb, a.n - k0);
    if (threadIdx.x < 32) {
      float x[kNb / 32];
#pragma unroll
      for (int q = 0; q < kNb / 32; ++q) {
        const int m = q * 32 + threadIdx.x;
        x[q] = m < jb ? a.y[k0 + m] : 0.f;
      }
      for (int i = jb - 1; i >= 0; --i) {
        const float* Uc = a.LU + (size_t)(k0 + i) * a.ld + k0;
        // x_i = y_i / U_ii on the owning lane, then broadcast
        const float d = Uc[i];
        float xi = 0.f;
        if ((i & 31) == (int)threadIdx.x) { x[i >> 5] = x[i >> 5] / d; }
        xi = __shfl_sync(0xffffffffu, x[i >> 5], i & 31);
#pragma unroll
        for (int q = 0; q < kNb / 32; ++q) {
          const int m = q * 32 + threadIdx.x;
          if (m < i) x[q] = fmaf(-Uc[m], xi, x[q]);
        }
      }
#pragma unroll
      for (int q = 0; q < kNb / 32; ++q) {
        const int m = q * 32 + threadIdx.x;
        if (m < jb) yd[m] = x[q];
      }
    }
    __syncthreads();
    // rows above: y[i] -= sum_m U(i, k0+m) yd[m], i < k0
    const int chunk = (k0 + G - 1) / G;
    const int i0 = blockIdx.x * chunk, i1 = min(k0, i0 + chunk);
    for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
      float s = 0.f;
      for (int m = 0; m < jb; ++m) s = fmaf(a.LU[(size_t)(k0 + m) * a.ld + i], yd[m], s);
      a.y[i] -= s;
    }
    if (blockIdx.x == 0 && threadIdx.x < jb) a.y[k0 + threadIdx.x] = yd[threadIdx.x];
    if (!grid_sync(a.bar)) return;
  }
}

// FP64 residual partials: part[cb][i] = sum_{j in chunk cb} A(i,j) x(j)
__global__ void k_resid_part(const float* __restrict__ A, long long ld, int n, const double* __restrict__ x,
                             int cchunk, double* __restrict__ part) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int cb = blockIdx.y;
  if (i >= n) return;
  const int j0 = cb * cchunk, j1 = min(n, j0 + cchunk);
  double s = 0.0;
  for (int j = j0; j < j1; ++j) s = fma((double)A[(size_t)j * ld + i], x[j], s);
  part[(size_t)cb * n + i] = s;
}
// r = b - sum_cb part[cb]; also accumulates ||r||^2 and ||b||^2 per block into nrm[2*blockIdx]
__global__ void k_resid_finish(const double* __restrict__ part, int ncb, int n, const double* __restrict__ b,
                               double* __restrict__ r, double* __restrict__ nrm) {
  __shared__ double s1[8], s2[8];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double rr = 0.0, bb = 0.0;
  if (i < n) {
    double s = 0.0;
    for (int k = 0; k < ncb; ++k) s += part[(size_t)k * n + i];
    const double ri = b[i] - s;
    r[i] = ri;
    rr = ri * ri;
    bb = b[i] * b[i];
  }
  for (int o = 16; o > 0; o >>= 1) {
    rr += __shfl_xor_sync(0xffffffffu, rr, o);
    bb += __shfl_xor_sync(0xffffffffu, bb, o);
  }
  if ((threadIdx.x & 31) == 0) { s1[threadIdx.x >> 5] = rr; s2[threadIdx.x >> 5] = bb; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a1 = 0.0, a2 = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { a1 += s1[w]; a2 += s2[w]; }
    nrm[2 * blockIdx.x] = a1;
    nrm[2 * blockIdx.x + 1] = a2;
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
  char* scratch = nullptr;
  size_t scratch_bytes = 0;
  int* flags = nullptr;   // [0] barrier error, [1] singular column + 1, [2..3] barrier count/gen
  cublasHandle_t cublas = nullptr;
  bool factored = false;
  int panel_blocks = 0, solve_blocks = 0;
};

using namespace o3g;

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
  cudaError_t e = cudaMalloc((void**)&h->A, mat);
  if (e == cudaSuccess) e = cudaMalloc((void**)&h->LU, mat);
  if (e == cudaSuccess) e = cudaMalloc((void**)&h->piv, n * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc((void**)&h->perm, n * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc((void**)&h->flags, 64 * sizeof(int));
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    set_error_cuda("o3g_bem_create: cudaMalloc", e);
    cudaFree(h->A); cudaFree(h->LU); cudaFree(h->piv); cudaFree(h->perm); cudaFree(h->flags);
    delete h;
    return O3G_ERR_ALLOC;
  }
  cudaMemset(h->A, 0, mat);
  if (cublasCreate(&h->cublas) != CUBLAS_STATUS_SUCCESS) {
    set_error("o3g_bem_create: cublasCreate failed");
    cudaFree(h->A); cudaFree(h->LU); cudaFree(h->piv); cudaFree(h->perm); cudaFree(h->flags);
    delete h;
    return O3G_ERR_CUDA;
  }
  cublasSetMathMode(h->cublas, CUBLAS_TF32_TENSOR_OP_MATH);
  *out = h;
  return O3G_OK;
}

extern "C" int32_t o3g_bem_destroy(o3g_bem_t* h) {
  if (!h) return O3G_OK;
  cudaDeviceSynchronize();
  cudaFree(h->A); cudaFree(h->LU); cudaFree(h->piv); cudaFree(h->perm); cudaFree(h->flags); cudaFree(h->scratch);
  if (h->cublas) cublasDestroy(h->cublas);
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
  cudaError_t e = cudaMalloc((void**)&h->scratch, bytes);
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
  int G = df.num_sms;
  int R = (n + G - 1) / G;
  size_t smem = ((size_t)kNb * R + kNb + 32) * sizeof(float);
  if (smem > max_smem) {
    set_error("o3g_bem_factor: matrix too large for the panel kernel's shared memory");
    return O3G_ERR_INVALID_ARG;
  }
  O3G_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_panel_lu, kPanelThreads, smem));
  if (per_sm < 1) {
    set_error("o3g_bem_factor: panel kernel cannot be resident");
    return O3G_ERR_INVALID_ARG;
  }
  const size_t cand = align_up(2 * (size_t)G * sizeof(float)) + align_up(2 * (size_t)G * sizeof(int)) +
                      align_up(2 * (size_t)G * kNb * sizeof(float)) + align_up(2 * (size_t)kNb * sizeof(float));
  O3G_TRY(bem_scratch(h, cand + align_up((size_t)n * 64)));
  Carve cv(h->scratch);
  float* cval = cv.take<float>(2 * (size_t)G);
  int* crow = cv.take<int>(2 * (size_t)G);
  float* crows = cv.take<float>(2 * (size_t)G * kNb);
  float* drow = cv.take<float>(2 * (size_t)kNb);
  O3G_CUDA_TRY(cudaMemsetAsync(h->flags, 0, 64 * sizeof(int), st));
  O3G_CUDA_TRY(cudaMemcpy2DAsync(h->LU, ld * sizeof(float), h->A, ld * sizeof(float), n * sizeof(float), n,
                                 cudaMemcpyDeviceToDevice, st));
  cublasSetStream(h->cublas, st);
  KernelTimer& tm = thread_timer();
  tm.begin(st);
  const float minus1 = -1.f, one = 1.f;
  for (int k0 = 0; k0 < n; k0 += kNb) {
    const int jb = n - k0 < kNb ? n - k0 : kNb;
    const int m = n - k0;
    int g = G;
    int r = (m + g - 1) / g;
    if (r < 32) {   // short panels: fewer blocks
      g = (m + 31) / 32;
      r = (m + g - 1) / g;
    }
    PanelArgs pa;
    pa.A = h->LU; pa.ld = ld; pa.n = n; pa.k0 = k0; pa.jb = jb; pa.R = r;
    pa.piv = h->piv; pa.cval = cval; pa.crow = crow; pa.crows = crows; pa.drow = drow;
    pa.singular = h->flags + 1;
    pa.bar = Barrier{(unsigned*)(h->flags + 2), (unsigned*)(h->flags + 3), h->flags};
    void* args[] = {&pa};
    const size_t sm = ((size_t)jb * r + jb + 32) * sizeof(float);
    O3G_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)k_panel_lu, dim3(g), dim3(kPanelThreads), args, sm, st));
    note_launch();
    if (n - jb > 0) {
      k_laswp<<<(n - jb + 255) / 256, 256, 0, st>>>(h->LU, ld, n, k0, jb, h->piv);
      note_launch();
    }
    const int rest = n - k0 - jb;
    if (rest > 0) {
      const size_t tsm = (size_t)jb * jb * sizeof(float);
      O3G_CUDA_TRY(cudaFuncSetAttribute(k_trsm_unit_lower, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsm));
      int tb = (rest + 7) / 8;
      if (tb > 4 * df.num_sms) tb = 4 * df.num_sms;
      k_trsm_unit_lower<<<tb, 256, tsm, st>>>(h->LU, ld, n, k0, jb);
      note_launch();
      float* A21 = h->LU + (size_t)k0 * ld + k0 + jb;
      float* A12 = h->LU + (size_t)(k0 + jb) * ld + k0;
      float* A22 = h->LU + (size_t)(k0 + jb) * ld + k0 + jb;
      const cublasStatus_t cs = cublasGemmEx(h->cublas, CUBLAS_OP_N, CUBLAS_OP_N, rest, rest, jb, &minus1, A21,
                                             CUDA_R_32F, (int)ld, A12, CUDA_R_32F, (int)ld, &one, A22, CUDA_R_32F,
                                             (int)ld, CUBLAS_COMPUTE_32F_FAST_TF32, CUBLAS_GEMM_DEFAULT);
      if (cs != CUBLAS_STATUS_SUCCESS) {
        set_error("o3g_bem_factor: cublasGemmEx (TF32 trailing update) failed");
        return O3G_ERR_CUDA;
      }
    }
  }
  tm.end(st);
  O3G_CUDA_TRY(cudaGetLastError());
  int fl[2] = {0, 0};
  O3G_CUDA_TRY(cudaMemcpyAsync(fl, h->flags, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
  std::vector<int> piv(n);
  O3G_CUDA_TRY(cudaMemcpyAsync(piv.data(), h->piv, n * sizeof(int), cudaMemcpyDeviceToHost, st));
  O3G_CUDA_TRY(cudaStreamSynchronize(st));
  if (fl[0]) {
    set_error("o3g_bem_factor: a grid barrier timed out");
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
  const int cchunk = 2048;
  const int ncb = (n + cchunk - 1) / cchunk;
  const int nrb = (n + 255) / 256;
  const size_t need = align_up((size_t)n * 8) * 3 + align_up((size_t)n * 4) * 3 + align_up((size_t)ncb * n * 8) +
                      align_up((size_t)nrb * 16);
  O3G_TRY(bem_scratch(h, need));
  Carve cv(h->scratch);
  double* bd = cv.take<double>(n);
  double* xd = cv.take<double>(n);
  double* rd = cv.take<double>(n);
  float* bf = cv.take<float>(n);
  float* y = cv.take<float>(n);
  float* xf = cv.take<float>(n);
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
  O3G_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trsv_lower, kSolveThreads, 0));
  if (per_sm < 1) return O3G_ERR_CUDA;
  TrsvArgs ta;
  ta.LU = h->LU; ta.ld = ld; ta.n = n; ta.y = y;
  ta.bar = Barrier{(unsigned*)(h->flags + 2), (unsigned*)(h->flags + 3), h->flags};
  void* targs[] = {&ta};
  std::vector<double> hn(2 * (size_t)nrb);
  double rel = 1.0, bnorm = 0.0;
  int it = 0;
  KernelTimer& tm = thread_timer();
  tm.begin(st);
  for (it = 0; it <= max_iter; ++it) {
    if (it > 0) {
      k_resid_part<<<dim3(nrb, ncb), 256, 0, st>>>(h->A, ld, n, xd, cchunk, part);
      note_launch();
    } else {
      // r = b at x = 0 (part = 0 is implied): reuse the finish kernel with zero partials
      O3G_CUDA_TRY(cudaMemsetAsync(part, 0, (size_t)n * 8, st));
    }
    k_resid_finish<<<nrb, 256, 0, st>>>(part, it > 0 ? ncb : 1, n, bd, rd, nrm);
    note_launch();
    O3G_CUDA_TRY(cudaMemcpyAsync(hn.data(), nrm, 2 * (size_t)nrb * 8, cudaMemcpyDeviceToHost, st));
    O3G_CUDA_TRY(cudaStreamSynchronize(st));
    double rr = 0.0, bb = 0.0;
    for (int k = 0; k < nrb; ++k) { rr += hn[2 * k]; bb += hn[2 * k + 1]; }
    bnorm = std::sqrt(bb);
    rel = bnorm > 0.0 ? std::sqrt(rr) / bnorm : std::sqrt(rr);
    if (rel <= tol || it == max_iter) break;
    k_permute_to_float<<<nrb, 256, 0, st>>>(rd, h->perm, y, n);
    O3G_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)k_trsv_lower, dim3(G), dim3(kSolveThreads), targs, 0, st));
    O3G_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)k_trsv_upper, dim3(G), dim3(kSolveThreads), targs, 0, st));
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
