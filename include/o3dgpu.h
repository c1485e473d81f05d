/*
 * o3dgpu.h -- C-ABI of the GB300 (sm_103a) Biot-Savart / BEM hot path of Omega3D.
 *
 * Every entry point is extern "C", takes plain pointers and sizes, and returns an
 * int32 status (O3G_OK == 0).  No entry point allocates caller-visible memory: the
 * caller owns every array, as in the reference (Influence.h / Coefficients.h /
 * BEM.h, where the caller's std::vector<float> SoA arrays are read and accumulated
 * into).  Array arguments follow the reference's SoA layout: one pointer per
 * component (x, y, z; u, v, w; nine velocity-gradient components in the order
 * du/dx, dv/dx, dw/dx, du/dy, dv/dy, dw/dy, du/dz, dv/dz, dw/dz -- Kernels.h:184-192).
 *
 * `mem` says where the arrays live: O3G_MEM_HOST (the library stages them through
 * device memory inside the call and returns after the results are back in host
 * memory) or O3G_MEM_DEVICE (device pointers; the call is asynchronous on `stream`).
 * `stream` is a cudaStream_t (NULL = the legacy default stream).
 *
 * Velocity results ACCUMULATE (+=) into the caller's arrays, exactly like the
 * reference's points_affect_points (Influence.h:299-308); zero_vels / finalize_vels
 * (the 1/4pi factor and the freestream) stay with the caller (Convection.h:161,175).
 */
#ifndef O3DGPU_H
#define O3DGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------ */
enum {
  O3G_OK = 0,
  O3G_ERR_INVALID_ARG = 1,   /* bad size, null pointer, unknown enum value          */
  O3G_ERR_CUDA = 2,          /* a CUDA runtime call failed (see o3g_last_error)    */
  O3G_ERR_NO_DEVICE = 3,     /* no usable sm_103 device                            */
  O3G_ERR_ALLOC = 4,         /* device workspace could not be allocated            */
  O3G_ERR_NOT_CONVERGED = 5, /* iterative refinement did not reach the tolerance   */
  O3G_ERR_TIMEOUT = 6,       /* a bounded device-side wait ran out                 */
  O3G_ERR_SINGULAR = 7,      /* zero or non-finite pivot in a factorisation        */
  O3G_ERR_NONFINITE = 8,     /* non-finite values where finite ones are required   */
  O3G_ERR_STATE = 9,         /* call made in the wrong state (e.g. solve before A) */
  O3G_ERR_CAPACITY = 10      /* output arrays too small; the needed count is returned */
};

/* ---- enumerations -------------------------------------------------------------- */
/* Regularised Biot-Savart cores.  RM/WL/EXP/V2 follow CoreFunc.h (:43-83, :241-289,
 * :86-238, :292-341); GAUSS is this library's own Gaussian core (no counterpart in
 * the reference, whose Gaussian kernels serve diffusion only). */
enum { O3G_CORE_RM = 0, O3G_CORE_WL = 1, O3G_CORE_EXP = 2, O3G_CORE_GAUSS = 3, O3G_CORE_V2 = 4 };

/* Arithmetic of the pair sums:
 *  PLAIN       FP32 pair arithmetic and FP32 accumulation (the reference's Vc path);
 *  COMPENSATED FP32 pair arithmetic with a Newton-refined rsqrt and per-tile partial
 *              sums folded into compensated (hi, lo) accumulators;
 *  FP64        everything in double (comparator / oracle on the device);
 *  ACCURATE    COMPENSATED sums of terms formed in double-single FP32 arithmetic: exact
 *              separations, d^2, core factor and cross product carried as float pairs,
 *              each velocity term rounded once (o3g_points_affect_points only, RM and
 *              Gaussian cores; gradients as in COMPENSATED). */
enum { O3G_PREC_PLAIN = 0, O3G_PREC_COMPENSATED = 1, O3G_PREC_FP64 = 2, O3G_PREC_ACCURATE = 3 };

enum { O3G_MEM_HOST = 0, O3G_MEM_DEVICE = 1 };

/* Diffusion core types (CoreType, Core.h:27): they set the neighbour weight of the split. */
enum { O3G_DIFFCORE_GAUSSIAN = 0, O3G_DIFFCORE_COMPACTG = 1 };

/* ---- library ------------------------------------------------------------------- */
/* Human-readable text for a status code (static storage). */
const char* o3g_status_string(int32_t status);
/* Last CUDA / validation message recorded by this thread (static per-thread storage). */
const char* o3g_last_error(void);
/* Library version as 10000*major + 100*minor + patch. */
int32_t o3g_version(void);
/* Device facts used for rooflines: SM count, SM clock (kHz), compute capability. */
int32_t o3g_device_info(int32_t* num_sms, int32_t* sm_clock_khz, int32_t* cc_major, int32_t* cc_minor);

/* Reference flop count per interaction (Kernels.h:49,93,154,252 + CoreFunc.h flops_*):
 * grads != 0 -> vel+grad kernel; have_tr != 0 -> thick-cored target.  Mirrors the
 * counts the reference uses to print GFlop/s (Influence.h:310,366,475,534). */
int32_t o3g_flops_per_pair(int32_t core, int32_t grads, int32_t have_tr);

/* Device time (ms) of the main kernel of the most recent call on this thread, when
 * timing is enabled with o3g_set_timing(1); returns O3G_ERR_STATE otherwise. */
int32_t o3g_set_timing(int32_t enable);
int32_t o3g_last_kernel_ms(float* ms);
/* Cumulative number of CUDA kernels this thread has launched through the library. */
int32_t o3g_launch_count(uint64_t* n);
/* Cumulative number of device allocations (cudaMalloc / cudaMallocAsync) the library has
 * made in this process, from any thread: its per-stream workspaces, BEM, RK2 and batch
 * handles, and the scratch of split, merge, reflection and shedding. */
int32_t o3g_alloc_count(uint64_t* n);

/* Wait test.  Some kernels wait on the device for one another's progress, each wait
 * bounded: the grid barriers of the BEM panel factorisation and triangular solves, and the
 * dependency waits of the particle split.  A wait that runs out sets an error word, every
 * other wait then returns at once, the kernels end, and the call returns O3G_ERR_TIMEOUT
 * with the device still usable.  With enable != 0 (process-wide, until called with 0)
 * those waits are given a condition that nothing fulfils (a barrier count one above the
 * number of blocks, a flag nothing sets) and a limit of about a millisecond, so that tests
 * can see them run out.  A split that runs out leaves the particles unchanged. */
int32_t o3g_debug_wait_test(int32_t enable);

/* Measures the FP32 FMA throughput of the current device (TFLOP/s, counting an FMA as
 * 2 flops) with a register-resident FMA-chain kernel: the measured denominator of the
 * pair kernels' roofline.  No counterpart in the reference. */
int32_t o3g_fp32_peak_probe(int32_t iters, void* stream, double* tflops, float* ms);

/* y[i] = exp(x[i]) (device arrays, n >= 0, asynchronous on `stream`) by the float exp the
 * plain FP32 exponential core uses in 1 - exp(-x) (CoreFunc.h:127-128), made for its
 * arguments, -16 < x < -0.001 (accurate for -20 <= x <= 0): rounded once from a float-float
 * value, so it is the correctly rounded float but for rare arguments within about 2^-12 ulp
 * of a rounding boundary, and 1 ulp from it there.  For tests and
 * measurement; no counterpart in the reference, which calls its host library's expf. */
int32_t o3g_exp_probe(int32_t n, const float* x, float* y, void* stream);
/* Check of the division-free x / 3 of the panel centroids against IEEE division on the
 * device, for the float bit patterns first .. first + count - 1 (count <= 2^32 - first):
 * *mismatches = how many results differ in any bit (synchronises on `stream`). */
int32_t o3g_div3_check(uint64_t first, uint64_t count, uint64_t* mismatches, void* stream);

/* C -= A B on the tensor cores (tcgen05, TF32 products, FP32 sums): the update of the BEM
 * factorisation (o3g_bem_factor), callable on its own.  Device arrays, column-major:
 * A m x k (leading dimension lda >= m), B k x n (ldb >= k, a multiple of 4, B 16-byte
 * aligned), C m x n (ldc >= m).  Synchronises the stream.  No counterpart in the
 * reference, which leaves the factorisation to Eigen on the host (BEM.h:182-195). */
int32_t o3g_gemm_tf32_sub(int32_t m, int32_t n, int32_t k, const float* A, int64_t lda, const float* B, int64_t ldb,
                          float* C, int64_t ldc, void* stream);

/* ---- points_affect_points -------------------------------------------------------
 * Replaces points_affect_points<float,A>(src, targ, restype, env), Influence.h:67-551,
 * and generalises the external solver hook external_vel_solver_f_, Influence.h:33-40.
 *   sources: ns vortex particles (sx,sy,sz position; sr core radius; ssx,ssy,ssz strength)
 *   targets: nt points; tr == NULL means field points (inert targets, Influence.h:205),
 *            otherwise thick-cored particles with radius tr
 *   results: tu,tv,tw += velocity sums; tug == NULL means velocity only
 *            (ResultsType velonly), else tug[0..8] += the nine gradient sums.
 * Sums carry no 1/4pi factor (finalize_vels applies it, ElementBase.h:187-193). */
int32_t o3g_points_affect_points(int32_t core, int32_t prec, int32_t mem,
                                 int32_t ns, const float* sx, const float* sy, const float* sz,
                                 const float* sr, const float* ssx, const float* ssy, const float* ssz,
                                 int32_t nt, const float* tx, const float* ty, const float* tz,
                                 const float* tr,
                                 float* tu, float* tv, float* tw, float* const* tug,
                                 void* stream);

/* Double-precision twin (S = A = double), mirrors external_vel_solver_d_, Influence.h:41-47.
 * Always computes in FP64. */
int32_t o3g_points_affect_points_d(int32_t core, int32_t mem,
                                   int32_t ns, const double* sx, const double* sy, const double* sz,
                                   const double* sr, const double* ssx, const double* ssy, const double* ssz,
                                   int32_t nt, const double* tx, const double* ty, const double* tz,
                                   const double* tr,
                                   double* tu, double* tv, double* tw, double* const* tug,
                                   void* stream);

/* ---- the reference's own external-solver hook -------------------------------------
 * Exactly the prototypes a reference built with EXTERNAL_VEL_SOLVE declares and calls
 * (Influence.h:33-48; call site :88-113), so that build links against this library with
 * no source change.  Arguments, in the reference's order: source count (by pointer),
 * source x, y, z, strengths sx, sy, sz, core radii; target count (by pointer), target
 * x, y, z; velocity u, v, w; the nine gradient arrays (Kernels.h:184-192 order).  All
 * arrays are host memory.  The targets carry no radius, so each is summed as a point
 * (the kernel_0v_0pg form, Kernels.h:253-290); results are ADDED (+=) to u, v, w and
 * the gradients, the caller zeroes them (Convection.h:161).  Nine NULL gradient
 * pointers give velocity only.  Synchronous on the legacy default stream.
 * Return: the flops of the call at the reference's own accounting,
 * nt (12 + flops_0v_0pg ns) (Influence.h:310), or -1 on an error (o3g_last_error).
 * The float hook uses the core and precision set by o3g_external_set_method, else the
 * environment (O3G_EXTERNAL_CORE = rm|wl|exp|gauss|v2, O3G_EXTERNAL_PREC =
 * plain|compensated), else WL and PLAIN: the reference's compiled-in core
 * (CoreFunc.h:37) and its float arithmetic.  The double hook computes in FP64. */
float external_vel_solver_f_(int* ns, const float* sx, const float* sy, const float* sz,
                             const float* ssx, const float* ssy, const float* ssz, const float* sr,
                             int* nt, const float* tx, const float* ty, const float* tz,
                             float* tu, float* tv, float* tw,
                             float* tux, float* tvx, float* twx, float* tuy, float* tvy, float* twy,
                             float* tuz, float* tvz, float* twz);
float external_vel_solver_d_(int* ns, const double* sx, const double* sy, const double* sz,
                             const double* ssx, const double* ssy, const double* ssz, const double* sr,
                             int* nt, const double* tx, const double* ty, const double* tz,
                             double* tu, double* tv, double* tw,
                             double* tux, double* tvx, double* twx, double* tuy, double* tvy, double* twy,
                             double* tuz, double* tvz, double* twz);
/* Core (O3G_CORE_*, or -1 for the environment / default) and precision (PLAIN or
 * COMPENSATED, or -1) of the float hook above, process-wide.  No counterpart in the
 * reference, which fixes the core at compile time (CoreFunc.h:35-39). */
int32_t o3g_external_set_method(int32_t core, int32_t prec);
/* The core and precision the float hook would use now. */
int32_t o3g_external_get_method(int32_t* core, int32_t* prec);

/* ---- surfaces ---------------------------------------------------------------------
 * A triangulated surface in the reference's Surfaces<S> layout (Surfaces.h:1463-1489):
 * node positions, three node indices per panel (Int = uint32_t, Omega3D.h:26), panel
 * areas and the per-panel basis x1 (edge 0->1), x2 (in-plane, toward node 2) and normal. */
typedef struct {
  int32_t nn;
  const float *x, *y, *z;
  int32_t np;
  const uint32_t* idx;
  const float* area;
  const float *x1x, *x1y, *x1z;
  const float *x2x, *x2y, *x2z;
  const float *nx, *ny, *nz;
} o3g_surface_t;

/* Node/panel counts of an icosahedral sphere refined `levels` times: 10*4^L+2, 20*4^L. */
int32_t o3g_ovoid_size(int32_t levels, int32_t* num_nodes, int32_t* num_panels);
/* generate_ovoid, GeomHelper.cpp:41-91 with igl::upsample numbering
 * (lib/igl/upsample.cpp:17-105): icosahedron of radius 0.5 refined `levels` times,
 * re-projected to r = 0.5 after each level, then scaled by (rx, ry, rz).  Host arrays. */
int32_t o3g_generate_ovoid(int32_t levels, float rx, float ry, float rz, float* x, float* y, float* z,
                           uint32_t* idx);
/* Surfaces::compute_bases, Surfaces.h:776-816 (host arrays). */
int32_t o3g_compute_bases(int32_t nn, const float* x, const float* y, const float* z, int32_t np,
                          const uint32_t* idx, float* x1x, float* x1y, float* x1z, float* x2x, float* x2y,
                          float* x2z, float* nx, float* ny, float* nz, float* area);
/* Surfaces::vortex_sheet_to_panel_strength, Surfaces.h:309-335: ts = (ps0 x1 + ps1 x2) area. */
int32_t o3g_sheet_to_panel_strength(int32_t np, const float* ps0, const float* ps1, const float* x1x,
                                    const float* x1y, const float* x1z, const float* x2x, const float* x2y,
                                    const float* x2z, const float* area, float* tsx, float* tsy, float* tsz);

/* ---- panels_affect_points ----------------------------------------------------------
 * Replaces panels_affect_points<float,A>, Influence.h:557-1099 (rkernel_2vs_0pg / _0p,
 * Kernels.h:1028-1211): velocity (+ gradient when tug != NULL) at nt points induced by np
 * flat vortex(+source) panels, adaptively subdivided down to maxlev levels (the reference
 * uses RECURSIVE_LEVELS = 3, Influence.h:23; accepted 0..6).  ts = absolute panel vortex
 * strengths (Surfaces::get_str); sss = source sheet strengths or NULL.  The targets' core
 * radii are not used (Influence.h:872-873).  Accumulates (+=).  prec PLAIN (FP32 sums, the
 * reference's arithmetic) or COMPENSATED (Newton-refined rsqrt, two-sum accumulators folded
 * per tile of 128 panels, partial sums added in double). */
int32_t o3g_panels_affect_points(int32_t prec, int32_t mem, int32_t maxlev,
                                 int32_t nn, const float* nx, const float* ny, const float* nz,
                                 int32_t np, const uint32_t* idx, const float* area,
                                 const float* tsx, const float* tsy, const float* tsz, const float* sss,
                                 int32_t nt, const float* tx, const float* ty, const float* tz,
                                 float* tu, float* tv, float* tw, float* const* tug, void* stream);

/* ---- panels_affect_panels ----------------------------------------------------------
 * Replaces panels_affect_panels<float,A>, Influence.h:1223-1243: the velocity the np source
 * panels induce at the tnp target panels' collocation points (centroid pushed 0.0001 along
 * the target normal, as Surfaces::represent_as_particles(0.0001, ...) places them), computed
 * like o3g_panels_affect_points (velocity only) and WRITTEN into tu, tv, tw: the reference
 * copies the result over the target's panel velocities instead of accumulating. */
int32_t o3g_panels_affect_panels(int32_t prec, int32_t mem, int32_t maxlev,
                                 int32_t nn, const float* nx, const float* ny, const float* nz,
                                 int32_t np, const uint32_t* idx, const float* area,
                                 const float* tsx, const float* tsy, const float* tsz, const float* sss,
                                 int32_t tnn, const float* tnx, const float* tny, const float* tnz,
                                 int32_t tnp, const uint32_t* tidx, const float* tnormx, const float* tnormy,
                                 const float* tnormz, float* tu, float* tv, float* tw, void* stream);

/* ---- points_affect_panels ----------------------------------------------------------
 * Replaces points_affect_panels<float,A>, Influence.h:1107-1221: panel-averaged velocity
 * induced by ns vortex particles on np panels (the BEM right-hand side), computed like the
 * reference by subdividing the target panel as a source carrying the particle's strength
 * and SUBTRACTING the result (Influence.h:1209-1212).  Particle core radii are not used.
 * prec PLAIN or COMPENSATED as for o3g_panels_affect_points (tiles of 128 particles). */
int32_t o3g_points_affect_panels(int32_t prec, int32_t mem, int32_t maxlev,
                                 int32_t ns, const float* sx, const float* sy, const float* sz,
                                 const float* ssx, const float* ssy, const float* ssz,
                                 int32_t nn, const float* nx, const float* ny, const float* nz,
                                 int32_t np, const uint32_t* idx, const float* area,
                                 float* pu, float* pv, float* pw, void* stream);

/* ---- panels_on_panels_coeff ----------------------------------------------------------
 * Replaces panels_on_panels_coeff<float>, Coefficients.h:169-447: the (targ->np*nunk) x
 * (src->np*nunk) influence block, column-major with leading dimension ld, into `coeffs`
 * (device memory; all surface arrays device memory).  nunk 2 = tangential vortex sheet
 * unknowns, 3 = plus the source sheet (Surfaces.h:71,261).  is_self writes the
 * self-influence diagonal (Coefficients.h:414-436).  maxlev 0..4 (reference: 3). */
int32_t o3g_panels_on_panels_coeff(int32_t maxlev, int32_t nunk, int32_t is_self, const o3g_surface_t* src,
                                   const o3g_surface_t* targ, float* coeffs, int64_t ld, void* stream);

/* ---- BEM system ------------------------------------------------------------------------
 * Replaces BEM<S,I> (BEM.h:44-234).  The handle owns the device-resident n x n FP32 matrix
 * (column-major, leading dimension from o3g_bem_matrix), its LU factors and scratch.
 * The reference solves with Eigen GMRES (BEM.h:182-202).  Here either the matrix is
 * factorised in FP32 with partial pivoting and TF32 tensor-core trailing updates and
 * solutions are refined with FP64-accurate residuals b - A x (o3g_bem_factor +
 * o3g_bem_solve), or GMRES runs on the unfactored matrix (o3g_bem_solve_gmres); both stop
 * at ||r||/||b|| <= tol, the residual the reference prints (BEM.h:227-230). */
typedef struct o3g_bem o3g_bem_t;
/* number of unknowns of the system */
int32_t o3g_bem_size(const o3g_bem_t* h, int64_t* n);
/* allocates the handle and ~2 n^2 floats of device memory (n <= 200000; the panel
 * factorisation needs n <= ~68000 on 152 SMs) */
int32_t o3g_bem_create(int64_t n, o3g_bem_t** h);
int32_t o3g_bem_destroy(o3g_bem_t* h);
/* device pointer and leading dimension of the matrix, e.g. to assemble blocks in place with
 * o3g_panels_on_panels_coeff(..., A + cstart*ld + rstart, ld, ...); marks A as changed */
int32_t o3g_bem_matrix(o3g_bem_t* h, float** A, int64_t* ld);
/* BEM::set_block, BEM.h:116-136: copy a column-major nrows x ncols block into A */
int32_t o3g_bem_set_block(o3g_bem_t* h, int64_t rstart, int64_t nrows, int64_t cstart, int64_t ncols,
                          const float* blk, int32_t mem, void* stream);
/* LU factorisation of the current A (BEM.h:184-195's solver.compute) */
int32_t o3g_bem_factor(o3g_bem_t* h, void* stream);
/* solve A x = b (BEM.h:202): b, x (float) and x64 (double, nullable) in `mem` memory;
 * returns the refinement count and the final FP64 relative residual; O3G_ERR_NOT_CONVERGED
 * when tol is not reached within max_iter refinements (x still holds the best iterate) */
int32_t o3g_bem_solve(o3g_bem_t* h, const float* b, float* x, double* x64, int32_t mem, double tol,
                      int32_t max_iter, int32_t* iters, double* relres, void* stream);
/* solve A x = b without factorising: restarted GMRES(restart), the reference's own method
 * (Eigen GMRES, BEM.h:182-202), with FP64 Krylov vectors and FP64-accurate products of the
 * FP32 matrix, until ||b - A x|| / ||b|| <= tol (checked on the true residual at every
 * restart) or max_iter iterations; arguments otherwise as o3g_bem_solve.  Needs only the
 * assembled matrix (o3g_bem_matrix / o3g_bem_set_block). */
int32_t o3g_bem_solve_gmres(o3g_bem_t* h, const float* b, float* x, double* x64, int32_t mem, double tol,
                            int32_t max_iter, int32_t restart, int32_t* iters, double* relres, void* stream);
/* unknowns per panel (1..3, dividing n; default 1) of the assembled system: the GMRES solves
 * (o3g_bem_solve_gmres, o3g_bem_solve_gmres_many) then precondition with the inverses of the
 * bs x bs diagonal blocks, a panel's self-influence (Coefficients.h:414-436), applied on the
 * right so that the residual stays ||b - A x||.  The reference's Eigen GMRES uses a diagonal
 * preconditioner (BEM.h:182-202); with 1 nothing changes (the vortex rows' diagonal is 0,
 * where a diagonal preconditioner is the identity). */
int32_t o3g_bem_set_unknowns_per_panel(o3g_bem_t* h, int32_t bs);
/* Several right-hand sides at once: B holds nrhs vectors of n floats back to back (column c
 * at B + c n, an n x nrhs column-major block), X (float) and X64 (double, nullable) the
 * solutions in the same layout, iters and relres (nullable) nrhs entries.  Each refinement
 * sweep (o3g_bem_solve_many, after o3g_bem_factor) or GMRES iteration
 * (o3g_bem_solve_gmres_many, restart as for o3g_bem_solve_gmres) streams the matrix once for
 * up to 8 right-hand sides, where o3g_bem_solve / o3g_bem_solve_gmres stream it once per
 * right-hand side; larger nrhs go in groups of 8.  Every column is solved as by the
 * single-vector entry points (refinements or GMRES iterations counted per column, converged
 * columns frozen) until ||b_c - A x_c|| / ||b_c|| <= tol.  The reference solves one b per
 * BEM::solve (BEM.h:200-203) and solves again per RK stage (Convection.h:197) and per
 * diffusion step (Diffusion.h:184-187); these take all of those right-hand sides in one call.
 * O3G_ERR_NOT_CONVERGED when any column misses tol (its relres says which). */
int32_t o3g_bem_solve_many(o3g_bem_t* h, int32_t nrhs, const float* B, float* X, double* X64, int32_t mem,
                           double tol, int32_t max_iter, int32_t* iters, double* relres, void* stream);
int32_t o3g_bem_solve_gmres_many(o3g_bem_t* h, int32_t nrhs, const float* B, float* X, double* X64, int32_t mem,
                                 double tol, int32_t max_iter, int32_t restart, int32_t* iters, double* relres,
                                 void* stream);
/* finalize_vels of panel velocities (u = fs + u/(4 pi), ElementBase.h:187-193) and
 * vels_to_rhs_panels (RHS.h:92-110) in one pass; device arrays; rhs has np*nunk entries */
int32_t o3g_panel_vels_to_rhs(int32_t np, int32_t nunk, const double* fs, float* pu, float* pv, float* pw,
                              const o3g_surface_t* surf, float* rhs, void* stream);

/* ---- convection: finalize_vels, moves, Ralston RK2 ------------------------------------------
 * Device arrays; u/s/x are arrays of 3 component pointers, ug of 9.  The element-wise
 * kernels reproduce the reference's float/double arithmetic exactly. */
/* finalize_vels, ElementBase.h:187-193 + Points.h:265-277: u = fs + u/(4 pi), ug *= 1/(4 pi) */
int32_t o3g_points_finalize(int32_t n, const double* fs, float* const* u, float* const* ug, void* stream);
/* Points::move first order, ElementBase.h:253-273 + Points.h:288-351: x += dt*wt1*u and, when
 * s, elong and ug are given, vortex stretching of s and elong */
int32_t o3g_points_move_euler(int32_t n, double dt, double wt1, float* const* x, float* const* s, float* elong,
                              float* const* u, float* const* ug, void* stream);
/* Points::move second order, ElementBase.h:276-304 + Points.h:356-439: u1 <- wt1 u1 + wt2 u2,
 * x += dt u1, stretching with wt1 ug1 + wt2 ug2 applied to the stage-0 strengths */
int32_t o3g_points_move_rk2(int32_t n, double dt, double wt1, float* const* u1, float* const* ug1, double wt2,
                            float* const* u2, float* const* ug2, float* const* x, float* const* s, float* elong,
                            void* stream);
/* Convection::advect_2nd_ralston (Convection.h:349-425) for a boundary-free set of n vortex
 * particles (x, s, r, elong: the caller's device arrays, advanced in place) and nf field points
 * (fx, may be 0): per step two vel+grad evaluations (core, prec PLAIN or COMPENSATED), the
 * 2/3 dt interim move and the 0.25/0.75 combine.  With use_graph != 0 the first step runs
 * directly and the step is then captured into a CUDA graph and replayed (stream must then be
 * a non-default stream).  o3g_rk2_velocities gives the velocities the last step moved the
 * particles with (0.25 u1 + 0.75 u2, Points.h:356-439) and its stage-1 gradients. */
typedef struct o3g_rk2 o3g_rk2_t;
int32_t o3g_rk2_create(int32_t core, int32_t prec, int32_t n, float* const* x, float* const* s, float* r,
                       float* elong, int32_t nf, float* const* fx, int32_t use_graph, o3g_rk2_t** h);
int32_t o3g_rk2_step(o3g_rk2_t* h, double dt, const double* fs, int32_t nsteps, void* stream);
int32_t o3g_rk2_velocities(o3g_rk2_t* h, float** u, float** ug);
int32_t o3g_rk2_destroy(o3g_rk2_t* h);
/* Adds one fixed body (Surfaces, device arrays) to a single-system RK2 handle: every stage
 * then first solves the BEM for that stage's particles -- solve_bem, BEMHelper.h:43-265:
 * panel velocities from the particles (o3g_points_affect_panels), freestream, RHS.h's
 * vels_to_rhs, the refined solve, Surfaces::set_str (Surfaces.h:267-335) -- and adds the
 * panels' velocity and gradient (o3g_panels_affect_points) to the particles' and field
 * points' sums before finalize_vels, as Convection::find_vels does (Convection.h:131-182).
 * The matrix (nunk unknowns per panel, subdivision maxlev) is assembled into `bem` and
 * factorised here, once: the body does not move.  The pair and panel sums use the handle's
 * precision.  With ips > 0, particles and field points are pushed out of the body after the
 * interim move and after the combine (clear_inner_layer method 1 with cutoff 0.5/sqrt(2 pi)
 * * ips, Convection.h:372,381,423-424); ips = 0 skips that.  Steps with a body run
 * directly (the solves' convergence checks read the residual on the host), not from a graph. */
int32_t o3g_rk2_attach_body(o3g_rk2_t* h, const o3g_surface_t* surf, int32_t nunk, int32_t maxlev, o3g_bem_t* bem,
                            double tol, int32_t max_iter, float ips, void* stream);
/* Solve statistics of the attached body: number of solves, refinements and relative residual
 * of the last one, the largest final residual over all solves, and the number of points
 * pushed out of the body so far (synchronises the device when `pushed` is given). */
int32_t o3g_rk2_body_stats(const o3g_rk2_t* h, int64_t* solves, int32_t* last_iters, double* last_relres,
                           double* max_relres, int64_t* pushed);
/* Copies the body's panel strengths ts[3] (np each) and BEM solution (np * nunk) of the last
 * stage solved into the caller's arrays (host or device; either may be NULL) and waits. */
int32_t o3g_rk2_body_strengths(const o3g_rk2_t* h, float* const* ts, float* solution, void* stream);

/* ---- many independent particle systems in one launch ----------------------------------
 * No counterpart in the reference, which runs points_affect_points once per (source
 * collection, target collection) pair (Convection.h:144-172).  Each system's particles are
 * the sources and the thick-cored targets of that system only; its field points are
 * further targets (no radius).  Sums ACCUMULATE (+=) like o3g_points_affect_points.
 * All arrays are device arrays.  precision PLAIN or COMPENSATED; grads != 0 needs ug (and
 * fug when nf > 0); grads == 0 computes velocities only. */
typedef struct {
  int32_t np;                        /* particles                                           */
  const float *x, *y, *z, *r;        /* positions and core radii                            */
  const float *sx, *sy, *sz;         /* strengths                                           */
  float *u, *v, *w;                  /* particle velocity sums (+=)                         */
  float* ug[9];                      /* particle gradient sums (+=)                         */
  int32_t nf;                        /* field points (may be 0)                             */
  const float *fx, *fy, *fz;
  float *fu, *fv, *fw;
  float* fug[9];
} o3g_system_t;

/* The batch handle: packed copies of the systems (Morton-ordered per system for the
 * Gaussian and exponential cores), a plan of (target block, source-tile range) work items
 * drained by ONE persistent kernel launch, and its tuned configuration.  The descriptor
 * pointers are fixed at creation; their contents may change between runs. */
typedef struct o3g_batch o3g_batch_t;
int32_t o3g_batch_create(int32_t core, int32_t prec, int32_t grads, int32_t nsys, const o3g_system_t* systems,
                         o3g_batch_t** h);
/* Queues one evaluation on `stream`.  When the shape -- (core, precision, grads, SM count,
 * every system's (np, nf)) -- has no cached configuration and the stream is not capturing,
 * the first run first times the candidate configurations (targets per thread, work-item
 * size, blocks per SM) on this data, caches the fastest (in the process and in the text
 * file $O3G_TUNE_CACHE, default ~/.cache/o3dgpu/batch_tune.txt) and synchronises the
 * stream.  O3G_BATCH_TUNE=0 disables tuning.  Capturable into a graph once tuned. */
int32_t o3g_batch_run(o3g_batch_t* h, void* stream);
/* Retunes now (synchronous). */
int32_t o3g_batch_tune(o3g_batch_t* h, void* stream);
/* Forces a configuration: tpt in {1, 2, 4} ({1, 2} for compensated with gradients),
 * blocks_per_sm (0 = full occupancy), split in {0, 4, 16}.  Synchronises the device. */
int32_t o3g_batch_set_config(o3g_batch_t* h, int32_t tpt, int32_t blocks_per_sm, int32_t split);
/* Current configuration: targets per thread, grid size (blocks), split, largest item in
 * source tiles, number of work items, and whether it was tuned (or set / cached). */
int32_t o3g_batch_get_config(const o3g_batch_t* h, int32_t* tpt, int32_t* grid, int32_t* split, int32_t* chunk,
                             int32_t* nitems, int32_t* tuned);
int32_t o3g_batch_destroy(o3g_batch_t* h);
/* One-shot: create, run, synchronise `stream`, destroy. */
int32_t o3g_batch_velgrad(int32_t core, int32_t prec, int32_t grads, int32_t nsys, const o3g_system_t* systems,
                          void* stream);
/* Host only (no device needed): the work-item plan for per-system counts np, nf at tpt
 * targets per thread, `grid` resident blocks and `split`: counts of items and target blocks,
 * the largest item in source tiles and the partial-sum slabs.  When not NULL, items receives
 * {target block, first tile, end tile, split index} and tbs {system, first target slot,
 * first slab or -1, number of splits}, 4 int32 each, items longest first. */
int32_t o3g_batch_plan(int32_t nsys, const int32_t* np, const int32_t* nf, int32_t tpt, int32_t grid, int32_t split,
                       int32_t* nitems, int32_t* ntbs, int32_t* chunk, int64_t* nslabs, int32_t* items,
                       int32_t* tbs);
/* Ralston RK2 (as o3g_rk2_create) of nsys independent systems stored back to back in the
 * device arrays x, s, r, elong (system i: particles [P_i, P_i + np[i]), P_i = sum of the
 * earlier np) and fx (field points, likewise by nf).  Both velocity evaluations of a step
 * are one batched persistent launch each.  Step, read and destroy with o3g_rk2_step,
 * o3g_rk2_velocities, o3g_rk2_destroy. */
int32_t o3g_batch_rk2_create(int32_t core, int32_t prec, int32_t nsys, const int32_t* np, const int32_t* nf,
                             float* const* x, float* const* s, float* r, float* elong, float* const* fx,
                             int32_t use_graph, o3g_rk2_t** h);

/* ---- shedding ------------------------------------------------------------------------------
 * Replaces Surfaces::represent_as_particles (Surfaces.h:959-1008), which diffusion calls after
 * its solve_bem (Diffusion.h:187-224): particle i at the centroid of panel i pushed `offset`
 * along the normal, with strength ts_i, plus (bc1 x1 + bc2 x2) area when bc1 and bc2 (the
 * reactive boundary-condition values) are given.  Device arrays; np particles out; the
 * positions and strengths are bit-identical to the reference's float arithmetic. */
int32_t o3g_represent_as_particles(const o3g_surface_t* surf, float offset, const float* tsx, const float* tsy,
                                   const float* tsz, const float* bc1, const float* bc2, float* px, float* py,
                                   float* pz, float* sx, float* sy, float* sz, void* stream);

/* ---- clear_inner_layer ------------------------------------------------------------------
 * Replaces clear_inner_panp2 method 1 (Reflect.h:446-656): every one of the n points (device
 * arrays x, y, z, moved in place) whose height above its closest panels -- the mean normal
 * and mean contact point of every panel within 10 float epsilon of the closest squared
 * distance (Reflect.h:56-183 per panel) -- is below cutoff_mult * ips is pushed out to that
 * height along the mean normal.  surf: device arrays with nodes, idx and normals.  The
 * positions are bit-identical to the reference's float arithmetic.  With npushed given the
 * call waits and returns the number pushed; otherwise it is asynchronous. */
int32_t o3g_clear_inner_layer(int32_t n, float* x, float* y, float* z, const o3g_surface_t* surf, float cutoff_mult,
                              float ips, int32_t* npushed, void* stream);

/* ---- particle split and merge --------------------------------------------------------
 * Replaces split_elongated<float> (Split.h:44-270; called after every step by
 * split_operation, Simulation.cpp:833): every particle with elong > threshold is split in
 * two along its strength direction, half the strength each, with the reference's
 * curvature correction from its neighbours within 3 r / overlap (weights from core_func,
 * O3G_DIFFCORE_*).  Device arrays of `capacity` particles; the split ones are updated in
 * place and their children appended at [n, n + nsplit) in index order.  When capacity is
 * below n + nsplit nothing is changed, *nsplit is set and O3G_ERR_CAPACITY returned.
 * Waits for the result.  Bit-identical to the reference's sequential loop, except where two
 * neighbours of a split particle are at exactly equal distance (visited here in index
 * order, by the reference in its kd-tree's order). */
int32_t o3g_split_elongated(int32_t n, int32_t capacity, float* x, float* y, float* z, float* r, float* elong,
                            float* sx, float* sy, float* sz, int32_t core_func, float particle_overlap,
                            float threshold, int32_t* nsplit, void* stream);

/* Replaces merge_close_particles<float> (Merge.h:45-218; called by merge_operation in
 * diffusion, Diffusion.h:298,355): in index order, each surviving particle absorbs the
 * surviving neighbours closer than half a nominal separation (r / overlap) whose merge error
 * is below threshold (relative to the mean strength) or that are closer than a tenth of it;
 * absorbed particles are removed and the survivors compacted in place, in order, to
 * n - nremoved.  adapt_radii: merged radii follow the reference's volume rule.  Waits for the
 * result.  Bit-identical to the reference's sequential loop (ties in distance as above). */
int32_t o3g_merge_close_particles(int32_t n, float* x, float* y, float* z, float* sx, float* sy, float* sz,
                                  float* r, float particle_overlap, float threshold, int32_t adapt_radii,
                                  int32_t* nremoved, void* stream);

/* ---- points_affect_points without device allocation ------------------------------
 * No counterpart in the reference.  For callers that may not allocate device memory
 * after start-up (applications that give all device memory to their own pool, real-time
 * loops that cannot absorb an allocation or the synchronisation of cudaFree, plugin
 * hosts that forbid allocation): the same sums as o3g_points_affect_points on
 * device-resident arrays (mem is always device; prec PLAIN or COMPENSATED), with every
 * scratch byte taken from one fixed 64 MiB array in the library's device image.
 *  - The first call on a device resolves that array's address (cudaGetSymbolAddress);
 *    make it before capturing a stream into a graph.  The address is looked up again
 *    when the device's context changes (e.g. after cudaDeviceReset).
 *  - All calls share the array: calls that overlap on the GPU race; use one stream.
 *  - Problems whose packed tiles do not fit (about 1.3 million sources + targets) return
 *    O3G_ERR_INVALID_ARG before any work is queued.
 * Sources are not Morton-sorted: the Gaussian and exponential cores still test each
 * source tile against each warp's targets, but with unsorted points the test almost
 * never finds a far tile, so nearly every pair takes the full core. */
int32_t o3g_points_affect_points_noalloc(int32_t core, int32_t prec,
                                         int32_t ns, const float* sx, const float* sy, const float* sz,
                                         const float* sr, const float* ssx, const float* ssy, const float* ssz,
                                         int32_t nt, const float* tx, const float* ty, const float* tz,
                                         const float* tr,
                                         float* tu, float* tv, float* tw, float* const* tug,
                                         void* stream);

#ifdef __cplusplus
}
#endif
#endif /* O3DGPU_H */
