/*
 * lxgb.h — C ABI of the GB300 (sm_103a) solve engine behind lineax's solver API.
 *
 * Every entry point is stream-ordered and returns an lxgb_status.  The caller
 * owns every device buffer; the library keeps no pointer after a call returns.
 * Scratch memory is sized by the matching *_workspace_size call and allocated
 * by the caller.  Matrices are row-major (the JAX default layout); a batch of
 * equal-size matrices is addressed by a base pointer plus an element stride,
 * a ragged batch by a per-system offset array into one packed buffer.
 * Right-hand sides of one system are stored as nrhs contiguous vectors of
 * length n (the layout of a vmapped `(nrhs, n)` JAX array).
 *
 * Pivots are 0-based swap indices as returned by jax.scipy.linalg.lu_factor:
 * row k was interchanged with row piv[k] during step k.
 *
 * `stream` is a cudaStream_t passed as void* so that the header needs no CUDA
 * include; 0 means the legacy default stream.
 */
#ifndef LXGB_H_
#define LXGB_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  0..6 equal the indices of lineax.RESULTS
 * (lineax/_solution.py:52-68, declaration order of the eqxi.Enumeration), so
 * the Python layer maps a status to a RESULTS member without a table.  Codes
 * >= 100 are argument or runtime errors that lineax raises as exceptions. */
typedef enum lxgb_status {
  LXGB_SUCCESSFUL = 0,
  LXGB_MAX_STEPS_REACHED = 1,
  LXGB_SINGULAR = 2,
  LXGB_BREAKDOWN = 3,
  LXGB_STAGNATION = 4,
  LXGB_CONLIM = 5,
  LXGB_NONFINITE_INPUT = 6,
  LXGB_INVALID_ARG = 100,
  LXGB_CUDA_ERROR = 101,
  LXGB_NOT_SUPPORTED = 102,
  LXGB_TIMEOUT = 103,
  LXGB_WORKSPACE_TOO_SMALL = 104
} lxgb_status;

/* Library version (major*10000 + minor*100 + patch). */
int lxgb_version(void);
/* Human-readable text for a status code. */
const char* lxgb_status_string(int status);
/* Text of the last failure on the calling thread ("" if none). */
const char* lxgb_last_error(void);

/* ------------------------------------------------------------------------ */
/* LU with partial pivoting.                                                 */
/* ------------------------------------------------------------------------ */

/* In-place P·A = L·U of `batch` row-major n×n FP64 matrices (unit-lower L
 * below the diagonal, U on and above it), A_b at a + b*stride_a.  piv_b at
 * piv + b*stride_piv receives n 0-based swap indices; info[b] = 0 on success
 * or k+1 for the first exactly-zero pivot k (LAPACK getrf convention; the
 * factorisation still completes).  The pivot search returns the first row of
 * maximal |a| (LAPACK idamax).
 * Replaces jax.scipy.linalg.lu_factor at lineax/_solver/lu.py:53 (vmapped). */
int lxgb_getrf_batched_f64(int64_t batch, int32_t n, double* a, int64_t stride_a,
                           int32_t* piv, int64_t stride_piv, int32_t* info,
                           void* stream);

/* Kernel choice of lxgb_getrf_batched_f64 for 32 <= n <= 168 (a tuning
 * switch, process-wide; factors, pivots and info are bit-identical either
 * way): 1 factors each matrix on a cluster of two CTAs (columns split by
 * parity, multipliers exchanged through distributed shared memory, one
 * cluster barrier per column) when 2 * batch <= the SM count, so that small
 * batches occupy twice as many SMs; 0 (the default) uses one CTA per matrix,
 * whose pivot search for column k+1 overlaps the update of step k — faster on
 * GB300, where the per-column cluster barrier costs more than the halved FP64
 * work saves (0.33 ms against 0.44 ms for 64 matrices of order 128). */
int lxgb_getrf_set_pair(int32_t on);

/* Solve A_b X = B_b (trans = 0) or A_bᵀ X = B_b (trans = 1) in place on B
 * with the factor from lxgb_getrf_batched_f64.  B_b holds nrhs vectors of
 * length n at b + b*stride_b (vector r at offset r*n).
 * Replaces jax.scipy.linalg.lu_solve(..., trans) at lineax/_solver/lu.py:64;
 * trans = 1 serves LU.transpose (lineax/_solver/lu.py:68-81). */
int lxgb_getrs_batched_f64(int64_t batch, int32_t n, int32_t nrhs,
                           const double* lu, int64_t stride_a,
                           const int32_t* piv, int64_t stride_piv, double* b,
                           int64_t stride_b, int32_t trans, void* stream);

/* ------------------------------------------------------------------------ */
/* Cholesky (upper factor, A = Uᵀ U), ragged batches.                        */
/* ------------------------------------------------------------------------ */

/* In-place upper Cholesky of a ragged batch of row-major symmetric FP64
 * matrices: system s has order n[s] <= max_n and starts at a + a_off[s]
 * (n and a_off are device arrays; max_n is a host value that sizes shared
 * memory).  Only the upper triangle is read; on return it holds U with
 * A = Uᵀ U and the strictly lower triangle is zero (the output layout of
 * jax.scipy.linalg.cho_factor(lower=False)).  info[s] = 0, or k+1 when the
 * leading minor of order k+1 is not positive definite (LAPACK potrf), or -2
 * when n[s] > max_n; a failed system's factor is unspecified.
 * CTAs take the systems round-robin (system s by CTA s mod grid), so placing
 * the largest first balances the launch.
 * Replaces jax.scipy.linalg.cho_factor(lower=False) at
 * lineax/_solver/cholesky.py:60. */
int lxgb_potrf_ragged_f64(int64_t batch, int32_t max_n, const int32_t* n,
                          const int64_t* a_off, double* a, int32_t* info,
                          void* stream);

/* Upper Cholesky A = Uᵀ U of one n×n SPD matrix (row stride lda), in place,
 * on many CTAs: 64-row block rows, the diagonal block by one CTA, the block
 * row by column-parallel substitution, the trailing matrix by
 * lxgb_syrk_f64's update.  Every element receives the same FMA chain as in
 * lxgb_potrf_ragged_f64, so the two return the same bits; the strictly lower
 * triangle is zeroed.  *info (device) = 0, or k+1 for the first pivot that is
 * not positive (the factor is then unspecified).  Replaces
 * jax.scipy.linalg.cho_factor(lower=False) at lineax/_solver/cholesky.py:60
 * for one large matrix. */
int lxgb_potrf_f64(int64_t n, double* a, int64_t lda, int32_t* info,
                   void* stream);

/* Symmetric rank-k product, FP64, on the upper triangle of the n×n C (row
 * stride ldc): S = AᵀA (trans 0, A k×n) or S = AAᵀ (trans 1, A n×k), A
 * row-major with row stride lda.  update 0: C = S, and with fill = 1 the
 * lower triangle receives the mirror (a full symmetric Gram matrix, the
 * materialised normal-equations operator of lineax/_solver/normal.py:112-118);
 * update 1: C -= S on j >= i, each element continuing its FMA chain from its
 * stored value in k order (the Cholesky trailing update).  fill requires
 * update 0. */
int lxgb_syrk_f64(int32_t trans, int64_t n, int64_t k, const double* a,
                  int64_t lda, int32_t update, double* c, int64_t ldc,
                  int32_t fill, void* stream);

/* Solve (Uᵀ U) X = B in place on B for each system of a ragged batch; system
 * s has nrhs[s] vectors of length n[s] starting at b + b_off[s].
 * Replaces jax.scipy.linalg.cho_solve at lineax/_solver/cholesky.py:74. */
int lxgb_potrs_ragged_f64(int64_t batch, int32_t max_n, const int32_t* n,
                          const int32_t* nrhs, const int64_t* a_off,
                          const double* u, const int64_t* b_off, double* b,
                          void* stream);

/* Mixed-precision SPD solve of a ragged batch: the factor is computed in FP32
 * from the FP64 matrix (upper triangle read), then FP64 iterative refinement
 * (residual r = b - A x in FP64, correction solved with the FP32 factor, x
 * accumulated in FP64) runs until the normwise backward error
 *     ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf)
 * of every right-hand side is <= tol, or max_iter corrections were applied.
 * A and B are read only; X receives the solutions (layout of B).  Per system:
 * info[s] = 0, k+1 if the FP32 factor broke down at k, -1 if refinement did
 * not reach tol, -2 if n[s] > max_n or nrhs[s] > max_nrhs; iters[s] = number
 * of FP32 solves applied (1 = the initial solve alone); berr[s] = largest
 * backward error over its right-hand sides.
 * `work` must hold lxgb_posv_ragged_mixed_workspace_size(batch, max_n,
 * max_nrhs) bytes, 256-byte aligned; its contents need no initialisation.
 * One persistent launch solves the batch; its CTAs take systems largest n
 * first (a counting sort by n runs ahead of it), so the launch does not end
 * on a tail of large systems started last.
 * This is the batched form of lineax's Cholesky solve
 * (lineax/_solver/cholesky.py:43-78) with FP64 accuracy recovered by
 * refinement; it has no single-call counterpart in lineax. */
int64_t lxgb_posv_ragged_mixed_workspace_size(int64_t batch, int32_t max_n,
                                              int32_t max_nrhs);
int lxgb_posv_ragged_mixed(int64_t batch, int32_t max_n, int32_t max_nrhs,
                           const int32_t* n, const int32_t* nrhs,
                           const int64_t* a_off, const double* a,
                           const int64_t* b_off, const double* b, double* x,
                           double tol, int32_t max_iter, int32_t* info,
                           int32_t* iters, double* berr, void* work,
                           int64_t work_bytes, void* stream);

/* lxgb_posv_ragged_mixed with the FP32 factors kept between calls: the
 * factor state a lineax solver returns from `init` and reuses in every
 * `compute` (lineax/_solve.py:785-790 — linear_solve skips init when a state
 * is passed; lineax/_solver/cholesky.py:43-62 is the state).  fmode[s]
 * (device int32) selects per system: 0 factor A and keep nothing, 1 factor A
 * and store the factor at factors[s], 2 skip the factorisation and use the
 * factor stored at factors[s] (A is still read by the refinement residual).
 * `factors` is a device array of `batch` device pointers (entries of systems
 * with fmode 0 are not read), each to n[s]² FP32 (row-major, upper triangle,
 * lower zeroed).  A stored factor is the one a fresh factorisation makes, so
 * results are bit-identical with and without reuse.  Other arguments and the
 * workspace as for lxgb_posv_ragged_mixed. */
int lxgb_posv_ragged_mixed_factors(int64_t batch, int32_t max_n, int32_t max_nrhs,
                                   const int32_t* n, const int32_t* nrhs,
                                   const int64_t* a_off, const double* a,
                                   const int64_t* b_off, const double* b, double* x,
                                   double tol, int32_t max_iter, int32_t* info,
                                   int32_t* iters, double* berr, const int32_t* fmode,
                                   float* const* factors, void* work, int64_t work_bytes,
                                   void* stream);

/* Tuning table of the mixed solve (no counterpart in the reference): the
 * largest order whose FP32 factor is formed in shared memory; larger systems
 * use a per-CTA slice of the workspace (through L2).  0 <= small_max <= 144,
 * default 144.  The host sets it once at initialisation from its autotune
 * table (lineax_gb300/autotune.py, per GPU model), before solves are issued;
 * lxgb_posv_ragged_mixed_workspace_size follows the current value, and each
 * solve call reads it once. */
int lxgb_posv_mixed_set_small_max(int32_t small_max);
int32_t lxgb_posv_mixed_small_max(void);

/* Second tuning switch of the mixed solve (no counterpart in the reference):
 * on = 1 runs the trailing updates of the factor of systems above small_max
 * (up to order 544) on the tcgen05 tensor cores (split TF32 products,
 * FP32-level accuracy), on = 0 (default) on the CUDA cores.  Set at
 * initialisation, like small_max.  A tensor-core completion wait that times
 * out abandons that system with info[s] = -3 and the kernel goes on. */
int lxgb_posv_mixed_set_tensor_cores(int32_t on);

/* Allocation-free form of lxgb_posv_ragged_mixed (no counterpart in the
 * reference).  It is for callers that cannot allocate device memory when they
 * solve — an XLA/JAX FFI handler, whose device memory belongs to XLA and where
 * a cudaMalloc can synchronise the device or break a graph capture, or a
 * serving / real-time loop that forbids allocation after start-up.  Arguments
 * and results are those of lxgb_posv_ragged_mixed without `work`: the scratch
 * is a fixed array of LXGB_POSV_NOALLOC_SCRATCH_BYTES (16 MiB + 256 B) inside
 * the library, which every GPU that loads the library holds until the process
 * exits.  Limits: max_n <= 1024 (larger is rejected with LXGB_INVALID_ARG).
 * When max_n > 144 (the largest order factored in shared memory) every CTA of
 * the launch needs one FP32 factor slice of 4·ld² bytes (ld = max_n rounded up
 * to a multiple of 32) in the array, so the WHOLE launch, small systems
 * included, runs on 16 MiB / (4·ld²) CTAs instead of two per SM: 16 CTAs at
 * max_n = 512, 4 at max_n = 1024.  Callers with mostly small systems should
 * pass their large systems in a separate call.  With max_n <= 144 no slice is
 * needed and the grid is the workspace form's.  Systems are taken longest
 * first when the slices leave room for the order (4 bytes per system), else
 * in index order.
 * The first call on each device looks up the array's device address
 * (cudaGetSymbolAddress); make that first call before any stream capture.
 * Every call uses the same array and leaves its contents behind (the call
 * clears the work-queue counter itself): calls that overlap on the GPU — on
 * two streams, or from two threads — race and must be serialised by the
 * caller.  Calls nothing that allocates. */
#define LXGB_POSV_NOALLOC_SCRATCH_BYTES (16u * 1024u * 1024u + 256u)
int lxgb_posv_ragged_mixed_noalloc(int64_t batch, int32_t max_n,
                                   int32_t max_nrhs, const int32_t* n,
                                   const int32_t* nrhs, const int64_t* a_off,
                                   const double* a, const int64_t* b_off,
                                   const double* b, double* x, double tol,
                                   int32_t max_iter, int32_t* info,
                                   int32_t* iters, double* berr, void* stream);

/* ------------------------------------------------------------------------ */
/* Householder QR.                                                           */
/* ------------------------------------------------------------------------ */

/* QR of a tall m×n FP64 matrix M (n <= m) by Householder reflectors.  Input:
 * a_layout 0 — `a` is M itself, row-major m×n; a_layout 1 — `a` already holds
 * Mᵀ (n×m row-major, e.g. a wide operator that lineax transposes).  Output in
 * the raw layout of jnp.linalg.qr(M, mode="raw"): h = n×m row-major with R on
 * and above the diagonal of hᵀ and the reflectors v_k (v_k[k] = 1 implied)
 * below it, tau[n] the reflector scalars (LAPACK geqrf/larfg rules), and
 * t[lxgb_geqrf_t_elems(n)] the compact-WY T matrices of each 32-reflector
 * panel (used by lxgb_ormqr_f64).  `work`: lxgb_geqrf_workspace_size(m, n)
 * bytes.  Replaces jnp.linalg.qr(matrix, mode="raw") at
 * lineax/_solver/qr.py:62. */
int64_t lxgb_geqrf_t_elems(int64_t n);
int64_t lxgb_geqrf_workspace_size(int64_t m, int64_t n);
int lxgb_geqrf_f64(int64_t m, int64_t n, const double* a, int32_t a_layout,
                   double* h, double* tau, double* t, void* work,
                   int64_t work_bytes, void* stream);

/* Apply Qᵀ (trans 1) or Q (trans 0) of a factor from lxgb_geqrf_f64 to nrhs
 * vectors of length m stored back to back in c (in place).  `work`:
 * lxgb_ormqr_workspace_size(m, nrhs) bytes.  Replaces lax.linalg.ormqr at
 * lineax/_solver/qr.py:86 (Q, minimum-norm solutions) and :89 (Qᵀ, least
 * squares). */
int64_t lxgb_ormqr_workspace_size(int64_t m, int32_t nrhs);
int lxgb_ormqr_f64(int64_t m, int64_t n, const double* h, const double* tau,
                   const double* t, int32_t nrhs, double* c, int32_t trans,
                   void* work, int64_t work_bytes, void* stream);

/* ------------------------------------------------------------------------ */
/* Krylov solvers (k right-hand sides at once, FP64).                        */
/* ------------------------------------------------------------------------ */
/* lineax runs CG and GMRES as lax.while_loops (cg.py:209, gmres.py:215,292).
 * Here the host drives the loop and forms operator / preconditioner products
 * (the operator may be a user function); the entry points below run the rest
 * of each iteration on the device.  Every right-hand side carries device-side
 * flags double-buffered by iteration parity: a right-hand side that has
 * stopped is left untouched by later launches, so the host may run past
 * convergence and check the flags (…_status) only now and then.  Vectors of
 * a block are k vectors of length n back to back.  Workspaces need no
 * initialisation and must be 256-byte aligned. */

/* CG (lineax/_solver/cg.py:114-227).  Host sequence per iteration, parity
 * p = iteration & 1:  mat_p = A p;  lxgb_cg_step_alpha (alpha with the
 * breakdown guard, y += alpha p, r -= alpha A p unless cheap_r == 0);  on a
 * stabilising step  ay = A y, lxgb_cg_true_residual;  z = M r;
 * lxgb_cg_step_beta (gamma, beta, step, two-space stopping test, p = z + beta
 * p).  Before the loop: r = b - A y0, z = M r, lxgb_cg_start. */
int64_t lxgb_cg_workspace_size(int32_t nrhs, int64_t n);
int lxgb_cg_start(int32_t k, int64_t n, const double* r, const double* z,
                  double* p, int64_t max_steps, int32_t has_scale, void* work,
                  int64_t work_bytes, void* stream);
int lxgb_cg_step_alpha(int32_t k, int64_t n, const double* mat_p, double* p,
                       double* y, double* r, int32_t cheap_r, int32_t parity,
                       double rtol, double atol, double rcond, void* work,
                       int64_t work_bytes, void* stream);
int lxgb_cg_true_residual(int32_t k, int64_t n, const double* b,
                          const double* ay, double* r, int32_t parity,
                          void* work, int64_t work_bytes, void* stream);
int lxgb_cg_step_beta(int32_t k, int64_t n, const double* b, const double* r,
                      const double* z, double* p, int32_t parity,
                      int64_t max_steps, int32_t has_scale, double rtol,
                      double atol, void* work, int64_t work_bytes,
                      void* stream);
/* steps[c], active[c] (device int32) for the flags of the given parity. */
int lxgb_cg_status(int32_t k, int64_t n, int32_t parity, int32_t* steps,
                   int32_t* active, void* work, int64_t work_bytes,
                   void* stream);

/* BiCGStab (lineax/_solver/bicgstab.py:78-205), right-preconditioned, FP64,
 * for k right-hand sides stored back to back (vector c at base + c*n).  Each
 * right-hand side has its own scalars and a flag from lineax's loop condition
 * (no breakdown, stopping test not met, step < max_steps); every call leaves
 * an inactive right-hand side untouched.  Host sequence: r = b - A y0, then
 * lxgb_bicgstab_start(r -> r0 copy, p = v = 0); per iteration
 *   lxgb_bicgstab_direction  (rho' = <r0, r>, p = r + beta (p - omega v)),
 *   x = M p, v = A x,
 *   lxgb_bicgstab_s          (alpha = rho'/<r0, v>, s = r - alpha v),
 *   z = M s, t = A z,
 *   lxgb_bicgstab_update     (omega = <s,t>/<t,t>, y += alpha x + omega z,
 *                             r = s - omega t, stopping test, next flag).
 * lxgb_bicgstab_status copies steps, flags, (rho, alpha, omega) as three
 * k-arrays and the last "not converged" value to device arrays (any may be
 * NULL); with them the caller forms lineax's result codes (:188-202).
 * r must not alias s, t, x or z; y must not alias x, z, s or t. */
int64_t lxgb_bicgstab_workspace_size(int32_t nrhs, int64_t n);
int lxgb_bicgstab_start(int32_t k, int64_t n, const double* r, double* r0,
                        double* p, double* v, int64_t max_steps,
                        int32_t has_scale, void* work, int64_t work_bytes,
                        void* stream);
int lxgb_bicgstab_direction(int32_t k, int64_t n, const double* r0,
                            const double* r, const double* v, double* p,
                            void* work, int64_t work_bytes, void* stream);
int lxgb_bicgstab_s(int32_t k, int64_t n, const double* r0, const double* r,
                    const double* v, double* s, void* work, int64_t work_bytes,
                    void* stream);
int lxgb_bicgstab_update(int32_t k, int64_t n, const double* x, const double* z,
                         const double* s, const double* t, const double* b,
                         double* y, double* r, double rtol, double atol,
                         int64_t max_steps, int32_t has_scale, void* work,
                         int64_t work_bytes, void* stream);
int lxgb_bicgstab_status(int32_t k, int64_t n, int32_t* steps, int32_t* active,
                         double* scal, int32_t* nc, void* work,
                         int64_t work_bytes, void* stream);

/* GMRES (lineax/_solver/gmres.py:106-413), restart <= 128.  Host sequence per
 * outer iteration (parity p): unless first pass, lxgb_gmres_cycle_begin(r),
 * then for kk < restart: w = M A V[kk] (V[kk] of right-hand side c at work +
 * lxgb_gmres_basis_offset(...) + c*(restart+1)*n doubles), lxgb_gmres_arnoldi;
 * lxgb_gmres_cycle_end (least squares, y += V z, diff); t = M(b - A y);
 * lxgb_gmres_outer (r = t, stagnation, deferred breakdown, stopping test).
 * Start with lxgb_gmres_init, r = 0, diff = +inf. */
int64_t lxgb_gmres_workspace_size(int32_t nrhs, int64_t n, int32_t restart);
int64_t lxgb_gmres_basis_offset(int32_t k, int64_t n, int32_t restart,
                                int32_t kk);
int lxgb_gmres_init(int32_t k, int64_t n, int32_t restart, void* work,
                    int64_t work_bytes, void* stream);
int lxgb_gmres_cycle_begin(int32_t k, int64_t n, int32_t restart,
                           int32_t parity, const double* r, void* work,
                           int64_t work_bytes, void* stream);
int lxgb_gmres_arnoldi(int32_t k, int64_t n, int32_t restart, int32_t parity,
                       int32_t kk, double* w, int32_t* on, void* work,
                       int64_t work_bytes, void* stream);
int lxgb_gmres_cycle_end(int32_t k, int64_t n, int32_t restart,
                         int32_t parity, int32_t first, double* y,
                         double* diff, void* work, int64_t work_bytes,
                         void* stream);
int lxgb_gmres_outer(int32_t k, int64_t n, int32_t restart, int32_t parity,
                     int32_t first, const double* b, const double* t,
                     double* r, const double* diff, const double* y,
                     double rtol, double atol, int64_t max_steps,
                     int32_t stagnation_iters, int32_t has_scale, void* work,
                     int64_t work_bytes, void* stream);
/* Per right-hand side 5 ints: active (next), steps, stagnation counter,
 * breakdown (deferred), not-converged at the last test. */
int lxgb_gmres_status(int32_t k, int64_t n, int32_t restart, int32_t parity,
                      int32_t* out, void* work, int64_t work_bytes,
                      void* stream);

/* Single-call solves: the whole CG / GMRES loop on the device, the form a
 * jax.ffi custom call needs (one call per lax.while_loop of
 * lineax/_solver/cg.py:209 and gmres.py:215,292).  The call enqueues the
 * start-up launches and one CUDA graph whose conditional WHILE node runs
 * rounds of iterations until no right-hand side is active (lineax's loop
 * condition per right-hand side) or the step budget is spent; the host never
 * waits.  The operator (and the optional preconditioner, NULL for none) is
 * described by value, always multiplied by `scale` (1.0 for the operator
 * itself, -1.0 for the negated operator CG uses on negative-definite
 * operators, lineax/_solver/cg.py:100-101):
 *   LXGB_OP_DENSE     a: row-major n×n FP64 matrix, row stride lda
 *                     (MatrixLinearOperator.mv, lineax/_operator.py:269);
 *   LXGB_OP_POISSON5  the 5-point negative Laplacian on an nx×ny interior
 *                     grid (n = nx*ny), matrix-free (a FunctionLinearOperator).
 * b, y: k vectors of length n back to back; y holds y0 on entry when
 * y0_given (else it is zeroed) and the solutions on return.  max_steps < 0
 * means lineax's default 10*n with result `singular` when it is reached
 * (cg.py:213-216); steps[c] and results[c] (device int32, RESULTS codes)
 * are written per right-hand side.  Iterates, step counts and result codes
 * are those of the per-iteration entry points above.  The call launches a
 * graph of its own, so it cannot itself be captured into a stream capture.
 * Workspaces: 256-byte aligned, no initialisation. */
typedef enum lxgb_operator_kind {
  LXGB_OP_DENSE = 0,
  LXGB_OP_POISSON5 = 1,
  LXGB_OP_SPLIT_DF = 2,  /* A = hi + lo (FP32 pair, row stride lda) applied in
                            double-float arithmetic, as lxgb_gemv_df mode 1 */
  LXGB_OP_LU32_INV = 3,  /* M = U^{-1} L^{-1} P from lxgb_lu32_inverse (hi =
                            L^{-1}, lo = U^{-1}, perm), as lxgb_lu32_apply
                            mode 1: the GMRES-IR preconditioner */
  LXGB_OP_QR32 = 4       /* M = R^{-1} Qᵀ of a square FP32 QR (hi = Qᵀ, lo =
                            R^{-1}, both n×n FP32), as lxgb_qr32_apply mode
                            1: the GMRES-IR preconditioner of a QR solve */
} lxgb_operator_kind;

typedef struct lxgb_linear_operator {
  int32_t kind;          /* lxgb_operator_kind */
  int32_t reserved;      /* 0 */
  int64_t n;             /* order */
  const double* a;       /* LXGB_OP_DENSE */
  int64_t lda;           /* LXGB_OP_DENSE, LXGB_OP_SPLIT_DF */
  int64_t nx, ny;        /* LXGB_OP_POISSON5 */
  double scale;          /* factor applied to the operator (1.0: as given) */
  const float* hi;       /* LXGB_OP_SPLIT_DF, LXGB_OP_LU32_INV, LXGB_OP_QR32 */
  const float* lo;       /* LXGB_OP_SPLIT_DF, LXGB_OP_LU32_INV, LXGB_OP_QR32 */
  const int32_t* perm;   /* LXGB_OP_LU32_INV */
} lxgb_linear_operator;

/* CG (lineax/_solver/cg.py:114-227), stabilise_every in [0, 64] (0: never
 * recompute the true residual; lineax's default is 10). */
int64_t lxgb_cg_run_workspace_size(int32_t k, int64_t n, int32_t has_precond);
int lxgb_cg_run(int32_t k, int64_t n, const lxgb_linear_operator* op,
                const lxgb_linear_operator* precond, const double* b, double* y,
                int32_t y0_given, double rtol, double atol, int64_t max_steps,
                int32_t stabilise_every, int32_t* steps, int32_t* results,
                void* work, int64_t work_bytes, void* stream);

/* Restarted GMRES (lineax/_solver/gmres.py:106-413), left-preconditioned,
 * restart = min(restart, n) <= 128. */
int64_t lxgb_gmres_run_workspace_size(int32_t k, int64_t n, int32_t restart);
int lxgb_gmres_run(int32_t k, int64_t n, const lxgb_linear_operator* op,
                   const lxgb_linear_operator* precond, const double* b, double* y,
                   int32_t y0_given, double rtol, double atol, int64_t max_steps,
                   int32_t restart, int32_t stagnation_iters, int32_t* steps,
                   int32_t* results, void* work, int64_t work_bytes, void* stream);

/* GMRES-IR for the mixed-precision LU (no reference counterpart as a
 * precision mode: lineax's GMRES, lineax/_solver/gmres.py:106-413,
 * preconditioned by an LU, lineax/_solver/lu.py:53, refined to FP64
 * backward error), the whole refinement loop in one call.  op: the operator
 * as LXGB_OP_SPLIT_DF (A = hi + lo, FP64-accurate products); precond: the
 * low-precision factor as LXGB_OP_LU32_INV.  x = 0, r = b; per outer step
 * plain refinement x += M r until a step stalls (an inner solve that fails or
 * a largest backward error that does not halve), from then on GMRES(restart,
 * at most inner_max_steps restart cycles, rtol = atol = inner_rtol) on
 * r / max|r| and x += max|r| y; then r = b - A x and the normwise backward
 * error of each right-hand side with *anorm (device) = ||A||_inf.  Ends when
 * every berr[c] <= tol (status[2] = 0), when a GMRES step stalls and
 * stop_on_stall is set (status[2] = 1: the caller falls back to an FP64
 * factorisation) or after max_outer steps (status[2] = 2); status[0] = outer
 * steps, status[1] = 1 if
 * the GMRES tier was reached (device int32[3]).  The loop is a while node
 * holding an if/else node (the tier) holding the GMRES while node. */
int64_t lxgb_gmres_ir_run_workspace_size(int32_t k, int64_t n, int32_t restart);
int lxgb_gmres_ir_run(int32_t k, int64_t n, const lxgb_linear_operator* op,
                      const lxgb_linear_operator* precond, const double* b, double* x,
                      const double* anorm, double tol, double inner_rtol,
                      int32_t max_outer, int32_t restart, int32_t inner_max_steps,
                      int32_t stagnation_iters, int32_t stop_on_stall, double* berr,
                      int32_t* status, void* work, int64_t work_bytes, void* stream);

/* Batched k-vector reductions into out[c] (device): op 0 <x_c, y_c>,
 * 1 max |x_c| (NaN propagates), 2 sum x_c².  Vector c at x + c*ldx. */
int64_t lxgb_kreduce_workspace_size(int32_t k, int64_t n);
int lxgb_kreduce_f64(int32_t op, int32_t k, int64_t n, const double* x,
                     int64_t ldx, const double* y, int64_t ldy, double* out,
                     void* work, int64_t work_bytes, void* stream);

/* 5-point negative Laplacian on an nx×ny interior grid with zero Dirichlet
 * boundary, times `scale`, applied to k grids back to back (the matrix-free
 * FunctionLinearOperator of the CG benchmark configuration). */
int lxgb_poisson5_f64(int64_t nx, int64_t ny, int32_t k, double scale,
                      const double* u, double* out, void* stream);

/* ------------------------------------------------------------------------ */
/* Tensor-core GEMM.                                                         */
/* ------------------------------------------------------------------------ */

/* C = alpha * A Bᵀ + beta * C on the tcgen05 tensor cores with TF32 inputs
 * and FP32 accumulation in tensor memory.  A is m×k, B is n×k (row-major, k
 * contiguous; lda, ldb multiples of 4, A and B 16-byte aligned), C is m×n
 * row-major FP32.  *err (device int) is set to 1 if a pipeline wait timed out
 * (the result is then incomplete); the caller zeroes it.  The trailing-matrix
 * update of the mixed-precision LU (A22 -= L21 U12), the dense contraction of
 * the blocked factorisations that lineax reaches through getrf
 * (lineax/_solver/lu.py:53). */
int lxgb_gemm_tf32_nt(int32_t m, int32_t n, int32_t k, const float* a,
                      int64_t lda, const float* b, int64_t ldb, float* c,
                      int64_t ldc, float alpha, float beta, int32_t* err,
                      void* stream);

/* The same with 3xTF32 products: a = a_hi + a_lo, b = b_hi + b_lo where the
 * hi parts are TF32-exact (a and b pass the hi parts; a_lo, b_lo share their
 * leading dimensions), C += alpha (Ah Bhᵀ + Ah Blᵀ + Al Bhᵀ): FP32-level
 * accuracy from three tensor-core products per step. */
int lxgb_gemm_3xtf32_nt(int32_t m, int32_t n, int32_t k, const float* a,
                        const float* a_lo, int64_t lda, const float* b,
                        const float* b_lo, int64_t ldb, float* c, int64_t ldc,
                        float alpha, float beta, int32_t* err, void* stream);

/* C = alpha * A Bᵀ + beta * C on the tcgen05 tensor cores with BF16 inputs
 * (A m×k, B n×k, __nv_bfloat16 row-major, k contiguous; lda, ldb multiples
 * of 8, 16-byte aligned) and FP32 accumulation; C FP32 row-major.  *err as for
 * lxgb_gemm_tf32_nt.  The trailing update of the BF16 factor tier of the
 * mixed-precision LU (lineax/_solver/lu.py:53). */
int lxgb_gemm_bf16_nt(int32_t m, int32_t n, int32_t k, const void* a, int64_t lda,
                      const void* b, int64_t ldb, float* c, int64_t ldc, float alpha,
                      float beta, int32_t* err, void* stream);

/* Kernel choice of the three GEMMs above (a tuning switch, process-wide;
 * results are the same up to the order of the FP32 accumulation): 1 (the
 * default) runs them as one persistent launch of one CTA per SM with two
 * tensor-memory accumulators (128×256 tiles; 128×128 for 3xTF32), so the
 * epilogue of one tile overlaps the products of the next — used whenever C is
 * 16-byte aligned with ldc a multiple of 4; 0 runs one CTA per 128×128 tile. */
int lxgb_gemm_set_persistent(int32_t on);

/* Mixed-precision LU for GMRES-IR: P A = L U in FP32 with partial pivoting
 * (first row of max |a|), 64-column panels, trailing updates on the tcgen05
 * tensor cores with FP32 accumulation: precision 0 = TF32 products, 1 =
 * 3xTF32 (hi/lo operand split, FP32-level accuracy), 2 = BF16 products
 * (L21 and U12 rounded to BF16 for each update, tcgen05 kind::f16).  If a64 is not NULL the
 * row-major FP64 matrix is first rounded into lu (n×n FP32, 16-byte aligned);
 * otherwise lu already holds the FP32 matrix.  n must be a multiple of 4.
 * piv: 0-based swaps; info as getrf; *err (device, zeroed by the caller) = 1
 * if a tensor-core pipeline wait timed out.  `work`: 256-byte aligned,
 * lxgb_getrf_f32_tc_workspace_size(n) bytes.  The low-precision factor of
 * the GMRES-IR configuration (lineax/_solver/gmres.py preconditioned by an LU
 * of lineax/_solver/lu.py:53). */
int64_t lxgb_getrf_f32_tc_workspace_size(int32_t n, int32_t precision);
int lxgb_getrf_f32_tc(int32_t n, const double* a64, float* lu, int32_t* piv,
                      int32_t* info, int32_t precision, int32_t* err,
                      void* work, int64_t work_bytes, void* stream);

/* FP32 Cholesky A = L Lᵀ of one SPD matrix (row-major n×n FP64, read from
 * its upper triangle as lineax's cho_factor(lower=False) reads it; n % 4 == 0,
 * n < 32768) for mixed-precision refinement: l (n×n FP32, 16-byte aligned)
 * receives L in its lower triangle (the upper triangle is scratch).  64-column
 * panels: the diagonal block factored by one CTA, the panel below it by FP32
 * substitution (one row per thread), the trailing update on the tiles of the
 * lower triangle as a tcgen05 GEMM with 3xTF32 products.  *info = 0, or the 1-based index of the first pivot that is not
 * positive in FP32 (the factor is then unusable); *err is set if a tensor-core
 * pipeline wait gave up.  work 256-byte aligned, work_bytes >=
 * lxgb_potrf_f32_tc_workspace_size(n).  The low-precision counterpart of
 * cho_factor at lineax/_solver/cholesky.py:60. */
int64_t lxgb_potrf_f32_tc_workspace_size(int64_t n);
int lxgb_potrf_f32_tc(int64_t n, const double* a, float* l, int32_t* info,
                      int32_t* err, void* work, int64_t work_bytes, void* stream);

/* The factor of lxgb_potrf_f32_tc in the form of lxgb_getrf_f32_tc (L' =
 * L D^{-1} unit lower below the diagonal, U' = D Lᵀ on and above it, D =
 * diag(L)) with piv = 0..n-1, so that lxgb_lu32_inverse and GMRES-IR apply
 * to it unchanged.  l and lu may not alias. */
int lxgb_chol32_to_lu32(int64_t n, const float* l, float* lu, int32_t* piv,
                        void* stream);

/* uinv = U'^{-1} = L'^{-T} D^{-2} from linv = L'^{-1} (lxgb_lu32_inverse with
 * uinv NULL) and lu from lxgb_chol32_to_lu32 (D^2 on its diagonal): the second
 * triangular inverse of a Cholesky factor by a transposing copy. */
int lxgb_chol32_uinv(int64_t n, const float* lu, const float* linv, float* uinv,
                     void* stream);

/* x_r = U^{-1} L^{-1} P b_r for nrhs FP64 vectors (length n, back to back),
 * computed in FP32 with a factor from lxgb_getrf_f32_tc: the preconditioner
 * apply of GMRES-IR.  b and x may not alias. */
int lxgb_getrs_f32(int32_t n, int32_t nrhs, const float* lu, const int32_t* piv,
                   const double* b, double* x, void* stream);

/* Inverse factors of a factor from lxgb_getrf_f32_tc: linv = L^{-1} (unit
 * lower, zeros above the diagonal) and uinv = U^{-1} (zeros below; either one
 * may be NULL, then only the other is formed), both row-major n×n FP32, and
 * perm with (P b)_i = b[perm[i]].  Off-diagonal
 * updates on the tensor cores: precision 0 TF32, 1 3xTF32.  n <= 25600,
 * n % 4 == 0, lu 16-byte and work 256-byte aligned, work_bytes >=
 * lxgb_lu32_inverse_workspace_size.  *err is set if a tensor-core pipeline
 * wait gave up.  No reference counterpart: the build's GMRES-IR applies the
 * preconditioner (lineax/_solver/gmres.py:106-240 with an LU of
 * lineax/_solver/lu.py:53) as two triangular products with these. */
int64_t lxgb_lu32_inverse_workspace_size(int32_t n, int32_t precision);
int lxgb_lu32_inverse(int32_t n, const float* lu, const int32_t* piv,
                      float* linv, float* uinv, int32_t* perm, int32_t precision,
                      int32_t* err, void* work, int64_t work_bytes, void* stream);

/* y_r = U^{-1} L^{-1} P x_r for nrhs FP64 vectors (length n, back to back)
 * with the inverse factors above; mode 0 FP32 arithmetic, mode 1
 * double-float (about 48 significant bits, FP64-accurate).  x and y may not
 * alias. */
int64_t lxgb_lu32_apply_workspace_size(int32_t n, int32_t nrhs);
int lxgb_lu32_apply(int32_t n, int32_t nrhs, const float* linv,
                    const float* uinv, const int32_t* perm, int32_t mode,
                    const double* x, double* y, void* work, int64_t work_bytes,
                    void* stream);

/* hi = a truncated to 24 significant bits, lo = the next 24 (lo may be
 * null): a row-major rows×cols FP64 block as an FP32 pair. */
int lxgb_split_f64(int64_t rows, int64_t cols, const double* a, int64_t lda,
                   float* hi, float* lo, int64_t ld, void* stream);

/* y_r = A x_r, or y_r = b_r - A x_r when b is given (b_r at b + r*ldy), for
 * nrhs vectors, A m×n given as FP32 hi (+ optional lo) with row stride lda.
 * mode 0: FP32 arithmetic on hi; mode 1: double-float arithmetic (FP64
 * accurate for hi + lo).  The operator product and residual of GMRES-IR
 * (lineax/_operator.py:269 at FP64 accuracy). */
int64_t lxgb_gemv_df_workspace_size(int32_t n, int32_t nrhs);
int lxgb_gemv_df(int32_t m, int32_t n, const float* a_hi, const float* a_lo,
                 int64_t lda, int32_t nrhs, const double* x, int64_t ldx,
                 const double* b, double* y, int64_t ldy, int32_t mode,
                 void* work, int64_t work_bytes, void* stream);

/* Mixed-precision CG for the 5-point Poisson operator (the matrix-free
 * FunctionLinearOperator of lxgb_poisson5_f64 with scale 1) on an nx×ny grid,
 * k right-hand sides: FP32 iteration vectors p, r, Ap and correction x_lo;
 * FP64 solution x and right-hand side b (k vectors of nx*ny back to back).
 * lxgb_cg32_refresh folds x_lo into x, replaces r by the FP64 true residual
 * and applies lineax's max-norm stopping test to it (the solve of
 * lineax/_solver/cg.py:114-227 with FP32 iterations between FP64 residual
 * replacements; no reference counterpart as a precision mode).  Driver:
 * init, refresh, start_direction, then (iterate, refresh) until status
 * reports no active right-hand side.  status: 3 ints per right-hand side
 * (active, steps, 0 running / max steps, 1 converged, 2 breakdown or NaN). */
int64_t lxgb_cg32_workspace_size(int32_t nrhs);
int lxgb_cg32_init(int32_t k, int64_t nx, int64_t ny, int64_t max_steps,
                   void* work, int64_t work_bytes, void* stream);
int lxgb_cg32_refresh(int32_t k, int64_t nx, int64_t ny, const double* b,
                      double* x, float* xlo, float* r, double rtol, double atol,
                      int64_t max_steps, void* work, int64_t work_bytes,
                      void* stream);
int lxgb_cg32_start_direction(int32_t k, int64_t n, const float* r, float* p,
                              void* stream);
int lxgb_cg32_iterate(int32_t k, int64_t nx, int64_t ny, int32_t iters,
                      float* p, float* ap, float* xlo, float* r, void* work,
                      int64_t work_bytes, void* stream);
int lxgb_cg32_status(int32_t k, int32_t* out, void* work, int64_t work_bytes,
                     void* stream);

/* Householder QR of a tall FP64 matrix A (m × n row-major, n <= m, m % 4 ==
 * 0) in FP32 with the trailing updates on the tcgen05 tensor cores (TF32
 * products): h (n × m FP32) in the raw layout of lxgb_geqrf_f64, tau (n),
 * t (lxgb_geqrf_t_elems(n) FP32: each panel's compact-WY T).  h 16-byte and
 * work 256-byte aligned; *err is set if a tensor-core pipeline wait gave up.
 * The factor of the mixed-precision least-squares solve (no reference
 * counterpart as a precision mode of lineax/_solver/qr.py:55-118). */
int64_t lxgb_geqrf_f32_tc_workspace_size(int64_t m, int64_t n);
int lxgb_geqrf_f32_tc(int64_t m, int64_t n, const double* a, float* h, float* tau,
                      float* t, int32_t* err, void* work, int64_t work_bytes,
                      void* stream);

/* lxgb_geqrf_f32_tc that also forms Q explicitly: the reflectors are applied
 * to the m×m identity in the same tensor-core trailing updates, leaving q
 * (m×m FP32 row-major, 16-byte aligned) = Q with A = Q [R; 0].  `work`:
 * lxgb_geqrf_f32_tc_q_workspace_size(m, n) bytes.  With the triangular
 * inverse of R (lxgb_lu32_inverse on R with identity pivots) it gives the
 * square-system preconditioner M = R^{-1} Qᵀ of lxgb_qr32_apply: the
 * low-precision QR factor of a mixed-precision square solve (lineax's QR
 * solver, lineax/_solver/qr.py:55-94, recovered to FP64 accuracy by GMRES
 * refinement; no reference counterpart as a precision mode). */
int64_t lxgb_geqrf_f32_tc_q_workspace_size(int64_t m, int64_t n);
int lxgb_geqrf_f32_tc_q(int64_t m, int64_t n, const double* a, float* h, float* tau,
                        float* t, float* q, int32_t* err, void* work, int64_t work_bytes,
                        void* stream);

/* y_r = R^{-1} (Qᵀ x_r) for nrhs FP64 vectors of length n (back to back):
 * qt = Qᵀ (n×n FP32 row-major, full), rinv = R^{-1} (n×n FP32, upper
 * triangle read).  mode 0 FP32, 1 double-float arithmetic.  x and y may not
 * alias.  `work`: lxgb_qr32_apply_workspace_size(n, nrhs) bytes. */
int64_t lxgb_qr32_apply_workspace_size(int32_t n, int32_t nrhs);
int lxgb_qr32_apply(int32_t n, int32_t nrhs, const float* qt, const float* rinv,
                    int32_t mode, const double* x, double* y, void* work,
                    int64_t work_bytes, void* stream);

/* ------------------------------------------------------------------------ */
/* Triangular solves.                                                        */
/* ------------------------------------------------------------------------ */

/* Solve op(T) X = B in place on B, T row-major n×n (ldt >= n) FP64,
 * op = T (trans 0) or Tᵀ (trans 1), lower/upper and unit-diagonal flags as in
 * jax.scipy.linalg.solve_triangular.  B holds nrhs vectors of length n.
 * Replaces solve_triangular at lineax/_solver/triangular.py:81 and
 * lineax/_solver/qr.py:83,90. */
int lxgb_trsm_f64(int32_t n, int32_t nrhs, const double* t, int64_t ldt,
                  int32_t lower, int32_t trans, int32_t unit_diag, double* b,
                  void* stream);

/* ------------------------------------------------------------------------ */
/* Level-2 helpers.                                                          */
/* ------------------------------------------------------------------------ */

/* y_v = alpha op(A) x_v + beta y_v for v < nvec (x_v at x + v*ldx, y_v at
 * y + v*ldy), A row-major m×n FP64 with row stride lda >= n, op = A (trans 0)
 * or Aᵀ (trans 1).  beta == 0 does not read y.  Deterministic reduction order.
 * Replaces the matmul of MatrixLinearOperator.mv at lineax/_operator.py:269
 * (precision HIGHEST) and the residual b - A x of refinement. */
int lxgb_gemv_f64(int64_t m, int64_t n, const double* a, int64_t lda,
                  int32_t trans, int32_t nvec, const double* x, int64_t ldx,
                  double* y, int64_t ldy, double alpha, double beta,
                  void* stream);

/* flag[0] = 1 if any of x[0..n) is NaN or ±inf, else 0 (device int32).
 * The scan lineax applies to every solution and right-hand side at
 * lineax/_solve.py:104-123. */
int lxgb_nonfinite_f64(int64_t n, const double* x, int32_t* flag, void* stream);

/* Deterministic reductions of FP64 vectors into out[0] (device):
 *   op 0: Σ x_i y_i   (tree_dot, lineax/_norm.py:27-47)
 *   op 1: max |x_i|   (max_norm, lineax/_norm.py:123-143; NaN propagates)
 *   op 2: Σ x_i²      (sum_squares, lineax/_norm.py:50-56)
 *   op 3: sqrt(Σ x_i²), |x_0| when n == 1 (two_norm, lineax/_norm.py:59-77)
 * The split of the sum depends on n only, so equal inputs give equal bits.
 * `work` holds lxgb_reduce_workspace_size(n) bytes. */
int64_t lxgb_reduce_workspace_size(int64_t n);
int lxgb_reduce_f64(int32_t op, int64_t n, const double* x, const double* y,
                    double* out, void* work, int64_t work_bytes, void* stream);

/* Blocks of k FP64 vectors of length n (vector c at x + c*n), per-vector
 * scalars s[c] on the device:  x_c *= s[c] (invert: x_c *= 1/s[c], a zero
 * scale giving zeros), and y_c += s[c] x_c.  The vector updates of the
 * GMRES-IR outer loop (correction scaling, x += d). */
int lxgb_rows_scale_f64(int32_t k, int64_t n, const double* s, int32_t invert,
                        double* x, void* stream);
int lxgb_rows_axpy_f64(int32_t k, int64_t n, const double* s, const double* x,
                       double* y, void* stream);

/* out[0] = ||A||_inf = max_i sum_j |a_ij| (device), for normwise backward
 * errors; `work` holds lxgb_norm_inf_workspace_size(m) bytes. */
int64_t lxgb_norm_inf_workspace_size(int64_t m);
int lxgb_norm_inf_f64(int64_t m, int64_t n, const double* a, int64_t lda,
                      double* out, void* work, int64_t work_bytes, void* stream);

/* x_i = b_i / a[i*stride] (stride n+1 walks a matrix diagonal); with
 * well_posed == 0 a zero diagonal entry gives x_i = 0 (pseudo-inverse).
 * The solve of lineax/_solver/diagonal.py, reached by AutoLinearSolver for
 * diagonal-tagged and 1×1 operators (lineax/_solve.py:569-570). */
int lxgb_diag_solve_f64(int64_t n, const double* a, int64_t stride,
                        const double* b, double* x, int32_t well_posed,
                        void* stream);

#ifdef __cplusplus
}
#endif

#endif /* LXGB_H_ */
