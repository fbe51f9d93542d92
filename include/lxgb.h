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
 * Systems are taken from a work queue in index order, so placing the largest
 * first balances the launch.
 * Replaces jax.scipy.linalg.cho_factor(lower=False) at
 * lineax/_solver/cholesky.py:60. */
int lxgb_potrf_ragged_f64(int64_t batch, int32_t max_n, const int32_t* n,
                          const int64_t* a_off, double* a, int32_t* info,
                          void* stream);

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

/* Allocation-free form of lxgb_posv_ragged_mixed (no counterpart in the
 * reference).  It is for callers that cannot allocate device memory when they
 * solve — an XLA/JAX FFI handler, whose device memory belongs to XLA and where
 * a cudaMalloc can synchronise the device or break a graph capture, or a
 * serving / real-time loop that forbids allocation after start-up.  Arguments
 * and results are those of lxgb_posv_ragged_mixed without `work`: the scratch
 * is a fixed array of LXGB_POSV_NOALLOC_SCRATCH_BYTES (16 MiB + 256 B) inside
 * the library, which every GPU that loads the library holds until the process
 * exits.  Limits: max_n <= 2048 (larger is rejected with LXGB_INVALID_ARG);
 * systems with n > 224 factor in 16 MiB / (4·max_n²) slices, so fewer CTAs run
 * them than in the workspace form (at max_n = 512, 16 at a time).
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
