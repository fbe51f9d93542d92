// Level-2 helpers of the solve path: dense FP64 matrix-vector products
// (MatrixLinearOperator.mv, residuals b - A x) and the non-finite scan that
// lineax applies to every solution and right-hand side.  Reductions are
// deterministic: a fixed split of the work and a fixed combination order.
#include <math.h>

#include "common.cuh"

namespace lxgb {

constexpr int kGemvThreads = 256;

// y_v = alpha * A x_v + beta * y_v, A row-major m×n.  One warp per row.
__global__ void __launch_bounds__(kGemvThreads)
gemv_n_kernel(int64_t m, int64_t n, const double* __restrict__ a, int64_t lda, int nvec,
              const double* __restrict__ x, int64_t ldx, double* __restrict__ y, int64_t ldy,
              double alpha, double beta) {
  const int lane = threadIdx.x & 31;
  const int64_t warp_global = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = warp_global; i < m; i += nwarps) {
    const double* row = a + i * lda;
    for (int v = 0; v < nvec; ++v) {
      const double* xv = x + (int64_t)v * ldx;
      double acc = 0.0;
      for (int64_t j = lane; j < n; j += 32) acc = fma(row[j], xv[j], acc);
      acc = warp_sum(acc);
      if (lane == 0) {
        double* yv = y + (int64_t)v * ldy + i;
        *yv = (beta == 0.0) ? alpha * acc : fma(beta, *yv, alpha * acc);
      }
    }
  }
}

// y_v = alpha * Aᵀ x_v + beta * y_v.  One CTA per strip of 32 columns; its 8
// warps split the rows and their partial sums are combined in warp order.
__global__ void __launch_bounds__(kGemvThreads)
gemv_t_kernel(int64_t m, int64_t n, const double* __restrict__ a, int64_t lda, int nvec,
              const double* __restrict__ x, int64_t ldx, double* __restrict__ y, int64_t ldy,
              double alpha, double beta) {
  __shared__ double part[kGemvThreads / 32][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
  const int64_t j = blockIdx.x * 32LL + lane;
  for (int v = 0; v < nvec; ++v) {
    const double* xv = x + (int64_t)v * ldx;
    double acc = 0.0;
    if (j < n)
      for (int64_t i = warp; i < m; i += nw) acc = fma(a[i * lda + j], xv[i], acc);
    part[warp][lane] = acc;
    __syncthreads();
    if (warp == 0 && j < n) {
      double s = 0.0;
      for (int w = 0; w < nw; ++w) s += part[w][lane];
      double* yv = y + (int64_t)v * ldy + j;
      *yv = (beta == 0.0) ? alpha * s : fma(beta, *yv, alpha * s);
    }
    __syncthreads();
  }
}

__global__ void nonfinite_kernel(int64_t n, const double* __restrict__ x, int32_t* flag) {
  int found = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    found |= !isfinite(x[i]);
  found = __syncthreads_or(found);
  if (found && threadIdx.x == 0) atomicOr(flag, 1);
}

__global__ void set_i32_kernel(int32_t* p, int32_t v) { *p = v; }

// x_i = b_i / d_i with d_i = a[i * stride]; the pseudo-inverse variant maps
// d_i == 0 to x_i = 0 (lineax/_solver/diagonal.py).
__global__ void diag_solve_kernel(int64_t n, const double* __restrict__ a, int64_t stride,
                                  const double* __restrict__ b, double* __restrict__ x,
                                  int well_posed) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double d = a[i * stride];
  x[i] = (!well_posed && d == 0.0) ? 0.0 : b[i] / d;
}

// Deterministic reductions: a fixed grid (a function of n only) writes one
// partial per CTA, a single-CTA pass combines the partials in index order.
// op 0: sum x*y; 1: max|x| (NaN propagates, as jnp.max); 2: sum x*x;
// 3: sqrt(sum x*x) (|x| when n == 1, lineax/_norm.py:66-75).
constexpr int kRedThreads = 256;

__device__ __forceinline__ double nanmax(double a, double b) {
  return (a != a || b != b) ? NAN : fmax(a, b);
}

__global__ void __launch_bounds__(kRedThreads)
reduce_partial_kernel(int op, int64_t n, const double* __restrict__ x,
                      const double* __restrict__ y, double* __restrict__ part) {
  __shared__ double sm[kRedThreads / 32];
  double acc = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double v = x[i];
    if (op == 0) acc = fma(v, y[i], acc);
    else if (op == 1) acc = nanmax(acc, fabs(v));
    else acc = fma(v, v, acc);
  }
  if (op == 1) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc = nanmax(acc, __shfl_xor_sync(0xffffffffu, acc, o));
  } else {
    acc = warp_sum(acc);
  }
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = sm[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) t = (op == 1) ? nanmax(t, sm[w]) : t + sm[w];
    part[blockIdx.x] = t;
  }
}

__global__ void reduce_final_kernel(int op, int nparts, int64_t n, const double* __restrict__ x,
                                    const double* __restrict__ part, double* __restrict__ out) {
  if (threadIdx.x != 0) return;
  double t = (nparts > 0) ? part[0] : 0.0;
  for (int i = 1; i < nparts; ++i) t = (op == 1) ? nanmax(t, part[i]) : t + part[i];
  if (op == 3) t = (n == 1) ? fabs(x[0]) : sqrt(t);
  *out = t;
}

static int reduce_parts(int64_t n) {
  const int64_t want = (n + kRedThreads * 8 - 1) / (kRedThreads * 8);
  const int64_t cap = 4LL * 152;  // fixed (not the device's SM count) so results never
                                  // depend on which GPU ran them
  return (int)(want < 1 ? 1 : (want < cap ? want : cap));
}

// Row-wise helpers for blocks of k vectors of length n (vector c at x + c*n):
// scale x_c by s[c] (or 1/s[c]; a zero scale leaves zeros), and y_c += s[c] x_c.
__global__ void rows_scale_kernel(int k, int64_t n, const double* __restrict__ s, int invert,
                                  double* __restrict__ x) {
  const int c = blockIdx.y;
  const double sc = s[c];
  const double f = invert ? (sc != 0.0 ? 1.0 / sc : 0.0) : sc;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[(int64_t)c * n + i] *= f;
}

__global__ void rows_axpy_kernel(int k, int64_t n, const double* __restrict__ s,
                                 const double* __restrict__ x, double* __restrict__ y) {
  const int c = blockIdx.y;
  const double sc = s[c];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[(int64_t)c * n + i] = fma(sc, x[(int64_t)c * n + i], y[(int64_t)c * n + i]);
}

// out = max_i sum_j |a_ij| (||A||_inf), one warp per row, fixed combination order.
__global__ void __launch_bounds__(256)
norm_inf_partial_kernel(int64_t m, int64_t n, const double* __restrict__ a, int64_t lda,
                        double* __restrict__ part) {
  __shared__ double sm[8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double best = 0.0;
  for (int64_t i = blockIdx.x * 8LL + warp; i < m; i += (int64_t)gridDim.x * 8) {
    double acc = 0.0;
    for (int64_t j = lane; j < n; j += 32) acc += fabs(a[i * lda + j]);
    acc = warp_sum(acc);
    best = nanmax(best, acc);
  }
  if (lane == 0) sm[warp] = best;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = sm[0];
    for (int w = 1; w < 8; ++w) t = nanmax(t, sm[w]);
    part[blockIdx.x] = t;
  }
}

}  // namespace lxgb

using namespace lxgb;

extern "C" int lxgb_rows_scale_f64(int32_t k, int64_t n, const double* s, int32_t invert,
                                   double* x, void* stream) {
  LXGB_REQUIRE(k >= 0 && k <= 65535 && n >= 0, "rows_scale: bad sizes");
  if (k == 0 || n == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(s && x, "rows_scale: null pointer");
  const int64_t bx = (n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024;
  rows_scale_kernel<<<dim3((unsigned)bx, (unsigned)k), 256, 0, as_stream(stream)>>>(k, n, s, invert, x);
  return check_launch("rows_scale");
}

extern "C" int lxgb_rows_axpy_f64(int32_t k, int64_t n, const double* s, const double* x, double* y,
                                  void* stream) {
  LXGB_REQUIRE(k >= 0 && k <= 65535 && n >= 0, "rows_axpy: bad sizes");
  if (k == 0 || n == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(s && x && y, "rows_axpy: null pointer");
  const int64_t bx = (n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024;
  rows_axpy_kernel<<<dim3((unsigned)bx, (unsigned)k), 256, 0, as_stream(stream)>>>(k, n, s, x, y);
  return check_launch("rows_axpy");
}

extern "C" int lxgb_norm_inf_f64(int64_t m, int64_t n, const double* a, int64_t lda, double* out,
                                 void* work, int64_t work_bytes, void* stream) {
  LXGB_REQUIRE(m >= 0 && n >= 0 && out && work, "norm_inf: bad arguments");
  LXGB_REQUIRE(m == 0 || (a && lda >= n), "norm_inf: bad matrix");
  const int parts = reduce_parts(m * 32);
  if (work_bytes < (int64_t)parts * 8) {
    set_last_error("norm_inf: workspace too small");
    return LXGB_WORKSPACE_TOO_SMALL;
  }
  cudaStream_t st = as_stream(stream);
  double* part = reinterpret_cast<double*>(work);
  norm_inf_partial_kernel<<<parts, 256, 0, st>>>(m, n, a, lda, part);
  reduce_final_kernel<<<1, 32, 0, st>>>(1, parts, 0, nullptr, part, out);
  return check_launch("norm_inf");
}

extern "C" int64_t lxgb_norm_inf_workspace_size(int64_t m) {
  return (int64_t)reduce_parts((m > 0 ? m : 1) * 32) * 8;
}

extern "C" int64_t lxgb_reduce_workspace_size(int64_t n) {
  return (int64_t)reduce_parts(n < 0 ? 0 : n) * (int64_t)sizeof(double);
}

extern "C" int lxgb_reduce_f64(int32_t op, int64_t n, const double* x, const double* y,
                               double* out, void* work, int64_t work_bytes, void* stream) {
  LXGB_REQUIRE(op >= 0 && op <= 3, "reduce: op must be 0..3");
  LXGB_REQUIRE(n >= 0 && out && work, "reduce: bad arguments");
  LXGB_REQUIRE(n == 0 || x, "reduce: null x");
  LXGB_REQUIRE(op != 0 || n == 0 || y, "reduce: null y");
  if (work_bytes < lxgb_reduce_workspace_size(n)) {
    set_last_error("reduce: workspace too small");
    return LXGB_WORKSPACE_TOO_SMALL;
  }
  cudaStream_t st = as_stream(stream);
  const int parts = reduce_parts(n);
  double* part = reinterpret_cast<double*>(work);
  reduce_partial_kernel<<<parts, kRedThreads, 0, st>>>(op, n, x, y, part);
  reduce_final_kernel<<<1, 32, 0, st>>>(op, parts, n, x, part, out);
  return check_launch("reduce");
}

extern "C" int lxgb_gemv_f64(int64_t m, int64_t n, const double* a, int64_t lda, int32_t trans,
                             int32_t nvec, const double* x, int64_t ldx, double* y, int64_t ldy,
                             double alpha, double beta, void* stream) {
  LXGB_REQUIRE(m >= 0 && n >= 0 && nvec >= 0, "gemv: negative size");
  if (nvec == 0 || (trans ? n : m) == 0) return LXGB_SUCCESSFUL;  // empty output
  LXGB_REQUIRE(y && (a || m * n == 0) && (x || (trans ? m : n) == 0), "gemv: null pointer");
  LXGB_REQUIRE(m == 0 || lda >= n, "gemv: lda < n");
  cudaStream_t st = as_stream(stream);
  if (!trans) {
    const int64_t want = (m + 7) / 8;
    const int64_t cap = 16LL * sm_count();
    gemv_n_kernel<<<(unsigned)(want < cap ? want : cap), kGemvThreads, 0, st>>>(
        m, n, a, lda, nvec, x, ldx, y, ldy, alpha, beta);
  } else {
    gemv_t_kernel<<<(unsigned)((n + 31) / 32), kGemvThreads, 0, st>>>(m, n, a, lda, nvec, x, ldx,
                                                                      y, ldy, alpha, beta);
  }
  return check_launch("gemv");
}

extern "C" int lxgb_nonfinite_f64(int64_t n, const double* x, int32_t* flag, void* stream) {
  LXGB_REQUIRE(n >= 0 && flag, "nonfinite: bad arguments");
  cudaStream_t st = as_stream(stream);
  set_i32_kernel<<<1, 1, 0, st>>>(flag, 0);
  if (n > 0) {
    LXGB_REQUIRE(x, "nonfinite: null pointer");
    const int64_t want = (n + 255) / 256;
    const int64_t cap = 8LL * sm_count();
    nonfinite_kernel<<<(unsigned)(want < cap ? want : cap), 256, 0, st>>>(n, x, flag);
  }
  return check_launch("nonfinite");
}

extern "C" int lxgb_diag_solve_f64(int64_t n, const double* a, int64_t stride, const double* b,
                                   double* x, int32_t well_posed, void* stream) {
  LXGB_REQUIRE(n >= 0, "diag_solve: negative size");
  if (n == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(a && b && x, "diag_solve: null pointer");
  diag_solve_kernel<<<(unsigned)((n + 255) / 256), 256, 0, as_stream(stream)>>>(n, a, stride, b, x,
                                                                               well_posed);
  return check_launch("diag_solve");
}
