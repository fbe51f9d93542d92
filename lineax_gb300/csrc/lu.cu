// LU factorisation with partial pivoting (getrf) and the matching solve
// (getrs), FP64, row-major.
//
// Two factor paths share one arithmetic definition, the unblocked
// right-looking recurrence of LAPACK getf2:
//   p      = first row of max |a(i,k)|, i >= k            (idamax)
//   swap rows k and p (whole row)
//   a(i,k) = a(i,k) * (1/a(k,k))   (a(i,k) / a(k,k) when |a(k,k)| < DBL_MIN)
//   a(i,j) = fma(-a(i,k), a(k,j), a(i,j))   for i > k, j > k, k ascending
//
//  * n <= kSmallMax: one CTA per matrix, the matrix resident in shared memory.
//  * larger n: right-looking blocked LU with a panel of kNB columns (panel
//    getf2 by one CTA, row interchanges of the other columns, a TRSM for the
//    block row, a GEMM for the trailing matrix).  The TRSM and the GEMM apply
//    their updates to each element as an FMA chain over k in ascending order
//    starting from the stored value, which is exactly the operation sequence
//    getf2 applies to that element, so both paths give bit-identical factors
//    and pivots for the same input.
#include <float.h>
#include <limits.h>

#include "common.cuh"
#include "tri.cuh"

namespace lxgb {

constexpr int kSmallMax = 168;   // 168*169*8 B = 227 KB of shared memory
constexpr int kSmallThreads = 256;
constexpr int kNB = 32;          // panel width of the blocked path
constexpr int kPanelThreads = 1024;

__device__ __forceinline__ double scale_pivot(double v, double akk, double r, bool use_recip) {
  return use_recip ? v * r : v / akk;
}

// ---------------------------------------------------------------------------
// n <= kSmallMax: one CTA per matrix, matrix in shared memory (row stride ld,
// odd so that column walks hit distinct banks).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kSmallThreads)
getrf_small_kernel(int n, double* __restrict__ a, int64_t stride_a, int32_t* __restrict__ piv,
                   int64_t stride_piv, int32_t* __restrict__ info) {
  extern __shared__ double smem_lu[];
  __shared__ int s_p;
  __shared__ double s_akk, s_old;
  const int ld = n | 1;
  double* A = smem_lu;
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int b = blockIdx.x;
  double* g = a + (int64_t)b * stride_a;
  int32_t* gp = piv + (int64_t)b * stride_piv;
  for (int e = tid; e < n * n; e += blockDim.x) {
    const int i = e / n, j = e - i * n;
    A[i * ld + j] = g[e];
  }
  int my_info = 0;
  __syncthreads();
  const int tx = tid & 31, ty = tid >> 5;
  for (int k = 0; k < n; ++k) {
    if (tid < 32) {
      double v = -1.0;
      int idx = INT_MAX;
      for (int i = k + lane; i < n; i += 32) {
        const double x = fabs(A[i * ld + k]);
        if (x > v) { v = x; idx = i; }
      }
      warp_argmax_first(v, idx);
      if (lane == 0) {
        if (idx == INT_MAX) idx = k;  // column of NaNs: keep the row
        s_p = idx;
        s_akk = A[idx * ld + k];
        s_old = A[k * ld + k];
        gp[k] = idx;
      }
    }
    __syncthreads();
    const int p = s_p;
    const double akk = s_akk;
    if (akk != 0.0) {
      if (p != k) {
        for (int j = tid; j < n; j += blockDim.x) {
          if (j == k) continue;
          const double t = A[k * ld + j];
          A[k * ld + j] = A[p * ld + j];
          A[p * ld + j] = t;
        }
      }
      const bool use_recip = fabs(akk) >= DBL_MIN;
      const double r = 1.0 / akk;
      if (tid == 0) A[k * ld + k] = akk;
      for (int i = k + 1 + tid; i < n; i += blockDim.x) {
        const double v = (i == p) ? s_old : A[i * ld + k];
        A[i * ld + k] = scale_pivot(v, akk, r, use_recip);
      }
    } else if (my_info == 0) {
      my_info = k + 1;
    }
    __syncthreads();
    // rank-1 update of the trailing block; u(k,j) cached in registers.  Only
    // the 32-column chunks that hold trailing columns are visited (a
    // warp-uniform break): a predicated-off FP64 instruction still occupies
    // GB300's narrow FP64 pipe, and unrolling over all kSmallMax columns
    // issued about three times the needed DFMAs at n = 128.
    const int nchunk = (n - k - 1 + 31) >> 5;
    double u[(kSmallMax + 31) / 32];
#pragma unroll
    for (int c = 0; c < (kSmallMax + 31) / 32; ++c) {
      if (c >= nchunk) break;
      const int j = k + 1 + tx + 32 * c;
      u[c] = (j < n) ? A[k * ld + j] : 0.0;
    }
    for (int i = k + 1 + ty; i < n; i += (kSmallThreads >> 5)) {
      const double l = A[i * ld + k];
#pragma unroll
      for (int c = 0; c < (kSmallMax + 31) / 32; ++c) {
        if (c >= nchunk) break;
        const int j = k + 1 + tx + 32 * c;
        if (j < n) A[i * ld + j] = fma(-l, u[c], A[i * ld + j]);
      }
    }
    __syncthreads();
  }
  for (int e = tid; e < n * n; e += blockDim.x) {
    const int i = e / n, j = e - i * n;
    g[e] = A[i * ld + j];
  }
  if (tid == 0) info[b] = my_info;
}

// ---------------------------------------------------------------------------
// Blocked path, one matrix at a time (lda = n).
// ---------------------------------------------------------------------------

// getf2 on the panel columns [j0, j0+nb) over rows [j0, n) by one CTA.
// Row interchanges touch only the panel columns; the other columns receive
// them from laswp_kernel.
__global__ void __launch_bounds__(kPanelThreads)
panel_getf2_kernel(int n, int j0, int nb, double* __restrict__ a, int32_t* __restrict__ piv,
                   int32_t* __restrict__ info) {
  __shared__ double s_v[32];
  __shared__ int s_i[32];
  __shared__ int s_p;
  __shared__ double s_akk, s_old;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nwarps = blockDim.x >> 5;
  for (int k = j0; k < j0 + nb; ++k) {
    double v = -1.0;
    int idx = INT_MAX;
    for (int i = k + tid; i < n; i += blockDim.x) {
      const double x = fabs(a[(int64_t)i * n + k]);
      if (x > v) { v = x; idx = i; }
    }
    warp_argmax_first(v, idx);
    if (lane == 0) { s_v[warp] = v; s_i[warp] = idx; }
    __syncthreads();
    if (warp == 0) {
      v = lane < nwarps ? s_v[lane] : -1.0;
      idx = lane < nwarps ? s_i[lane] : INT_MAX;
      warp_argmax_first(v, idx);
      if (lane == 0) {
        if (idx == INT_MAX) idx = k;
        s_p = idx;
        s_akk = a[(int64_t)idx * n + k];
        s_old = a[(int64_t)k * n + k];
        piv[k] = idx;
        if (s_akk == 0.0 && *info == 0) *info = k + 1;
      }
    }
    __syncthreads();
    const int p = s_p;
    const double akk = s_akk;
    if (akk != 0.0) {
      if (p != k) {
        for (int j = j0 + tid; j < j0 + nb; j += blockDim.x) {
          if (j == k) continue;
          const double t = a[(int64_t)k * n + j];
          a[(int64_t)k * n + j] = a[(int64_t)p * n + j];
          a[(int64_t)p * n + j] = t;
        }
      }
      const bool use_recip = fabs(akk) >= DBL_MIN;
      const double r = 1.0 / akk;
      if (tid == 0) a[(int64_t)k * n + k] = akk;
      for (int i = k + 1 + tid; i < n; i += blockDim.x) {
        const double x = (i == p) ? s_old : a[(int64_t)i * n + k];
        a[(int64_t)i * n + k] = scale_pivot(x, akk, r, use_recip);
      }
    }
    __syncthreads();
    // update the remaining panel columns (k, j0+nb) of rows i > k.
    const int w = j0 + nb - (k + 1);
    if (w > 0) {
      for (int e = tid; e < (n - k - 1) * w; e += blockDim.x) {
        const int i = k + 1 + e / w;
        const int j = k + 1 + e % w;
        a[(int64_t)i * n + j] = fma(-a[(int64_t)i * n + k], a[(int64_t)k * n + j], a[(int64_t)i * n + j]);
      }
    }
    __syncthreads();
  }
}

// Apply the panel's interchanges (rows k <-> piv[k], k = j0..j0+nb-1 in order)
// to every column outside the panel.  One thread per column.
__global__ void laswp_kernel(int n, int j0, int nb, double* __restrict__ a,
                             const int32_t* __restrict__ piv) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int outside = n - nb;
  if (c >= outside) return;
  const int j = (c < j0) ? c : c + nb;
  for (int k = j0; k < j0 + nb; ++k) {
    const int p = piv[k];
    if (p != k) {
      const double t = a[(int64_t)k * n + j];
      a[(int64_t)k * n + j] = a[(int64_t)p * n + j];
      a[(int64_t)p * n + j] = t;
    }
  }
}

// Block row U12 = L11^{-1} A12 (L11 unit lower, nb×nb) by column-oriented
// forward substitution: a(i,j) = fma(-l(i,k), a(k,j), a(i,j)), k ascending.
__global__ void __launch_bounds__(256)
trsm_blockrow_kernel(int n, int j0, int nb, double* __restrict__ a) {
  __shared__ double L[kNB][kNB + 1];
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
    const int i = e / nb, k = e % nb;
    L[i][k] = a[(int64_t)(j0 + i) * n + j0 + k];
  }
  __syncthreads();
  const int j = j0 + nb + blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  double col[kNB];
#pragma unroll
  for (int i = 0; i < kNB; ++i) col[i] = (i < nb) ? a[(int64_t)(j0 + i) * n + j] : 0.0;
#pragma unroll
  for (int k = 0; k < kNB; ++k) {
#pragma unroll
    for (int i = k + 1; i < kNB; ++i) col[i] = fma(-L[i][k], col[k], col[i]);
  }
#pragma unroll
  for (int i = 0; i < kNB; ++i)
    if (i < nb) a[(int64_t)(j0 + i) * n + j] = col[i];
}

// Trailing update A22 -= L21·U12 (k = j0..j0+nb-1), each element an FMA chain
// from its stored value.  64×64 tile per CTA, 4×4 per thread.
constexpr int kGT = 64;
__global__ void __launch_bounds__(256)
gemm_trailing_kernel(int n, int j0, int nb, double* __restrict__ a) {
  __shared__ double Ls[kGT][kNB + 1];
  __shared__ double Us[kNB][kGT + 1];
  const int s = j0 + nb;
  const int i0 = s + blockIdx.y * kGT;
  const int c0 = s + blockIdx.x * kGT;
  const int tid = threadIdx.x;
  for (int e = tid; e < kGT * kNB; e += blockDim.x) {
    const int r = e / kNB, k = e % kNB;
    const int i = i0 + r;
    Ls[r][k] = (i < n && k < nb) ? a[(int64_t)i * n + j0 + k] : 0.0;
  }
  for (int e = tid; e < kNB * kGT; e += blockDim.x) {
    const int k = e / kGT, c = e % kGT;
    const int j = c0 + c;
    Us[k][c] = (j < n && k < nb) ? a[(int64_t)(j0 + k) * n + j] : 0.0;
  }
  __syncthreads();
  const int tx = tid & 15, ty = tid >> 4;
  double acc[4][4];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int i = i0 + ty + 16 * r, j = c0 + tx + 16 * c;
      acc[r][c] = (i < n && j < n) ? a[(int64_t)i * n + j] : 0.0;
    }
  for (int k = 0; k < nb; ++k) {
    double l[4], u[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) l[r] = Ls[ty + 16 * r][k];
#pragma unroll
    for (int c = 0; c < 4; ++c) u[c] = Us[k][tx + 16 * c];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[r][c] = fma(-l[r], u[c], acc[r][c]);
  }
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int i = i0 + ty + 16 * r, j = c0 + tx + 16 * c;
      if (i < n && j < n) a[(int64_t)i * n + j] = acc[r][c];
    }
}

__global__ void zero_info_kernel(int32_t* info, int64_t count) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < count) info[i] = 0;
}

int getrf_blocked(int n, double* a, int32_t* piv, int32_t* info, cudaStream_t st) {
  zero_info_kernel<<<1, 32, 0, st>>>(info, 1);
  for (int j0 = 0; j0 < n; j0 += kNB) {
    const int nb = min(kNB, n - j0);
    panel_getf2_kernel<<<1, kPanelThreads, 0, st>>>(n, j0, nb, a, piv, info);
    const int outside = n - nb;
    if (outside > 0) laswp_kernel<<<(outside + 127) / 128, 128, 0, st>>>(n, j0, nb, a, piv);
    const int rest = n - j0 - nb;
    if (rest > 0) {
      trsm_blockrow_kernel<<<(rest + 255) / 256, 256, 0, st>>>(n, j0, nb, a);
      dim3 grid((rest + kGT - 1) / kGT, (rest + kGT - 1) / kGT);
      gemm_trailing_kernel<<<grid, 256, 0, st>>>(n, j0, nb, a);
    }
  }
  return check_launch("getrf blocked");
}

// ---------------------------------------------------------------------------
// getrs: one CTA per (system, right-hand side).  The vector and the pivots
// are staged in shared memory when they fit.
// ---------------------------------------------------------------------------
constexpr int kSolveThreads = 256;

__global__ void __launch_bounds__(kSolveThreads)
getrs_kernel(int n, int nrhs, const double* __restrict__ lu, int64_t stride_a,
             const int32_t* __restrict__ piv, int64_t stride_piv, double* __restrict__ b,
             int64_t stride_b, int trans, int in_smem) {
  extern __shared__ double smem_x[];
  __shared__ TrsvSmem<double> tsm;
  const int sys = blockIdx.x / nrhs;
  const int r = blockIdx.x % nrhs;
  const double* A = lu + (int64_t)sys * stride_a;
  const int32_t* P = piv + (int64_t)sys * stride_piv;
  double* g = b + (int64_t)sys * stride_b + (int64_t)r * n;
  double* x = g;
  int32_t* sp = nullptr;
  if (in_smem) {
    x = smem_x;
    sp = reinterpret_cast<int32_t*>(smem_x + n);
    for (int i = threadIdx.x; i < n; i += blockDim.x) { x[i] = g[i]; sp[i] = P[i]; }
    __syncthreads();
  }
  const int32_t* pp = in_smem ? sp : P;
  if (!trans) {
    if (threadIdx.x == 0)
      for (int k = 0; k < n; ++k) {
        const int p = pp[k];
        if (p != k) { const double t = x[k]; x[k] = x[p]; x[p] = t; }
      }
    __syncthreads();
    cta_trsv<double>(A, n, n, /*lower=*/true, /*trans=*/false, /*unit=*/true, x, tsm);
    cta_trsv<double>(A, n, n, /*lower=*/false, /*trans=*/false, /*unit=*/false, x, tsm);
  } else {
    cta_trsv<double>(A, n, n, /*lower=*/false, /*trans=*/true, /*unit=*/false, x, tsm);
    cta_trsv<double>(A, n, n, /*lower=*/true, /*trans=*/true, /*unit=*/true, x, tsm);
    if (threadIdx.x == 0)
      for (int k = n - 1; k >= 0; --k) {
        const int p = pp[k];
        if (p != k) { const double t = x[k]; x[k] = x[p]; x[p] = t; }
      }
    __syncthreads();
  }
  if (in_smem)
    for (int i = threadIdx.x; i < n; i += blockDim.x) g[i] = x[i];
}

}  // namespace lxgb

using namespace lxgb;

extern "C" int lxgb_getrf_batched_f64(int64_t batch, int32_t n, double* a, int64_t stride_a,
                                      int32_t* piv, int64_t stride_piv, int32_t* info,
                                      void* stream) {
  LXGB_REQUIRE(batch >= 0 && n >= 0, "getrf: batch and n must be non-negative");
  if (batch == 0 || n == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(a && piv && info, "getrf: null pointer");
  LXGB_REQUIRE(stride_a >= (int64_t)n * n && stride_piv >= n, "getrf: stride too small");
  cudaStream_t st = as_stream(stream);
  if (n <= kSmallMax) {
    const size_t smem = (size_t)n * (n | 1) * sizeof(double);
    LXGB_CUDA_TRY(ensure_dynamic_smem(reinterpret_cast<const void*>(getrf_small_kernel), (int)smem),
                  "getrf: set smem");
    for (int64_t off = 0; off < batch; off += 65535LL * 1024) {
      const int64_t cnt = (batch - off < 65535LL * 1024) ? batch - off : 65535LL * 1024;
      getrf_small_kernel<<<(unsigned)cnt, kSmallThreads, smem, st>>>(
          n, a + off * stride_a, stride_a, piv + off * stride_piv, stride_piv, info + off);
    }
    return check_launch("getrf small");
  }
  for (int64_t s = 0; s < batch; ++s) {
    int rc = getrf_blocked(n, a + s * stride_a, piv + s * stride_piv, info + s, st);
    if (rc) return rc;
  }
  return LXGB_SUCCESSFUL;
}

extern "C" int lxgb_getrs_batched_f64(int64_t batch, int32_t n, int32_t nrhs, const double* lu,
                                      int64_t stride_a, const int32_t* piv, int64_t stride_piv,
                                      double* b, int64_t stride_b, int32_t trans, void* stream) {
  LXGB_REQUIRE(batch >= 0 && n >= 0 && nrhs >= 0, "getrs: negative size");
  if (batch == 0 || n == 0 || nrhs == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(lu && piv && b, "getrs: null pointer");
  LXGB_REQUIRE(trans == 0 || trans == 1, "getrs: trans must be 0 or 1");
  LXGB_REQUIRE(stride_a >= (int64_t)n * n && stride_piv >= n && stride_b >= (int64_t)n * nrhs,
               "getrs: stride too small");
  LXGB_REQUIRE(batch * (int64_t)nrhs < (1LL << 31), "getrs: too many vectors in one call");
  const size_t need = (size_t)n * (sizeof(double) + sizeof(int32_t));
  const int in_smem = need <= 160 * 1024;
  const size_t smem = in_smem ? need : 0;
  if (in_smem)
    LXGB_CUDA_TRY(ensure_dynamic_smem(reinterpret_cast<const void*>(getrs_kernel), (int)smem),
                  "getrs: set smem");
  getrs_kernel<<<(unsigned)(batch * nrhs), kSolveThreads, smem, as_stream(stream)>>>(
      n, nrhs, lu, stride_a, piv, stride_piv, b, stride_b, trans, in_smem);
  return check_launch("getrs");
}
