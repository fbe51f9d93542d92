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
#include <cooperative_groups.h>
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
  // pivot of step k in slot k & 1: row, |a| test for the reciprocal, a(p,k),
  // the old a(k,k), 1/a(p,k)
  __shared__ int s_p[2], s_recip[2];
  __shared__ double s_akk[2], s_old[2], s_rcp[2];
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
  const int tx = tid & 31, ty = tid >> 5;
  constexpr int kUpdWarps = (kSmallThreads >> 5) - 1;   // warps 1.. update columns >= k + 2
  // Warp 0: pivot of column k (rows >= k) into slot k & 1; `upd` first
  // applies step k - 1 to that column (the lookahead: the pivot search of
  // step k overlaps the other warps' update of step k - 1).
  auto pivot_warp = [&](int k, bool upd) {
    long long v = -1;
    int idx = INT_MAX;
    const double uk = upd ? A[(k - 1) * ld + k] : 0.0;
    for (int i = k + lane; i < n; i += 32) {
      double x = A[i * ld + k];
      if (upd) {
        x = fma(-A[i * ld + k - 1], uk, x);
        A[i * ld + k] = x;
      }
      const long long key = pivot_key(x);
      if (key > v) { v = key; idx = i; }
    }
    warp_argmax_first_key(v, idx);
    __syncwarp();
    if (lane == 0) {
      if (idx == INT_MAX) idx = k;  // column of NaNs: keep the row
      const int sl = k & 1;
      const double akk = A[idx * ld + k];
      s_p[sl] = idx;
      s_akk[sl] = akk;
      s_old[sl] = A[k * ld + k];
      // the reciprocal once per column (a division is a long FP64 sequence)
      s_recip[sl] = fabs(akk) >= DBL_MIN;
      s_rcp[sl] = 1.0 / akk;
      gp[k] = idx;
    }
  };
  __syncthreads();
  if (tid < 32) pivot_warp(0, false);
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    const int sl = k & 1;
    const int p = s_p[sl];
    const double akk = s_akk[sl];
    if ((__double_as_longlong(akk) << 1) != 0) {   // akk != 0 (NaN included), integer test
      if (p != k) {
        for (int j = tid; j < n; j += blockDim.x) {
          if (j == k) continue;
          const double t = A[k * ld + j];
          A[k * ld + j] = A[p * ld + j];
          A[p * ld + j] = t;
        }
      }
      const bool use_recip = s_recip[sl] != 0;
      const double r = s_rcp[sl];
      if (tid == 0) A[k * ld + k] = akk;
      for (int i = k + 1 + tid; i < n; i += blockDim.x) {
        const double v = (i == p) ? s_old[sl] : A[i * ld + k];
        A[i * ld + k] = scale_pivot(v, akk, r, use_recip);
      }
    } else if (my_info == 0) {
      my_info = k + 1;
    }
    __syncthreads();
    if (ty == 0) {
      // column k + 1 updated and its pivot found while the others update
      if (k + 1 < n) pivot_warp(k + 1, true);
    } else {
      // rank-1 update of columns >= k + 2; u(k,j) cached in registers.  Only
      // the 32-column chunks that hold trailing columns are visited (a
      // warp-uniform break): a predicated-off FP64 instruction still occupies
      // GB300's narrow FP64 pipe.
      const int nchunk = (n - k - 2 + 31) >> 5;
      double u[(kSmallMax + 31) / 32];
#pragma unroll
      for (int c = 0; c < (kSmallMax + 31) / 32; ++c) {
        if (c >= nchunk) break;
        const int j = k + 2 + tx + 32 * c;
        u[c] = (j < n) ? A[k * ld + j] : 0.0;
      }
      for (int i = k + 1 + (ty - 1); i < n; i += kUpdWarps) {
        const double l = A[i * ld + k];
#pragma unroll
        for (int c = 0; c < (kSmallMax + 31) / 32; ++c) {
          if (c >= nchunk) break;
          const int j = k + 2 + tx + 32 * c;
          if (j < n) A[i * ld + j] = fma(-l, u[c], A[i * ld + j]);
        }
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
// n <= kSmallMax with fewer matrices than SMs: a cluster of two CTAs per
// matrix, so twice as many SMs share the FP64 work.  CTA r of the pair holds
// the columns j = r, r + 2, ... (local column j >> 1, row stride odd) in its
// shared memory.  Step k: the CTA that owns column k searches the pivot,
// swaps rows k and p in its columns, scales column k and writes the
// multipliers l(i) and p into both CTAs' buffers (distributed shared memory);
// after one cluster barrier the other CTA swaps rows in its columns and both
// apply the rank-1 update to their trailing columns.  Every element receives
// the same FMA chain as in getrf_small_kernel, so factors and pivots are
// bit-identical to it (and to getf2).  The l and p buffers alternate with the
// parity of k: the owner of step k + 2 (the same CTA) rewrites them only
// after both CTAs have passed the barrier of step k + 1.
// ---------------------------------------------------------------------------
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(kSmallThreads)
getrf_small_pair_kernel(int n, double* __restrict__ a, int64_t stride_a,
                        int32_t* __restrict__ piv, int64_t stride_piv,
                        int32_t* __restrict__ info) {
  namespace cg = cooperative_groups;
  extern __shared__ double smem_lu[];
  __shared__ double s_l[2][kSmallMax];
  __shared__ int s_p[2];
  __shared__ int s_info[2];
  __shared__ int s_pl, s_recip;
  __shared__ double s_akk, s_old, s_rcp;
  cg::cluster_group cluster = cg::this_cluster();
  const int r = (int)cluster.block_rank();
  const int peer = r ^ 1;
  const int ncl = (n + 1 - r) >> 1;          // columns j = r, r + 2, ... < n
  const int ldl = ((n + 1) >> 1) | 1;
  double* A = smem_lu;
  const int tid = threadIdx.x, lane = tid & 31;
  const int tx = tid & 31, ty = tid >> 5;
  const int64_t b = blockIdx.x >> 1;
  double* g = a + b * stride_a;
  int32_t* gp = piv + b * stride_piv;
  double* peer_l = cluster.map_shared_rank(&s_l[0][0], peer);
  int* peer_p = cluster.map_shared_rank(&s_p[0], peer);
  for (int e = tid; e < n * ncl; e += blockDim.x) {
    const int i = e / ncl, jl = e - i * ncl;
    A[i * ldl + jl] = g[(int64_t)i * n + 2 * jl + r];
  }
  int my_info = 0;
  cluster.sync();   // both CTAs run before any remote store
  for (int k = 0; k < n; ++k) {
    const int buf = k & 1;
    if (r == (k & 1)) {
      const int kl = k >> 1;
      if (tid < 32) {
        long long v = -1;
        int idx = INT_MAX;
        for (int i = k + lane; i < n; i += 32) {
          const long long x = pivot_key(A[i * ldl + kl]);
          if (x > v) { v = x; idx = i; }
        }
        warp_argmax_first_key(v, idx);
        if (lane == 0) {
          if (idx == INT_MAX) idx = k;  // column of NaNs: keep the row
          s_pl = idx;
          const double akk = A[idx * ldl + kl];
          s_akk = akk;
          s_old = A[k * ldl + kl];
          s_recip = fabs(akk) >= DBL_MIN;
          s_rcp = 1.0 / akk;
          gp[k] = idx;
        }
      }
      __syncthreads();
      const int p = s_pl;
      const double akk = s_akk;
      if (akk != 0.0) {
        if (p != k) {
          for (int jl = tid; jl < ncl; jl += blockDim.x) {
            if (jl == kl) continue;
            const double t = A[k * ldl + jl];
            A[k * ldl + jl] = A[p * ldl + jl];
            A[p * ldl + jl] = t;
          }
        }
        const bool use_recip = s_recip != 0;
        const double rcp = s_rcp;
        if (tid == 0) A[k * ldl + kl] = akk;
        for (int i = k + 1 + tid; i < n; i += blockDim.x) {
          const double v = (i == p) ? s_old : A[i * ldl + kl];
          const double lv = scale_pivot(v, akk, rcp, use_recip);
          A[i * ldl + kl] = lv;
          s_l[buf][i] = lv;
          peer_l[buf * kSmallMax + i] = lv;
        }
      } else {
        if (my_info == 0) my_info = k + 1;
        for (int i = k + 1 + tid; i < n; i += blockDim.x) {
          const double lv = A[i * ldl + kl];
          s_l[buf][i] = lv;
          peer_l[buf * kSmallMax + i] = lv;
        }
      }
      if (tid == 0) {
        const int pe = (akk != 0.0) ? p : k;   // the row the other CTA swaps with k
        s_p[buf] = pe;
        peer_p[buf] = pe;
      }
    }
    cluster.sync();
    if (r != (k & 1)) {
      const int p = s_p[buf];
      if (p != k) {
        for (int jl = tid; jl < ncl; jl += blockDim.x) {
          const double t = A[k * ldl + jl];
          A[k * ldl + jl] = A[p * ldl + jl];
          A[p * ldl + jl] = t;
        }
        __syncthreads();
      }
    }
    // rank-1 update of this CTA's trailing columns j = 2 jl + r > k
    const int jl0 = (k + 2 - r) >> 1;
    const int nchunk = (ncl - jl0 + 31) >> 5;
    constexpr int kMaxChunk = ((kSmallMax + 1) / 2 + 31) / 32;
    double u[kMaxChunk];
#pragma unroll
    for (int c = 0; c < kMaxChunk; ++c) {
      if (c >= nchunk) break;
      const int jl = jl0 + tx + 32 * c;
      u[c] = (jl < ncl) ? A[k * ldl + jl] : 0.0;
    }
    for (int i = k + 1 + ty; i < n; i += (kSmallThreads >> 5)) {
      const double l = s_l[buf][i];
#pragma unroll
      for (int c = 0; c < kMaxChunk; ++c) {
        if (c >= nchunk) break;
        const int jl = jl0 + tx + 32 * c;
        if (jl < ncl) A[i * ldl + jl] = fma(-l, u[c], A[i * ldl + jl]);
      }
    }
    __syncthreads();
  }
  for (int e = tid; e < n * ncl; e += blockDim.x) {
    const int i = e / ncl, jl = e - i * ncl;
    g[(int64_t)i * n + 2 * jl + r] = A[i * ldl + jl];
  }
  // info = the first zero pivot over both CTAs' steps
  if (tid == 0) *cluster.map_shared_rank(&s_info[r], 0) = my_info;
  cluster.sync();
  if (r == 0 && tid == 0) {
    const int i0 = s_info[0], i1 = s_info[1];
    info[b] = (i0 == 0) ? i1 : (i1 == 0 ? i0 : min(i0, i1));
  }
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
  __shared__ long long s_v[32];
  __shared__ int s_i[32];
  __shared__ int s_p, s_recip;
  __shared__ double s_akk, s_old, s_rcp;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nwarps = blockDim.x >> 5;
  for (int k = j0; k < j0 + nb; ++k) {
    long long v = -1;
    int idx = INT_MAX;
    for (int i = k + tid; i < n; i += blockDim.x) {
      const long long x = pivot_key(a[(int64_t)i * n + k]);
      if (x > v) { v = x; idx = i; }
    }
    warp_argmax_first_key(v, idx);
    if (lane == 0) { s_v[warp] = v; s_i[warp] = idx; }
    __syncthreads();
    if (warp == 0) {
      v = lane < nwarps ? s_v[lane] : -1;
      idx = lane < nwarps ? s_i[lane] : INT_MAX;
      warp_argmax_first_key(v, idx);
      if (lane == 0) {
        if (idx == INT_MAX) idx = k;
        s_p = idx;
        const double akk = a[(int64_t)idx * n + k];
        s_akk = akk;
        s_old = a[(int64_t)k * n + k];
        s_recip = fabs(akk) >= DBL_MIN;
        s_rcp = 1.0 / akk;
        piv[k] = idx;
        if (akk == 0.0 && *info == 0) *info = k + 1;
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
      const bool use_recip = s_recip != 0;
      const double r = s_rcp;
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

// ---------------------------------------------------------------------------
// getrs for n <= kSmallMax: one CTA per system, the factors staged in shared
// memory, one warp per right-hand side with x held in registers (lane l owns
// rows l, l + 32, ...).  Each substitution step broadcasts the finished
// unknown with a shuffle and updates the later rows with one FMA per lane, so
// the dependent chain per step is a shuffle and an FMA; the diagonal of U is
// inverted up front, off that chain (x_t * (1 / u_tt) instead of x_t / u_tt:
// within one rounding of the quotient).  The row interchanges are composed
// once into a gather index.
// ---------------------------------------------------------------------------
constexpr int kSmallRegs = (kSmallMax + 31) / 32;

__global__ void __launch_bounds__(kSolveThreads)
getrs_small_kernel(int n, int nrhs, const double* __restrict__ lu, int64_t stride_a,
                   const int32_t* __restrict__ piv, int64_t stride_piv, double* __restrict__ b,
                   int64_t stride_b, int trans) {
  extern __shared__ double smem_x[];
  const int ld = n | 1;
  double* T = smem_x;                                   // n × ld
  double* rinv = T + (int64_t)n * ld;                   // 1 / u_tt
  int* perm = reinterpret_cast<int*>(rinv + n);         // x_perm[i] = b[perm[i]]
  const int sys = blockIdx.x;
  const double* A = lu + (int64_t)sys * stride_a;
  const int32_t* P = piv + (int64_t)sys * stride_piv;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  for (int e = tid; e < n * n; e += blockDim.x) {
    const int i = e / n, j = e - i * n;
    T[i * ld + j] = A[e];
  }
  if (tid == 0) {
    // compose the interchanges: forward order for P b, and its inverse is
    // applied by scattering through the same index for Pᵀ y
    for (int i = 0; i < n; ++i) perm[i] = i;
    for (int k = 0; k < n; ++k) {
      const int p = P[k];
      if (p != k) { const int t = perm[k]; perm[k] = perm[p]; perm[p] = t; }
    }
  }
  __syncthreads();
  for (int i = tid; i < n; i += blockDim.x) rinv[i] = 1.0 / T[i * ld + i];
  __syncthreads();
  for (int rr = warp; rr < nrhs; rr += nw) {
    double* g = b + (int64_t)sys * stride_b + (int64_t)rr * n;
    double x[kSmallRegs];
    if (!trans) {
#pragma unroll
      for (int m = 0; m < kSmallRegs; ++m) {
        const int i = 32 * m + lane;
        x[m] = (i < n) ? g[perm[i]] : 0.0;
      }
      // L y = P b (unit lower): column t of L is read down the rows
#pragma unroll
      for (int tb = 0; tb < kSmallRegs; ++tb) {
        if (32 * tb >= n) break;
        for (int tt = 0; tt < 32; ++tt) {
          const int t = 32 * tb + tt;
          if (t >= n) break;
          const double xt = __shfl_sync(0xffffffffu, x[tb], tt);
#pragma unroll
          for (int m = tb; m < kSmallRegs; ++m) {
            const int i = 32 * m + lane;
            if (i > t && i < n) x[m] = fma(-T[i * ld + t], xt, x[m]);
          }
        }
      }
      // U x = y
#pragma unroll
      for (int tb = kSmallRegs - 1; tb >= 0; --tb) {
        if (32 * tb >= n) continue;
        for (int tt = 31; tt >= 0; --tt) {
          const int t = 32 * tb + tt;
          if (t >= n) continue;
          if (lane == tt) x[tb] *= rinv[t];
          const double xt = __shfl_sync(0xffffffffu, x[tb], tt);
#pragma unroll
          for (int m = 0; m <= tb; ++m) {
            const int i = 32 * m + lane;
            if (i < t) x[m] = fma(-T[i * ld + t], xt, x[m]);
          }
        }
      }
      __syncwarp();
#pragma unroll
      for (int m = 0; m < kSmallRegs; ++m) {
        const int i = 32 * m + lane;
        if (i < n) g[i] = x[m];
      }
    } else {
#pragma unroll
      for (int m = 0; m < kSmallRegs; ++m) {
        const int i = 32 * m + lane;
        x[m] = (i < n) ? g[i] : 0.0;
      }
      // Uᵀ z = b: column t of Uᵀ is row t of U
#pragma unroll
      for (int tb = 0; tb < kSmallRegs; ++tb) {
        if (32 * tb >= n) break;
        for (int tt = 0; tt < 32; ++tt) {
          const int t = 32 * tb + tt;
          if (t >= n) break;
          if (lane == tt) x[tb] *= rinv[t];
          const double xt = __shfl_sync(0xffffffffu, x[tb], tt);
#pragma unroll
          for (int m = tb; m < kSmallRegs; ++m) {
            const int i = 32 * m + lane;
            if (i > t && i < n) x[m] = fma(-T[t * ld + i], xt, x[m]);
          }
        }
      }
      // Lᵀ w = z (unit upper)
#pragma unroll
      for (int tb = kSmallRegs - 1; tb >= 0; --tb) {
        if (32 * tb >= n) continue;
        for (int tt = 31; tt >= 0; --tt) {
          const int t = 32 * tb + tt;
          if (t >= n) continue;
          const double xt = __shfl_sync(0xffffffffu, x[tb], tt);
#pragma unroll
          for (int m = 0; m <= tb; ++m) {
            const int i = 32 * m + lane;
            if (i < t) x[m] = fma(-T[t * ld + i], xt, x[m]);
          }
        }
      }
      // x = Pᵀ w: x[perm[i]] = w[i]
      __syncwarp();
#pragma unroll
      for (int m = 0; m < kSmallRegs; ++m) {
        const int i = 32 * m + lane;
        if (i < n) g[perm[i]] = x[m];
      }
    }
  }
}

}  // namespace lxgb

using namespace lxgb;

// 1: batches of at most half the SM count with n in [32, 168] run on two-CTA
// clusters; 0 (the default): one CTA per matrix.  The pair halves each SM's
// FP64 work but adds a cluster barrier and a distributed-shared-memory
// exchange to every column; on the 64 × n = 128 batch it factors in 0.44 ms
// against 0.33 ms for one CTA with the lookahead pivot search.
static int g_getrf_pair = 0;

extern "C" int lxgb_getrf_set_pair(int32_t on) {
  g_getrf_pair = on ? 1 : 0;
  return LXGB_SUCCESSFUL;
}

extern "C" int lxgb_getrf_batched_f64(int64_t batch, int32_t n, double* a, int64_t stride_a,
                                      int32_t* piv, int64_t stride_piv, int32_t* info,
                                      void* stream) {
  LXGB_REQUIRE(batch >= 0 && n >= 0, "getrf: batch and n must be non-negative");
  if (batch == 0 || n == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(a && piv && info, "getrf: null pointer");
  LXGB_REQUIRE(stride_a >= (int64_t)n * n && stride_piv >= n, "getrf: stride too small");
  cudaStream_t st = as_stream(stream);
  if (n <= kSmallMax && n >= 32 && 2 * batch <= sm_count() && g_getrf_pair) {
    // fewer matrices than SMs: two CTAs (a cluster) per matrix
    const size_t smem = (size_t)n * (((n + 1) >> 1) | 1) * sizeof(double);
    LXGB_CUDA_TRY(ensure_dynamic_smem(reinterpret_cast<const void*>(getrf_small_pair_kernel),
                                      (int)smem),
                  "getrf pair: set smem");
    getrf_small_pair_kernel<<<(unsigned)(2 * batch), kSmallThreads, smem, st>>>(
        n, a, stride_a, piv, stride_piv, info);
    return check_launch("getrf small pair");
  }
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
  if (n <= kSmallMax && batch < (1LL << 31)) {
    const size_t smem = (size_t)n * (n | 1) * sizeof(double) + (size_t)n * sizeof(double) +
                        (size_t)n * sizeof(int32_t);
    LXGB_CUDA_TRY(ensure_dynamic_smem(reinterpret_cast<const void*>(getrs_small_kernel), (int)smem),
                  "getrs small: set smem");
    getrs_small_kernel<<<(unsigned)batch, kSolveThreads, smem, as_stream(stream)>>>(
        n, nrhs, lu, stride_a, piv, stride_piv, b, stride_b, trans);
    return check_launch("getrs small");
  }
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
