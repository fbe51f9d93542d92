// Mixed-precision LU: FP32 storage, partial pivoting, trailing updates on the
// tcgen05 tensor cores (TF32 products, FP32 accumulation), and the matching
// FP32 solve used as the preconditioner of FP64 GMRES-IR.
//
// Right-looking blocked LU with 64-column panels:
//   panel_getf2_cluster_reg_kernel — getf2 on the panel with each row in
//                            one thread's registers across a thread-block
//                            cluster (up to 16 CTAs × 512 rows); pivot
//                            search and pivot row exchanged through
//                            distributed shared memory.
//   panel_getf2_cluster_kernel — the same with the panel in the cluster's
//                            shared memory (taller panels); and
//                            panel_getf2_f32_kernel (one CTA, panel in global
//                            memory) for panels too tall for either.
//   laswp_f32_kernel       — the panel's row interchanges on the other columns
//   launch_inv_diag_lower  — U12 = L11^{-1} A12 in place, and U12ᵀ into a
//                            K-major buffer for the GEMM (ir.cu)
//   gemm_tf32_nt           — A22 -= L21 U12 on the tensor cores
#include <cooperative_groups.h>
#include <float.h>
#include <limits.h>

#include <map>
#include <mutex>
#include <tuple>

#include "common.cuh"
#include "tc_gemm.cuh"
#include "tri.cuh"

namespace lxgb {

constexpr int kLu32NB = 64;
constexpr int kLu32PanelThreads = 1024;

__device__ __forceinline__ void warp_argmax_first_f(float& v, int& idx) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float ov = __shfl_xor_sync(0xffffffffu, v, o);
    const int oi = __shfl_xor_sync(0xffffffffu, idx, o);
    if (ov > v || (ov == v && oi < idx)) { v = ov; idx = oi; }
  }
}

__global__ void __launch_bounds__(kLu32PanelThreads)
panel_getf2_f32_kernel(int n, int j0, int nb, float* __restrict__ a, int32_t* __restrict__ piv,
                       int32_t* __restrict__ info) {
  __shared__ float s_v[32];
  __shared__ int s_i[32];
  __shared__ int s_p;
  __shared__ float s_akk, s_old;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nwarps = blockDim.x >> 5;
  for (int k = j0; k < j0 + nb; ++k) {
    float v = -1.0f;
    int idx = INT_MAX;
    for (int i = k + tid; i < n; i += blockDim.x) {
      const float x = fabsf(a[(int64_t)i * n + k]);
      if (x > v) { v = x; idx = i; }
    }
    warp_argmax_first_f(v, idx);
    if (lane == 0) { s_v[warp] = v; s_i[warp] = idx; }
    __syncthreads();
    if (warp == 0) {
      v = lane < nwarps ? s_v[lane] : -1.0f;
      idx = lane < nwarps ? s_i[lane] : INT_MAX;
      warp_argmax_first_f(v, idx);
      if (lane == 0) {
        if (idx == INT_MAX) idx = k;
        s_p = idx;
        s_akk = a[(int64_t)idx * n + k];
        s_old = a[(int64_t)k * n + k];
        piv[k] = idx;
        if (s_akk == 0.0f && *info == 0) *info = k + 1;
      }
    }
    __syncthreads();
    const int p = s_p;
    const float akk = s_akk;
    if (akk != 0.0f) {
      if (p != k) {
        for (int j = j0 + tid; j < j0 + nb; j += blockDim.x) {
          if (j == k) continue;
          const float t = a[(int64_t)k * n + j];
          a[(int64_t)k * n + j] = a[(int64_t)p * n + j];
          a[(int64_t)p * n + j] = t;
        }
      }
      const float r = 1.0f / akk;
      if (tid == 0) a[(int64_t)k * n + k] = akk;
      for (int i = k + 1 + tid; i < n; i += blockDim.x) {
        const float x = (i == p) ? s_old : a[(int64_t)i * n + k];
        a[(int64_t)i * n + k] = x * r;
      }
    }
    __syncthreads();
    const int w = j0 + nb - (k + 1);
    if (w > 0) {
      // rows i > k: one warp per row, lanes along the remaining panel columns
      for (int i = k + 1 + warp; i < n; i += nwarps) {
        const float l = a[(int64_t)i * n + k];
        for (int jj = lane; jj < w; jj += 32) {
          const int j = k + 1 + jj;
          a[(int64_t)i * n + j] = fmaf(-l, a[(int64_t)k * n + j], a[(int64_t)i * n + j]);
        }
      }
    }
    __syncthreads();
  }
}

namespace cg = cooperative_groups;

constexpr int kPanelCluThreads = 512;
constexpr int kPanelLd = kLu32NB + 1;  // padded row: column reads are conflict-free
constexpr int kPanelCluMax = 16;
constexpr size_t kPanelCluSmemMax = 200 * 1024;

// getf2 on the m×nb panel at (j0, j0) (m = n - j0), rows split over the
// cluster's CTAs (rows_per_cta each) and kept in shared memory for the whole
// panel.  Per column: each CTA's first max |a| is published; after a cluster
// barrier every CTA reduces the candidates (same order everywhere: first row
// of max |a|, as isamax), copies the pivot row and row kk out of their owners'
// shared memory, and after a second barrier the owners swap them and every CTA
// scales and updates its own rows.  Candidates are double-buffered by column
// parity, so one barrier pair per column suffices.  Arithmetic matches
// panel_getf2_f32_kernel (reciprocal scaling, fmaf rank-1 updates).
__global__ void __launch_bounds__(kPanelCluThreads)
panel_getf2_cluster_kernel(int n, int j0, int nb, int rows_per_cta, float* __restrict__ a,
                           int32_t* __restrict__ piv, int32_t* __restrict__ info) {
  extern __shared__ float P[];
  __shared__ float cand_v[2];
  __shared__ int cand_i[2];
  __shared__ float rowp[kLu32NB], rowk[kLu32NB];
  __shared__ float s_wv[kPanelCluThreads / 32];
  __shared__ int s_wi[kPanelCluThreads / 32];
  __shared__ int s_p;
  cg::cluster_group cluster = cg::this_cluster();
  const int ncta = (int)cluster.num_blocks();
  const int rank = (int)cluster.block_rank();
  const int m = n - j0;
  const int R = rows_per_cta;
  const int r0 = rank * R;
  const int mloc = max(0, min(R, m - r0));
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nwarps = blockDim.x >> 5;
  for (int e = tid; e < mloc * kLu32NB; e += blockDim.x) {
    const int i = e / kLu32NB, j = e % kLu32NB;
    P[i * kPanelLd + j] = (j < nb) ? a[(int64_t)(j0 + r0 + i) * n + j0 + j] : 0.0f;
  }
  __syncthreads();
  for (int kk = 0; kk < nb; ++kk) {
    const int par = kk & 1;
    float v = -1.0f;
    int idx = INT_MAX;
    for (int i = tid; i < mloc; i += blockDim.x) {
      if (r0 + i >= kk) {
        const float x = fabsf(P[i * kPanelLd + kk]);
        if (x > v) { v = x; idx = r0 + i; }
      }
    }
    warp_argmax_first_f(v, idx);
    if (lane == 0) { s_wv[warp] = v; s_wi[warp] = idx; }
    __syncthreads();
    if (warp == 0) {
      v = lane < nwarps ? s_wv[lane] : -1.0f;
      idx = lane < nwarps ? s_wi[lane] : INT_MAX;
      warp_argmax_first_f(v, idx);
      if (lane == 0) { cand_v[par] = v; cand_i[par] = idx; }
    }
    cluster.sync();
    if (warp == 0) {
      float cv = -1.0f;
      int ci = INT_MAX;
      if (lane < ncta) {
        cv = *cluster.map_shared_rank(&cand_v[par], lane);
        ci = *cluster.map_shared_rank(&cand_i[par], lane);
      }
      warp_argmax_first_f(cv, ci);
      if (lane == 0) s_p = (ci == INT_MAX) ? kk : ci;
    }
    __syncthreads();
    const int p = s_p;
    const int own_p = p / R, loc_p = p - own_p * R;
    const int own_k = kk / R, loc_k = kk - own_k * R;
    if (tid < kLu32NB) {
      rowp[tid] = cluster.map_shared_rank(P, own_p)[loc_p * kPanelLd + tid];
    } else if (tid < 2 * kLu32NB) {
      rowk[tid - kLu32NB] = cluster.map_shared_rank(P, own_k)[loc_k * kPanelLd + tid - kLu32NB];
    }
    cluster.sync();
    const float akk = rowp[kk];
    if (akk != 0.0f && p != kk) {
      if (rank == own_k && tid < kLu32NB) P[loc_k * kPanelLd + tid] = rowp[tid];
      if (rank == own_p && tid < kLu32NB) P[loc_p * kPanelLd + tid] = rowk[tid];
    }
    if (rank == 0 && tid == 0) {
      piv[j0 + kk] = j0 + p;
      if (akk == 0.0f && *info == 0) *info = j0 + kk + 1;
    }
    __syncthreads();
    const float rcp = (akk != 0.0f) ? 1.0f / akk : 0.0f;
    for (int i = tid; i < mloc; i += blockDim.x) {
      if (r0 + i > kk) {
        float* row = P + i * kPanelLd;
        float l = row[kk];
        if (akk != 0.0f) {
          l *= rcp;
          row[kk] = l;
        }
        for (int j = kk + 1; j < nb; ++j) row[j] = fmaf(-l, rowp[j], row[j]);
      }
    }
    __syncthreads();
  }
  for (int e = tid; e < mloc * kLu32NB; e += blockDim.x) {
    const int i = e / kLu32NB, j = e % kLu32NB;
    if (j < nb) a[(int64_t)(j0 + r0 + i) * n + j0 + j] = P[i * kPanelLd + j];
  }
}

// The same panel factorisation with every panel row held in the registers
// of one thread (a CTA owns up to 512 rows, a cluster up to 16 CTAs): the
// rank-1 update of a column is 63 independent FMAs per thread instead of a
// loop over shared memory.  Per column each CTA publishes, in a slot
// double-buffered by column parity, its first max |a| together with that
// row (and row kk, from its owner); after the column's single cluster
// barrier every CTA reduces the candidates in the same order, copies the
// winning row through distributed shared memory, and the owner of the pivot
// row takes row kk.  The global first max is also its CTA's first max, so the
// published row is the pivot row.  Same arithmetic and pivot choice (first
// row of max |a|, NaN never chosen) as the shared-memory kernels.
constexpr int kRegPanelThreads = 512;

// CLUSTER = false: a one-CTA panel (m <= 512) without the cluster barrier's
// cluster-scope release/acquire; the exchange slots are then local.
template <bool CLUSTER>
__global__ void __launch_bounds__(kRegPanelThreads, 1)
panel_getf2_cluster_reg_kernel(int n, int j0, int nb, int rows_per_cta, float* __restrict__ a,
                               int32_t* __restrict__ piv, int32_t* __restrict__ info) {
  __shared__ float cand_v[2];
  __shared__ int cand_i[2];
  __shared__ __align__(16) float xbuf[2][2][kLu32NB];  // [parity][pivot row, row kk]
  __shared__ __align__(16) float rowp[kLu32NB];
  __shared__ float s_wv[kRegPanelThreads / 32];
  __shared__ int s_wi[kRegPanelThreads / 32];
  __shared__ int s_p;
  cg::cluster_group cluster = cg::this_cluster();
  const int ncta = CLUSTER ? (int)cluster.num_blocks() : 1;
  const int rank = CLUSTER ? (int)cluster.block_rank() : 0;
  // shared memory of CTA `rk` of the cluster (this CTA's own without one)
  auto remote = [&](auto* ptr, int rk) { return CLUSTER ? cluster.map_shared_rank(ptr, rk) : ptr; };
  const int m = n - j0;
  const int R = rows_per_cta;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int gi = rank * R + tid;  // panel row held by this thread
  const bool has_row = tid < R && gi < m;
  float r[kLu32NB];
  if (has_row) {
    const float* src = a + (int64_t)(j0 + gi) * n + j0;
    if (nb == kLu32NB) {
#pragma unroll
      for (int q = 0; q < kLu32NB / 4; ++q) {
        const float4 v = reinterpret_cast<const float4*>(src)[q];
        r[4 * q] = v.x;
        r[4 * q + 1] = v.y;
        r[4 * q + 2] = v.z;
        r[4 * q + 3] = v.w;
      }
    } else {
#pragma unroll
      for (int j = 0; j < kLu32NB; ++j) r[j] = (j < nb) ? src[j] : 0.0f;
    }
  } else {
#pragma unroll
    for (int j = 0; j < kLu32NB; ++j) r[j] = 0.0f;
  }
#pragma unroll
  for (int kk = 0; kk < kLu32NB; ++kk) {
    if (kk < nb) {  // uniform over the cluster
      const int par = kk & 1;
      // this CTA's first max |a| in column kk, and its row published with it
      float v = -1.0f;
      int idx = INT_MAX;
      if (has_row && gi >= kk) {
        const float x = fabsf(r[kk]);
        if (x > v) { v = x; idx = gi; }
      }
      warp_argmax_first_f(v, idx);
      if (lane == 0) { s_wv[warp] = v; s_wi[warp] = idx; }
      __syncthreads();
      if (warp == 0) {
        v = lane < kRegPanelThreads / 32 ? s_wv[lane] : -1.0f;
        idx = lane < kRegPanelThreads / 32 ? s_wi[lane] : INT_MAX;
        warp_argmax_first_f(v, idx);
        if (lane == 0) { cand_v[par] = v; cand_i[par] = idx; }
      }
      __syncthreads();
      if (has_row && gi == cand_i[par]) {
#pragma unroll
        for (int j = 0; j < kLu32NB; ++j) xbuf[par][0][j] = r[j];
      }
      if (has_row && gi == kk) {
#pragma unroll
        for (int j = 0; j < kLu32NB; ++j) xbuf[par][1][j] = r[j];
      }
      if (CLUSTER) {
        cluster.sync();  // the one cluster barrier of this column
      } else {
        __syncthreads();
      }
      if (warp == 0) {
        float cv = -1.0f;
        int ci = INT_MAX;
        if (lane < ncta) {
          cv = *remote(&cand_v[par], lane);
          ci = *remote(&cand_i[par], lane);
        }
        warp_argmax_first_f(cv, ci);
        if (lane == 0) s_p = ci;  // INT_MAX: no candidate (all NaN), keep row kk
      }
      __syncthreads();
      const bool none = s_p == INT_MAX;
      const int p = none ? kk : s_p;
      const int own_p = p / R, own_k = kk / R;
      // pivot row: the winning CTA's published row (row kk itself when none)
      if (tid < kLu32NB)
        rowp[tid] = remote(&xbuf[par][none ? 1 : 0][0], none ? own_k : own_p)[tid];
      __syncthreads();
      const float akk = rowp[kk];
      if (akk != 0.0f && p != kk) {
        if (has_row && gi == kk) {
#pragma unroll
          for (int j = 0; j < kLu32NB; ++j) r[j] = rowp[j];
        } else if (has_row && gi == p) {
          const float* rk = remote(&xbuf[par][1][0], own_k);
#pragma unroll
          for (int j = 0; j < kLu32NB; ++j) r[j] = rk[j];
        }
      }
      if (rank == 0 && tid == 0) {
        piv[j0 + kk] = j0 + p;
        if (akk == 0.0f && *info == 0) *info = j0 + kk + 1;
      }
      if (has_row && gi > kk) {
        float l = r[kk];
        if (akk != 0.0f) {
          l *= 1.0f / akk;
          r[kk] = l;
        }
#pragma unroll
        for (int j = kk + 1; j < kLu32NB; ++j) r[j] = fmaf(-l, rowp[j], r[j]);
      }
    }
  }
  if (has_row) {
    float* dst = a + (int64_t)(j0 + gi) * n + j0;
    if (nb == kLu32NB) {
#pragma unroll
      for (int q = 0; q < kLu32NB / 4; ++q)
        reinterpret_cast<float4*>(dst)[q] =
            make_float4(r[4 * q], r[4 * q + 1], r[4 * q + 2], r[4 * q + 3]);
    } else {
#pragma unroll
      for (int j = 0; j < kLu32NB; ++j)
        if (j < nb) dst[j] = r[j];
    }
  }
}

// Cluster geometry for an m-row panel: 0 when it does not fit (or the device
// cannot co-schedule the cluster), else the CTA count (rows_per_cta set).
static int panel_cluster_size(int m, int* rows_per_cta) {
  int c = (m + kPanelCluThreads - 1) / kPanelCluThreads;
  c = c < 1 ? 1 : (c > kPanelCluMax ? kPanelCluMax : c);
  const int r = (m + c - 1) / c;
  if ((size_t)r * kPanelLd * sizeof(float) > kPanelCluSmemMax) return 0;
  *rows_per_cta = r;
  return c;
}

// Whether a cluster of c CTAs with `smem` bytes each can be co-scheduled on the
// current device (cached: the attribute and occupancy queries cost host time
// on every panel otherwise).
static bool panel_cluster_fits(int c, size_t smem) {
  static std::mutex mu;
  static std::map<std::tuple<int, int, size_t>, bool> known;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
  std::lock_guard<std::mutex> lock(mu);
  const auto key = std::make_tuple(dev, c, smem);
  auto it = known.find(key);
  if (it != known.end()) return it->second;
  bool ok = cudaFuncSetAttribute(panel_getf2_cluster_kernel,
                                 cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess &&
            ensure_dynamic_smem(reinterpret_cast<const void*>(panel_getf2_cluster_kernel),
                                (int)smem) == cudaSuccess;
  if (ok) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)c);
    cfg.blockDim = dim3(kPanelCluThreads);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)c;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int nclusters = 0;
    ok = cudaOccupancyMaxActiveClusters(&nclusters, panel_getf2_cluster_kernel, &cfg) ==
             cudaSuccess &&
         nclusters >= 1;
  }
  if (!ok) cudaGetLastError();
  known[key] = ok;
  return ok;
}

static bool reg_cluster_fits(int c) {
  static std::mutex mu;
  static std::map<std::pair<int, int>, bool> known;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
  std::lock_guard<std::mutex> lock(mu);
  const auto key = std::make_pair(dev, c);
  auto it = known.find(key);
  if (it != known.end()) return it->second;
  bool ok = cudaFuncSetAttribute(panel_getf2_cluster_reg_kernel<true>,
                                 cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess;
  if (ok) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)c);
    cfg.blockDim = dim3(kRegPanelThreads);
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)c;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int nclusters = 0;
    ok = cudaOccupancyMaxActiveClusters(&nclusters, panel_getf2_cluster_reg_kernel<true>, &cfg) ==
             cudaSuccess &&
         nclusters >= 1;
  }
  if (!ok) cudaGetLastError();
  known[key] = ok;
  return ok;
}

// Register-resident panel when every row fits one thread of a <=16-CTA
// cluster; 0 on launch, -1 when the caller must use another kernel.
static int launch_panel_cluster_reg(int n, int j0, int nb, float* a, int32_t* piv, int32_t* info,
                                    cudaStream_t st) {
  const int m = n - j0;
  int c = (m + kRegPanelThreads - 1) / kRegPanelThreads;
  if (c < 1) c = 1;
  if (c > kPanelCluMax) return -1;
  const int r = (m + c - 1) / c;
  if (c == 1) {
    panel_getf2_cluster_reg_kernel<false><<<1, kRegPanelThreads, 0, st>>>(n, j0, nb, r, a, piv,
                                                                          info);
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
  }
  if (!reg_cluster_fits(c)) return -1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)c);
  cfg.blockDim = dim3(kRegPanelThreads);
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)c;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (cudaLaunchKernelEx(&cfg, panel_getf2_cluster_reg_kernel<true>, n, j0, nb, r, a, piv, info) !=
      cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
  return 0;
}

static int launch_panel_cluster(int n, int j0, int nb, float* a, int32_t* piv, int32_t* info,
                                cudaStream_t st) {
  if (launch_panel_cluster_reg(n, j0, nb, a, piv, info, st) == 0) return 0;
  int r = 0;
  const int c = panel_cluster_size(n - j0, &r);
  if (c == 0) return -1;
  const size_t smem = (size_t)r * kPanelLd * sizeof(float);
  if (!panel_cluster_fits(c, smem)) return -1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)c);
  cfg.blockDim = dim3(kPanelCluThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)c;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (cudaLaunchKernelEx(&cfg, panel_getf2_cluster_kernel, n, j0, nb, r, a, piv, info) !=
      cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
  return 0;
}

__global__ void laswp_f32_kernel(int n, int j0, int nb, float* __restrict__ a,
                                 const int32_t* __restrict__ piv) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int outside = n - nb;
  if (c >= outside) return;
  const int j = (c < j0) ? c : c + nb;
  for (int k = j0; k < j0 + nb; ++k) {
    const int p = piv[k];
    if (p != k) {
      const float t = a[(int64_t)k * n + j];
      a[(int64_t)k * n + j] = a[(int64_t)p * n + j];
      a[(int64_t)p * n + j] = t;
    }
  }
}

__global__ void cvt_f64_to_f32_kernel(int64_t count, const double* __restrict__ src,
                                      float* __restrict__ dst) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = (float)src[i];
}

__global__ void zero_i32_kernel(int32_t* p, int count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) p[i] = 0;
}

// getrs with an FP32 factor on FP64 vectors: x = U^{-1} L^{-1} P b, computed
// in FP32 (the preconditioner apply of GMRES-IR).  One CTA per vector.
__global__ void __launch_bounds__(256)
getrs_f32_kernel(int n, const float* __restrict__ lu, const int32_t* __restrict__ piv,
                 const double* __restrict__ b, double* __restrict__ x) {
  extern __shared__ float xs[];
  __shared__ TrsvSmem<float> tsm;
  const double* bc = b + (int64_t)blockIdx.x * n;
  double* xc = x + (int64_t)blockIdx.x * n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) xs[i] = (float)bc[i];
  __syncthreads();
  if (threadIdx.x == 0)
    for (int k = 0; k < n; ++k) {
      const int p = piv[k];
      if (p != k) { const float t = xs[k]; xs[k] = xs[p]; xs[p] = t; }
    }
  __syncthreads();
  cta_trsv<float>(lu, n, n, true, false, true, xs, tsm);
  cta_trsv<float>(lu, n, n, false, false, false, xs, tsm);
  for (int i = threadIdx.x; i < n; i += blockDim.x) xc[i] = (double)xs[i];
}

}  // namespace lxgb

using namespace lxgb;

// Workspace: U12ᵀ (n×64), for 3xTF32 the hi/lo splits of L21 and U12ᵀ, for
// BF16 the BF16 copies of L21 and U12ᵀ.
extern "C" int64_t lxgb_getrf_f32_tc_workspace_size(int32_t n, int32_t precision) {
  const int64_t blk = (int64_t)(n > 0 ? n : 1) * kLu32NB * (int64_t)sizeof(float);
  const int blocks = precision == 1 ? 5 : (precision == 2 ? 4 : 1);
  return 256 + blocks * ((blk + 255) & ~(int64_t)255);
}

extern "C" int lxgb_getrf_f32_tc(int32_t n, const double* a64, float* lu, int32_t* piv,
                                 int32_t* info, int32_t precision, int32_t* err, void* work,
                                 int64_t work_bytes, void* stream) {
  LXGB_REQUIRE(precision >= 0 && precision <= 2,
               "getrf_f32_tc: precision must be 0 (TF32), 1 (3xTF32) or 2 (BF16)");
  LXGB_REQUIRE(n >= 0, "getrf_f32_tc: negative size");
  if (n == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(lu && piv && info && err && work, "getrf_f32_tc: null pointer");
  LXGB_REQUIRE((n % 4) == 0, "getrf_f32_tc: n must be a multiple of 4 (16-byte TMA rows)");
  LXGB_REQUIRE((((uintptr_t)lu) & 15) == 0 && (((uintptr_t)work) & 255) == 0,
               "getrf_f32_tc: lu must be 16-byte and work 256-byte aligned");
  if (work_bytes < lxgb_getrf_f32_tc_workspace_size(n, precision)) {
    set_last_error("getrf_f32_tc: workspace too small");
    return LXGB_WORKSPACE_TOO_SMALL;
  }
  cudaStream_t st = as_stream(stream);
  if (a64) {
    const int64_t cnt = (int64_t)n * n;
    cvt_f64_to_f32_kernel<<<(unsigned)(((cnt + 255) / 256) < 8192 ? (cnt + 255) / 256 : 8192), 256,
                            0, st>>>(cnt, a64, lu);
  }
  zero_i32_kernel<<<1, 32, 0, st>>>(info, 1);
  const int64_t blk = (((int64_t)n * kLu32NB * (int64_t)sizeof(float)) + 255) & ~(int64_t)255;
  char* wb = reinterpret_cast<char*>(work) + 256;
  float* bt = reinterpret_cast<float*>(wb);
  float* ah = reinterpret_cast<float*>(wb + blk);
  float* al = reinterpret_cast<float*>(wb + 2 * blk);
  float* bh = reinterpret_cast<float*>(wb + 3 * blk);
  float* bl = reinterpret_cast<float*>(wb + 4 * blk);
  for (int j0 = 0; j0 < n; j0 += kLu32NB) {
    const int nb = min(kLu32NB, n - j0);
    if (launch_panel_cluster(n, j0, nb, lu, piv, info, st) != 0)
      panel_getf2_f32_kernel<<<1, kLu32PanelThreads, 0, st>>>(n, j0, nb, lu, piv, info);
    const int outside = n - nb;
    if (outside > 0) laswp_f32_kernel<<<(outside + 127) / 128, 128, 0, st>>>(n, j0, nb, lu, piv);
    const int n2 = n - j0 - nb;
    if (n2 > 0) {
      // U12 = L11^{-1} A12 in place, and U12ᵀ (K-major) into bt for the GEMM
      int rc0 = launch_inv_diag_lower(n, j0, nb, lu, lu, j0 + nb, n, bt, st);
      if (rc0) return rc0;
      // A22 -= L21 U12   (A = L21: n2×nb at lu[(j0+nb)*n + j0], B = U12ᵀ: n2×nb)
      float* c22 = lu + (int64_t)(j0 + nb) * n + j0 + nb;
      const float* l21 = lu + (int64_t)(j0 + nb) * n + j0;
      int rc;
      if (precision == 1) {
        rc = tf32_split(n2, nb, l21, n, ah, al, kLu32NB, st);
        if (!rc) rc = tf32_split(n2, nb, bt, kLu32NB, bh, bl, kLu32NB, st);
        if (!rc)
          rc = gemm_tf32_nt_split(n2, n2, nb, ah, al, kLu32NB, bh, bl, kLu32NB, c22, n, -1.0f, 1.0f,
                                  err, st);
      } else if (precision == 2) {
        // BF16 operands (8-bit significands), FP32 accumulation in tensor memory
        rc = bf16_convert(n2, nb, l21, n, ah, kLu32NB, st);
        if (!rc) rc = bf16_convert(n2, nb, bt, kLu32NB, bh, kLu32NB, st);
        if (!rc)
          rc = gemm_bf16_nt(n2, n2, nb, ah, kLu32NB, bh, kLu32NB, c22, n, -1.0f, 1.0f, err, st);
      } else {
        rc = gemm_tf32_nt(n2, n2, nb, l21, n, bt, kLu32NB, c22, n, -1.0f, 1.0f, err, st);
      }
      if (rc) return rc;
    }
  }
  return check_launch("getrf_f32_tc");
}

extern "C" int lxgb_getrs_f32(int32_t n, int32_t nrhs, const float* lu, const int32_t* piv,
                              const double* b, double* x, void* stream) {
  LXGB_REQUIRE(n >= 0 && nrhs >= 0, "getrs_f32: negative size");
  if (n == 0 || nrhs == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(lu && piv && b && x, "getrs_f32: null pointer");
  const size_t smem = (size_t)n * sizeof(float);
  LXGB_REQUIRE(smem <= 180 * 1024, "getrs_f32: n too large for the shared-memory vector");
  LXGB_CUDA_TRY(ensure_dynamic_smem(reinterpret_cast<const void*>(getrs_f32_kernel), (int)smem),
                "getrs_f32: set smem");
  getrs_f32_kernel<<<(unsigned)nrhs, 256, smem, as_stream(stream)>>>(n, lu, piv, b, x);
  return check_launch("getrs_f32");
}
