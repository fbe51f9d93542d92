// Mixed-precision LU: FP32 storage, partial pivoting, trailing updates on the
// tcgen05 tensor cores (TF32 products, FP32 accumulation), and the matching
// FP32 solve used as the preconditioner of FP64 GMRES-IR.
//
// Right-looking blocked LU with 64-column panels:
//   panel_getf2_cluster_kernel — getf2 on the panel held in the shared memory
//                            of a thread-block cluster (up to 16 CTAs); the
//                            pivot search is exchanged through distributed
//                            shared memory.  panel_getf2_f32_kernel (one
//                            CTA, panel in global memory) covers panels too
//                            tall for the cluster.
//   laswp_f32_kernel       — the panel's row interchanges on the other columns
//   launch_inv_diag_lower  — U12 = L11^{-1} A12 in place, and U12ᵀ into a
//                            K-major buffer for the GEMM (ir.cu)
//   gemm_tf32_nt           — A22 -= L21 U12 on the tensor cores
#include <cooperative_groups.h>
#include <float.h>
#include <limits.h>

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

static int launch_panel_cluster(int n, int j0, int nb, float* a, int32_t* piv, int32_t* info,
                                cudaStream_t st) {
  int r = 0;
  const int c = panel_cluster_size(n - j0, &r);
  if (c == 0) return -1;
  const size_t smem = (size_t)r * kPanelLd * sizeof(float);
  if (cudaFuncSetAttribute(panel_getf2_cluster_kernel,
                           cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess ||
      cudaFuncSetAttribute(panel_getf2_cluster_kernel,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
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
  int nclusters = 0;
  if (cudaOccupancyMaxActiveClusters(&nclusters, panel_getf2_cluster_kernel, &cfg) != cudaSuccess ||
      nclusters < 1) {
    cudaGetLastError();
    return -1;
  }
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

// Workspace: U12ᵀ (n×64), and for 3xTF32 the hi/lo splits of L21 and U12ᵀ.
extern "C" int64_t lxgb_getrf_f32_tc_workspace_size(int32_t n, int32_t precision) {
  const int64_t blk = (int64_t)(n > 0 ? n : 1) * kLu32NB * (int64_t)sizeof(float);
  return 256 + (precision == 1 ? 5 : 1) * ((blk + 255) & ~(int64_t)255);
}

extern "C" int lxgb_getrf_f32_tc(int32_t n, const double* a64, float* lu, int32_t* piv,
                                 int32_t* info, int32_t precision, int32_t* err, void* work,
                                 int64_t work_bytes, void* stream) {
  LXGB_REQUIRE(precision == 0 || precision == 1, "getrf_f32_tc: precision must be 0 or 1");
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
  LXGB_CUDA_TRY(cudaFuncSetAttribute(getrs_f32_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem),
                "getrs_f32: set smem");
  getrs_f32_kernel<<<(unsigned)nrhs, 256, smem, as_stream(stream)>>>(n, lu, piv, b, x);
  return check_launch("getrs_f32");
}
