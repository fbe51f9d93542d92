// Mixed-precision LU: FP32 storage, partial pivoting, trailing updates on the
// tcgen05 tensor cores (TF32 products, FP32 accumulation), and the matching
// FP32 solve used as the preconditioner of FP64 GMRES-IR.
//
// Right-looking blocked LU with 64-column panels:
//   panel_getf2_f32_kernel — getf2 on the panel (one CTA; first row of max |a|)
//   laswp_f32_kernel       — the panel's row interchanges on the other columns
//   trsm_blockrow_f32_kernel — U12 = L11^{-1} A12
//   transpose_f32_kernel   — U12ᵀ into a K-major buffer for the GEMM
//   gemm_tf32_nt           — A22 -= L21 U12 on the tensor cores
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

// U12 = L11^{-1} A12, one column per thread (column-oriented substitution).
__global__ void __launch_bounds__(128)
trsm_blockrow_f32_kernel(int n, int j0, int nb, float* __restrict__ a) {
  __shared__ float L[kLu32NB][kLu32NB + 1];
  for (int e = threadIdx.x; e < kLu32NB * kLu32NB; e += blockDim.x) {
    const int i = e / kLu32NB, k = e % kLu32NB;
    L[i][k] = (i < nb && k < nb) ? a[(int64_t)(j0 + i) * n + j0 + k] : 0.0f;
  }
  __syncthreads();
  const int j = j0 + nb + blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  float col[kLu32NB];
#pragma unroll
  for (int i = 0; i < kLu32NB; ++i) col[i] = (i < nb) ? a[(int64_t)(j0 + i) * n + j] : 0.0f;
#pragma unroll
  for (int k = 0; k < kLu32NB; ++k) {
#pragma unroll
    for (int i = k + 1; i < kLu32NB; ++i) col[i] = fmaf(-L[i][k], col[k], col[i]);
  }
#pragma unroll
  for (int i = 0; i < kLu32NB; ++i)
    if (i < nb) a[(int64_t)(j0 + i) * n + j] = col[i];
}

// bt[j][p] = a[j0+p][j0+nb+j]  (U12ᵀ, K-major for the GEMM), ld of bt = kLu32NB.
__global__ void transpose_u12_kernel(int n, int j0, int nb, const float* __restrict__ a,
                                     float* __restrict__ bt) {
  __shared__ float tile[32][33];
  const int jb = blockIdx.x * 32, pb = blockIdx.y * 32;
  const int n2 = n - j0 - nb;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int p = pb + r, j = jb + threadIdx.x;
    tile[r][threadIdx.x] = (p < nb && j < n2) ? a[(int64_t)(j0 + p) * n + j0 + nb + j] : 0.0f;
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int j = jb + r, p = pb + threadIdx.x;
    if (j < n2) bt[(int64_t)j * kLu32NB + p] = tile[threadIdx.x][r];
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
    panel_getf2_f32_kernel<<<1, kLu32PanelThreads, 0, st>>>(n, j0, nb, lu, piv, info);
    const int outside = n - nb;
    if (outside > 0) laswp_f32_kernel<<<(outside + 127) / 128, 128, 0, st>>>(n, j0, nb, lu, piv);
    const int n2 = n - j0 - nb;
    if (n2 > 0) {
      trsm_blockrow_f32_kernel<<<(n2 + 127) / 128, 128, 0, st>>>(n, j0, nb, lu);
      dim3 tg((unsigned)((n2 + 31) / 32), (unsigned)((nb + 31) / 32));
      transpose_u12_kernel<<<tg, dim3(32, 8), 0, st>>>(n, j0, nb, lu, bt);
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
