// FP32 Cholesky of one large SPD matrix with tensor-core updates, for
// mixed-precision refinement (the serving route of Cholesky requests above
// the ragged kernel's order limit):
//
//   lxgb_potrf_f32_tc  — A = L Lᵀ in FP32, right-looking by 64-column panels:
//     the 64×64 diagonal block factored by one CTA in shared memory, the
//     panel below it L21 = A21 L_jj⁻ᵀ by FP32 substitution on the CUDA cores
//     (one row per thread), and the trailing update A22 -= L21 L21ᵀ
//     (lower-triangle tiles only) as a tcgen05 GEMM with 3xTF32 products
//     (FP32-level accuracy).  A is read from its upper triangle, as
//     lineax's Cholesky reads it (cho_factor(lower=False),
//     lineax/_solver/cholesky.py:60): L = Uᵀ.
//   lxgb_chol32_to_lu32 — the factor in the unit-lower / upper form of the
//     mixed LU (L' = L D⁻¹, U' = D Lᵀ, D = diag(L), no interchanges), so the
//     GMRES-IR machinery of the mixed LU applies unchanged.
//   lxgb_chol32_uinv    — U'⁻¹ = L'⁻ᵀ D⁻² from L'⁻¹: the second triangular
//     inverse by a transposing copy instead of a second substitution.
#include "common.cuh"
#include "tc_gemm.cuh"

namespace lxgb {

constexpr int kC32NB = 64;

// l[i][j] = fl32(a[j][i]) for j <= i (A's upper triangle, transposed), 0
// above the diagonal.  32×32 tiles through shared memory: coalesced reads of
// a's rows and writes of l's rows.
__global__ void c32_lower_from_upper_kernel(int64_t n, const double* __restrict__ a,
                                            float* __restrict__ l) {
  __shared__ float tile[32][33];
  const int64_t bi = (int64_t)blockIdx.y * 32, bj = (int64_t)blockIdx.x * 32;  // tile of l
  // read a[bj + r][bi + c] (a row segment) into tile[r][c]
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int64_t ar = bj + r, ac = bi + threadIdx.x;
    tile[r][threadIdx.x] = (ar < n && ac < n) ? __double2float_rn(a[ar * n + ac]) : 0.0f;
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int64_t li = bi + r, lj = bj + threadIdx.x;
    if (li < n && lj < n) l[li * n + lj] = (lj <= li) ? tile[threadIdx.x][r] : 0.0f;
  }
}

// Factor the nb×nb diagonal block at (j0, j0) of l (lower triangle) in
// shared memory with 256 threads: per column one thread takes the square
// root, the rows below divide by it, and the rank-1 update of the trailing
// lower triangle is spread over all threads element by element.  The first
// pivot that is not positive is recorded in *info (1-based, global index) and
// replaced by 1 so that the launch finishes.
constexpr int kC32DiagThreads = 256;

__global__ void __launch_bounds__(kC32DiagThreads)
c32_diag_kernel(int64_t n, int64_t j0, int nb, float* __restrict__ l, int32_t* __restrict__ info) {
  __shared__ float T[kC32NB][kC32NB + 1];
  __shared__ int s_bad;
  const int tid = threadIdx.x;
  for (int e = tid; e < kC32NB * kC32NB; e += kC32DiagThreads) {
    const int i = e / kC32NB, c = e % kC32NB;
    T[i][c] = (i < nb && c <= i) ? l[(j0 + i) * n + j0 + c] : 0.0f;
  }
  if (tid == 0) s_bad = 0;
  __syncthreads();
  for (int k = 0; k < nb; ++k) {
    if (tid == 0) {
      float d = T[k][k];
      if (!(d > 0.0f)) {
        if (s_bad == 0) s_bad = k + 1;
        d = 1.0f;
      }
      T[k][k] = sqrtf(d);
    }
    __syncthreads();
    const float s = T[k][k];
    for (int i = k + 1 + tid; i < nb; i += kC32DiagThreads) T[i][k] = T[i][k] / s;
    __syncthreads();
    const int w = nb - k - 1;
    for (int e = tid; e < w * w; e += kC32DiagThreads) {
      const int i = k + 1 + e / w, c = k + 1 + e % w;
      if (c <= i) T[i][c] = fmaf(-T[i][k], T[c][k], T[i][c]);
    }
    __syncthreads();
  }
  for (int e = tid; e < nb * nb; e += kC32DiagThreads) {
    const int i = e / nb, c = e % nb;
    if (c <= i) l[(j0 + i) * n + j0 + c] = T[i][c];
  }
  if (tid == 0 && s_bad) atomicCAS(reinterpret_cast<int*>(info), 0, (int)(j0 + s_bad));
}

// The panel below the diagonal block: L21 = A21 L_jj⁻ᵀ by forward
// substitution on the CUDA cores (FP32), one row per thread with the row in
// registers, 96 rows per CTA staged through shared memory for coalesced
// loads and stores; L21 goes back into l and, split into TF32-exact hi and lo
// parts, into ph / pl (row stride 64) for the trailing update.
constexpr int kC32Rows = 96;

__global__ void __launch_bounds__(kC32Rows)
c32_panel_kernel(int64_t n, int64_t j0, int m2, float* __restrict__ l, float* __restrict__ ph,
                 float* __restrict__ pl) {
  __shared__ float L[kC32NB][kC32NB];            // read as broadcasts: no padding
  __shared__ float X[kC32Rows][kC32NB + 1];       // row per thread: padded
  const int t = threadIdx.x;
  const int64_t rbase = (int64_t)blockIdx.x * kC32Rows;      // first panel row of this CTA
  for (int e = t; e < kC32NB * kC32NB; e += kC32Rows) {
    const int r = e / kC32NB, c = e % kC32NB;
    L[r][c] = (c <= r) ? l[(j0 + r) * n + j0 + c] : 0.0f;
  }
  for (int e = t; e < kC32Rows * kC32NB; e += kC32Rows) {
    const int r = e / kC32NB, c = e % kC32NB;
    const int64_t pr = rbase + r;
    X[r][c] = (pr < m2) ? l[(j0 + kC32NB + pr) * n + j0 + c] : 0.0f;
  }
  __syncthreads();
  float a[kC32NB];
#pragma unroll
  for (int c = 0; c < kC32NB; ++c) a[c] = X[t][c];
#pragma unroll
  for (int k = 0; k < kC32NB; ++k) {
    const float x = a[k] / L[k][k];
    a[k] = x;
#pragma unroll
    for (int j = k + 1; j < kC32NB; ++j) a[j] = fmaf(-x, L[j][k], a[j]);
  }
#pragma unroll
  for (int c = 0; c < kC32NB; ++c) X[t][c] = a[c];
  __syncthreads();
  for (int e = t; e < kC32Rows * kC32NB; e += kC32Rows) {
    const int r = e / kC32NB, c = e % kC32NB;
    const int64_t pr = rbase + r;
    if (pr < m2) {
      const float x = X[r][c];
      const float h = __uint_as_float(__float_as_uint(x) & 0xFFFFE000u);
      l[(j0 + kC32NB + pr) * n + j0 + c] = x;
      ph[pr * kC32NB + c] = h;
      pl[pr * kC32NB + c] = x - h;
    }
  }
}

// The mixed-LU form of a Cholesky factor: lu[i][j] = L[i][j] / L[j][j] for
// j < i, lu[i][j] = L[i][i] L[j][i] for j >= i (U' = D Lᵀ).  32×32 tiles:
// tile (bi, bj) of lu needs tile (bj, bi) of L (transposed) above the
// diagonal and tile (bi, bj) below it; the diagonal values come from global
// memory.
__global__ void c32_to_lu_kernel(int64_t n, const float* __restrict__ l, float* __restrict__ lu) {
  __shared__ float tile[32][33];
  const int64_t bi = (int64_t)blockIdx.y * 32, bj = (int64_t)blockIdx.x * 32;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int64_t tr = bj + r, tc = bi + threadIdx.x;   // L[bj + r][bi + x]
    tile[r][threadIdx.x] = (tr < n && tc < n) ? l[tr * n + tc] : 0.0f;
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int64_t i = bi + r, j = bj + threadIdx.x;
    if (i >= n || j >= n) continue;
    float v;
    if (j < i)
      v = l[i * n + j] / l[j * n + j];
    else
      v = l[i * n + i] * tile[threadIdx.x][r];          // L[i][i] * L[j][i]
    lu[i * n + j] = v;
  }
}

// uinv[i][j] = linv[j][i] / lu[j][j] for j >= i, 0 below the diagonal.
__global__ void c32_uinv_kernel(int64_t n, const float* __restrict__ lu,
                                const float* __restrict__ linv, float* __restrict__ uinv) {
  __shared__ float tile[32][33];
  const int64_t bi = (int64_t)blockIdx.y * 32, bj = (int64_t)blockIdx.x * 32;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int64_t tr = bj + r, tc = bi + threadIdx.x;   // linv[bj + r][bi + x]
    tile[r][threadIdx.x] = (tr < n && tc < n) ? linv[tr * n + tc] : 0.0f;
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int64_t i = bi + r, j = bj + threadIdx.x;
    if (i >= n || j >= n) continue;
    uinv[i * n + j] = (j >= i) ? tile[threadIdx.x][r] / lu[j * n + j] : 0.0f;
  }
}

__global__ void c32_iota_kernel(int64_t n, int32_t* __restrict__ piv) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    piv[i] = (int32_t)i;
}

static dim3 c32_tiles(int64_t n) {
  return dim3((unsigned)((n + 31) / 32), (unsigned)((n + 31) / 32));
}

}  // namespace lxgb

using namespace lxgb;

extern "C" int64_t lxgb_potrf_f32_tc_workspace_size(int64_t n) {
  const int64_t panel = (n > 0 ? n : 1) * kC32NB * 4;
  return 256 + 2 * ((panel + 255) / 256 * 256);
}

extern "C" int lxgb_potrf_f32_tc(int64_t n, const double* a, float* l, int32_t* info,
                                 int32_t* err, void* work, int64_t work_bytes, void* stream) {
  LXGB_REQUIRE(n >= 0, "potrf_f32_tc: negative size");
  if (n == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(a && l && info && err && work, "potrf_f32_tc: null pointer");
  LXGB_REQUIRE(n < 32768, "potrf_f32_tc: n above 32767");
  LXGB_REQUIRE((n % 4) == 0, "potrf_f32_tc: n must be a multiple of 4 (16-byte TMA rows)");
  LXGB_REQUIRE((((uintptr_t)l) & 15) == 0 && (((uintptr_t)work) & 255) == 0,
               "potrf_f32_tc: l must be 16-byte and work 256-byte aligned");
  if (work_bytes < lxgb_potrf_f32_tc_workspace_size(n)) {
    set_last_error("potrf_f32_tc: workspace too small");
    return LXGB_WORKSPACE_TOO_SMALL;
  }
  cudaStream_t st = as_stream(stream);
  LXGB_CUDA_TRY(cudaMemsetAsync(info, 0, sizeof(int32_t), st), "potrf_f32_tc: clear info");
  c32_lower_from_upper_kernel<<<c32_tiles(n), dim3(32, 8), 0, st>>>(n, a, l);
  const int64_t panel = ((n * kC32NB * 4) + 255) / 256 * 256;
  char* wb = reinterpret_cast<char*>(work) + 256;
  float* ph = reinterpret_cast<float*>(wb);
  float* pl = reinterpret_cast<float*>(wb + panel);
  for (int64_t j0 = 0; j0 < n; j0 += kC32NB) {
    const int nb = (int)(n - j0 < kC32NB ? n - j0 : kC32NB);
    c32_diag_kernel<<<1, kC32DiagThreads, 0, st>>>(n, j0, nb, l, info);
    const int m2 = (int)(n - j0 - nb);
    if (m2 <= 0) break;          // only the last block is narrower than 64
    c32_panel_kernel<<<(unsigned)((m2 + kC32Rows - 1) / kC32Rows), kC32Rows, 0, st>>>(
        n, j0, m2, l, ph, pl);
    // A22 -= L21 L21ᵀ (3xTF32) on the tiles holding A22's lower triangle
    const int64_t r0 = j0 + kC32NB;
    const int rc = gemm_tf32_nt_split_lower(m2, kC32NB, ph, pl, kC32NB, l + r0 * n + r0, n,
                                            -1.0f, 1.0f, err, st);
    if (rc) return rc;
  }
  return check_launch("potrf_f32_tc");
}

extern "C" int lxgb_chol32_to_lu32(int64_t n, const float* l, float* lu, int32_t* piv,
                                   void* stream) {
  LXGB_REQUIRE(n >= 0, "chol32_to_lu32: negative size");
  if (n == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(l && lu && piv && l != lu, "chol32_to_lu32: null or aliased pointer");
  cudaStream_t st = as_stream(stream);
  c32_to_lu_kernel<<<c32_tiles(n), dim3(32, 8), 0, st>>>(n, l, lu);
  c32_iota_kernel<<<(unsigned)((n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024), 256, 0, st>>>(
      n, piv);
  return check_launch("chol32_to_lu32");
}

extern "C" int lxgb_chol32_uinv(int64_t n, const float* lu, const float* linv, float* uinv,
                                void* stream) {
  LXGB_REQUIRE(n >= 0, "chol32_uinv: negative size");
  if (n == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(lu && linv && uinv && linv != uinv, "chol32_uinv: null or aliased pointer");
  c32_uinv_kernel<<<c32_tiles(n), dim3(32, 8), 0, as_stream(stream)>>>(n, lu, linv, uinv);
  return check_launch("chol32_uinv");
}
