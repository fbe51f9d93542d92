// FP64 symmetric rank-k products and the multi-CTA Cholesky of one large
// matrix.
//
// syrk_f64_kernel forms S = AᵀA (A k×n) or AAᵀ (A n×k) on the upper 64×64
// tiles of an n×n result, one CTA per tile (256 threads, 4×4 outputs each,
// A staged through shared memory in 16-deep slices).  Either as a Gram matrix
// (C = S, optionally mirrored into the lower triangle: the normal equations
// of lineax's Normal solver, lineax/_solver/normal.py:112-118) or as the
// Cholesky trailing update C -= S, where every element continues its FMA
// chain from its stored value in k order.
//
// lxgb_potrf_f64 factors one n×n SPD matrix (A = UᵀU, upper) right-looking
// by 64-row block rows: the diagonal block by one CTA in shared memory, the
// block row by a column-parallel substitution, the trailing matrix by the
// SYRK update above.  Every element receives exactly the update chain of the
// single-CTA factorisation (k ascending, scaling by the pivot reciprocal), so
// both give the same bits.
#include "common.cuh"
#include "potrf.cuh"

namespace lxgb {

constexpr int kSyTile = 64;
constexpr int kSyK = 16;
constexpr int kPoNB = 64;       // block rows of the multi-CTA Cholesky
constexpr int kPoCols = 128;    // columns per CTA of the block-row substitution

// Upper tile t (row-major over the triangle) of an nt×nt tile grid.
__device__ __forceinline__ void upper_tile(int t, int nt, int& ti, int& tj) {
  int rem = t, i = 0;
  while (rem >= nt - i) { rem -= nt - i; ++i; }
  ti = i;
  tj = i + rem;
}

// trans 0: S = AᵀA, element (kk, i) of the k×n operand at a[kk*lda + i];
// trans 1: S = AAᵀ, element (kk, i) at a[i*lda + kk].
// update 0: C = S (fill: also write C[j][i]); update 1: C -= S on j >= i.
__global__ void __launch_bounds__(256)
syrk_f64_kernel(int trans, int64_t n, int64_t k, const double* __restrict__ a, int64_t lda,
                int update, double* __restrict__ c, int64_t ldc, int fill) {
  __shared__ double as[kSyK][kSyTile + 1];
  __shared__ double bs[kSyK][kSyTile + 1];
  const int nt = (int)((n + kSyTile - 1) / kSyTile);
  int ti, tj;
  upper_tile(blockIdx.x, nt, ti, tj);
  const int64_t i0 = (int64_t)ti * kSyTile, j0 = (int64_t)tj * kSyTile;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  double acc[4][4];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int64_t i = i0 + ty + 16 * r, j = j0 + tx + 16 * q;
      acc[r][q] = (update && i < n && j < n && j >= i) ? c[i * ldc + j] : 0.0;
    }
  for (int64_t k0 = 0; k0 < k; k0 += kSyK) {
#pragma unroll
    for (int e4 = 0; e4 < (kSyK * kSyTile) / 256; ++e4) {
      const int e = tid + 256 * e4;
      int kk, ii;
      if (trans == 0) { kk = e / kSyTile; ii = e % kSyTile; }
      else { ii = e / kSyK; kk = e % kSyK; }
      const int64_t gk = k0 + kk, gi = i0 + ii, gj = j0 + ii;
      double va = 0.0, vb = 0.0;
      if (gk < k) {
        if (trans == 0) {
          if (gi < n) va = a[gk * lda + gi];
          if (gj < n) vb = a[gk * lda + gj];
        } else {
          if (gi < n) va = a[gi * lda + gk];
          if (gj < n) vb = a[gj * lda + gk];
        }
      }
      as[kk][ii] = va;
      bs[kk][ii] = vb;
    }
    __syncthreads();
    const int kn = (int)((k - k0 < kSyK) ? (k - k0) : kSyK);
    for (int kk = 0; kk < kn; ++kk) {
      double ai[4], bj[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) ai[r] = as[kk][ty + 16 * r];
#pragma unroll
      for (int q = 0; q < 4; ++q) bj[q] = bs[kk][tx + 16 * q];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int q = 0; q < 4; ++q)
          acc[r][q] = update ? fma(-ai[r], bj[q], acc[r][q]) : fma(ai[r], bj[q], acc[r][q]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int64_t i = i0 + ty + 16 * r, j = j0 + tx + 16 * q;
      if (i < n && j < n && j >= i) {
        c[i * ldc + j] = acc[r][q];
        if (fill && !update && j > i) c[j * ldc + i] = acc[r][q];
      }
    }
}

// The diagonal block [j0, j0+nb)² factored by one CTA in shared memory.
// info[0] records the first pivot that is not positive (global index + 1).
__global__ void __launch_bounds__(256)
potrf_diag_kernel(int64_t n, double* __restrict__ a, int64_t lda, int64_t j0, int nb,
                  int32_t* __restrict__ info) {
  __shared__ double blk[kPoNB * (kPoNB + 1)];
  const int ld = nb | 1;
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
    const int i = e / nb, j = e % nb;
    if (j >= i) blk[i * ld + j] = a[(j0 + i) * lda + j0 + j];
  }
  __syncthreads();
  const int rc = cta_potrf_upper<double, 16>(blk, ld, nb);
  __syncthreads();
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
    const int i = e / nb, j = e % nb;
    if (j >= i) a[(j0 + i) * lda + j0 + j] = blk[i * ld + j];
  }
  if (threadIdx.x == 0 && rc != 0 && info[0] == 0) info[0] = (int32_t)(j0 + rc);
}

// Block row [j0, j0+nb) × columns [j1, n): U12 = U11⁻ᵀ A12 by substitution,
// one column per thread, in the order of the single-CTA factorisation: row p
// scaled by 1/U11[p][p], then rows q > p updated by an FMA.
struct PoRowSmem {
  double u[kPoNB][kPoNB + 1];
  double rinv[kPoNB];
  double x[kPoNB][kPoCols + 1];
};

__global__ void __launch_bounds__(kPoCols)
potrf_blockrow_kernel(int64_t n, double* __restrict__ a, int64_t lda, int64_t j0, int nb,
                      int64_t j1) {
  extern __shared__ double po_smem[];
  PoRowSmem& sm = *reinterpret_cast<PoRowSmem*>(po_smem);
  auto& u = sm.u;
  auto& rinv = sm.rinv;
  auto& x = sm.x;
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
    const int i = e / nb, j = e % nb;
    u[i][j] = (j >= i) ? a[(j0 + i) * lda + j0 + j] : 0.0;
  }
  __syncthreads();
  if (threadIdx.x < nb) rinv[threadIdx.x] = 1.0 / u[threadIdx.x][threadIdx.x];
  const int64_t col0 = j1 + (int64_t)blockIdx.x * kPoCols;
  const int t = threadIdx.x;
  const int64_t col = col0 + t;
  for (int p = 0; p < nb; ++p) x[p][t] = (col < n) ? a[(j0 + p) * lda + col] : 0.0;
  __syncthreads();
  for (int p = 0; p < nb; ++p) {
    const double xp = x[p][t] * rinv[p];
    x[p][t] = xp;
    for (int q = p + 1; q < nb; ++q) x[q][t] = fma(-u[p][q], xp, x[q][t]);
  }
  if (col < n)
    for (int p = 0; p < nb; ++p) a[(j0 + p) * lda + col] = x[p][t];
}

__global__ void zero_lower_kernel(int64_t n, double* __restrict__ a, int64_t lda) {
  for (int64_t i = blockIdx.x; i < n; i += gridDim.x)
    for (int64_t j = threadIdx.x; j < i; j += blockDim.x) a[i * lda + j] = 0.0;
}

__global__ void set_info_kernel(int32_t* info) { info[0] = 0; }

static int syrk_launch(int trans, int64_t n, int64_t k, const double* a, int64_t lda, int update,
                       double* c, int64_t ldc, int fill, cudaStream_t st) {
  const int64_t nt = (n + kSyTile - 1) / kSyTile;
  const int64_t tiles = nt * (nt + 1) / 2;
  LXGB_REQUIRE(tiles < (1LL << 31), "syrk: n too large");
  syrk_f64_kernel<<<(unsigned)tiles, 256, 0, st>>>(trans, n, k, a, lda, update, c, ldc, fill);
  return check_launch("syrk_f64");
}

}  // namespace lxgb

using namespace lxgb;

extern "C" int lxgb_syrk_f64(int32_t trans, int64_t n, int64_t k, const double* a, int64_t lda,
                             int32_t update, double* c, int64_t ldc, int32_t fill, void* stream) {
  LXGB_REQUIRE(n >= 0 && k >= 0, "syrk: negative size");
  LXGB_REQUIRE(trans == 0 || trans == 1, "syrk: trans must be 0 or 1");
  LXGB_REQUIRE(!(update && fill), "syrk: fill is for the Gram form (update == 0)");
  if (n == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(c && (k == 0 || a), "syrk: null pointer");
  LXGB_REQUIRE(ldc >= n && lda >= (trans == 0 ? n : k), "syrk: leading dimension too small");
  return syrk_launch(trans, n, k, a, lda, update, c, ldc, fill, as_stream(stream));
}

extern "C" int lxgb_potrf_f64(int64_t n, double* a, int64_t lda, int32_t* info, void* stream) {
  LXGB_REQUIRE(n >= 0, "potrf: negative size");
  LXGB_REQUIRE(info, "potrf: null info");
  cudaStream_t st = as_stream(stream);
  set_info_kernel<<<1, 1, 0, st>>>(info);
  if (n == 0) return check_launch("potrf_f64");
  LXGB_REQUIRE(a && lda >= n, "potrf: null pointer or lda < n");
  LXGB_CUDA_TRY(ensure_dynamic_smem(reinterpret_cast<const void*>(potrf_blockrow_kernel),
                                    (int)sizeof(PoRowSmem)),
                "potrf: set smem");
  for (int64_t j0 = 0; j0 < n; j0 += kPoNB) {
    const int nb = (int)((n - j0 < kPoNB) ? (n - j0) : kPoNB);
    const int64_t j1 = j0 + nb;
    potrf_diag_kernel<<<1, 256, 0, st>>>(n, a, lda, j0, nb, info);
    if (j1 < n) {
      const int64_t cols = n - j1;
      potrf_blockrow_kernel<<<(unsigned)((cols + kPoCols - 1) / kPoCols), kPoCols,
                              sizeof(PoRowSmem), st>>>(n, a, lda, j0, nb, j1);
      int rc = syrk_launch(0, cols, nb, a + j0 * lda + j1, lda, 1, a + j1 * lda + j1, lda, 0, st);
      if (rc) return rc;
    }
  }
  const int64_t g = (n < 4096) ? n : 4096;
  zero_lower_kernel<<<(unsigned)g, 256, 0, st>>>(n, a, lda);
  return check_launch("potrf_f64");
}
