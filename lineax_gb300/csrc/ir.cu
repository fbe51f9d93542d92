// GMRES-IR building blocks for the FP32 LU (lu32.cu):
//
//   lxgb_lu32_inverse — L^{-1} and U^{-1} of the FP32 factor as dense FP32
//     triangles, by blocked substitution against the identity: 64-row
//     diagonal-block solves on the CUDA cores and the off-diagonal updates on
//     the tcgen05 tensor cores (TF32 or 3xTF32, as the factor was made).
//     M = U^{-1} L^{-1} P is then applied with two triangular matrix-vector
//     products that every SM shares, instead of two sequential substitutions.
//   lxgb_lu32_apply — y = U^{-1} (L^{-1} (P x)) for a block of FP64 vectors,
//     in FP32 or in double-float arithmetic (FP64-accurate on the FP32 pipe).
//   lxgb_gemv_df — y = A x or y = b - A x with A held as an FP32 hi + lo pair
//     (48 significant bits), in double-float arithmetic: the FP64 operator
//     product and residual of the refinement at a fraction of the FP64-pipe
//     cost.
//
// The products share one kernel: a CTA owns 16 rows and 16 right-hand sides;
// its eight warps each keep 4 rows x 8 right-hand sides of accumulators while
// the lanes walk the columns, then reduce across lanes.  No cross-CTA
// reduction: results are bitwise reproducible.
#include "common.cuh"
#include "df.cuh"
#include "tc_gemm.cuh"

namespace lxgb {

constexpr int kInvNB = 64;     // diagonal block size of the inversion
constexpr int kInvCols = 128;  // columns per CTA in the diagonal-block solves
constexpr int kGvRows = 16;    // rows per CTA of the products
constexpr int kGvRhs = 16;     // right-hand sides per CTA of the products
constexpr int kPermMaxN = 25600;

// (P b)_i = b[perm[i]]: the getrf row interchanges composed into one gather.
__global__ void perm_from_swaps_kernel(int n, const int32_t* __restrict__ piv,
                                       int32_t* __restrict__ perm) {
  extern __shared__ int32_t sp[];
  int32_t* spiv = sp + n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    sp[i] = i;
    spiv[i] = piv[i];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 0; k < n; ++k) {
      const int p = spiv[k];
      if (p != k && p >= 0 && p < n) {
        const int t = sp[k];
        sp[k] = sp[p];
        sp[p] = t;
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) perm[i] = sp[i];
}

__global__ void set_identity_f32_kernel(int n, float* __restrict__ w) {
  for (int r = blockIdx.x; r < n; r += gridDim.x)
    for (int c = threadIdx.x; c < n; c += blockDim.x) w[(int64_t)r * n + c] = (r == c) ? 1.0f : 0.0f;
}

// X = T_jj^{-1} W_j on rows [j0, j0+nb) of w and columns [c_begin, c_end):
// T_jj the unit-lower (LOWER) or upper diagonal block of the factor.  X goes
// back into w and, transposed (column c - c_begin, 64 entries, zero padded),
// into xt: the K-major operand of the following tensor-core update.
template <bool LOWER>
__global__ void __launch_bounds__(kInvCols)
inv_diag_kernel(int n, int j0, int nb, const float* __restrict__ lu, float* __restrict__ w,
                int c_begin, int c_end, float* __restrict__ xt) {
  // Tt[k][i] = T[i][k]: for a fixed k the multipliers of all rows i are
  // contiguous (16-byte broadcast loads).  Padding rows/columns past nb hold
  // the identity, so the fully unrolled substitution needs no bounds.
  __shared__ __align__(16) float Tt[kInvNB][kInvNB];
  __shared__ float X[kInvNB][kInvCols + 1];
  for (int e = threadIdx.x; e < kInvNB * kInvNB; e += blockDim.x) {
    const int i = e / kInvNB, k = e % kInvNB;
    Tt[k][i] = (i < nb && k < nb) ? lu[(int64_t)(j0 + i) * n + j0 + k] : (i == k ? 1.0f : 0.0f);
  }
  const int t = threadIdx.x;
  const int cbase = c_begin + blockIdx.x * kInvCols;
  const int c = cbase + t;
  // Each thread substitutes its own column, held in registers.
  float x[kInvNB];
#pragma unroll
  for (int i = 0; i < kInvNB; ++i)
    x[i] = (i < nb && c < c_end) ? w[(int64_t)(j0 + i) * n + c] : 0.0f;
  __syncthreads();
  if (LOWER) {
#pragma unroll
    for (int k = 0; k < kInvNB; ++k) {
      const float xk = x[k];
#pragma unroll
      for (int i4 = (k + 1) / 4; i4 < kInvNB / 4; ++i4) {
        const float4 tq = *reinterpret_cast<const float4*>(&Tt[k][4 * i4]);
        if (4 * i4 + 0 > k) x[4 * i4 + 0] = fmaf(-tq.x, xk, x[4 * i4 + 0]);
        if (4 * i4 + 1 > k) x[4 * i4 + 1] = fmaf(-tq.y, xk, x[4 * i4 + 1]);
        if (4 * i4 + 2 > k) x[4 * i4 + 2] = fmaf(-tq.z, xk, x[4 * i4 + 2]);
        if (4 * i4 + 3 > k) x[4 * i4 + 3] = fmaf(-tq.w, xk, x[4 * i4 + 3]);
      }
    }
  } else {
#pragma unroll
    for (int k = kInvNB - 1; k >= 0; --k) {
      const float xk = x[k] / Tt[k][k];
      x[k] = xk;
#pragma unroll
      for (int i4 = 0; i4 < (k + 3) / 4; ++i4) {
        const float4 tq = *reinterpret_cast<const float4*>(&Tt[k][4 * i4]);
        if (4 * i4 + 0 < k) x[4 * i4 + 0] = fmaf(-tq.x, xk, x[4 * i4 + 0]);
        if (4 * i4 + 1 < k) x[4 * i4 + 1] = fmaf(-tq.y, xk, x[4 * i4 + 1]);
        if (4 * i4 + 2 < k) x[4 * i4 + 2] = fmaf(-tq.z, xk, x[4 * i4 + 2]);
        if (4 * i4 + 3 < k) x[4 * i4 + 3] = fmaf(-tq.w, xk, x[4 * i4 + 3]);
      }
    }
  }
  if (c < c_end) {
#pragma unroll
    for (int i = 0; i < kInvNB; ++i)
      if (i < nb) w[(int64_t)(j0 + i) * n + c] = x[i];
  }
#pragma unroll
  for (int i = 0; i < kInvNB; ++i) X[i][t] = x[i];
  __syncthreads();
  // Transposed copy, coalesced along the 64 entries of each column.
  const int ncols = min(kInvCols, c_end - cbase);
  for (int e = threadIdx.x; e < ncols * kInvNB; e += blockDim.x) {
    const int col = e / kInvNB, i = e % kInvNB;
    xt[(int64_t)(cbase - c_begin + col) * kInvNB + i] = X[i][col];
  }
}

// ---------------------------------------------------------------------------
// Products.  MODE 0: FP32 products and sums (x rounded to FP32, no lo parts).
// MODE 1: double-float, exact FP32 matrix.  MODE 2: double-float, matrix
// hi + lo.  TRI 0 full; 1 lower (columns < the row block's end: the matrix
// holds zeros above its diagonal); 2 upper (columns from the row block's
// start).  OUT 0: (yh, yl) pair; 1: y64 = value; 2: y64 = b64 - value.
// ---------------------------------------------------------------------------
template <int MODE>
__device__ __forceinline__ void acc_step(float& sh, float& sl, float m, float ml, float xh,
                                         float xl) {
  if (MODE == 0) {
    sh = fmaf(m, xh, sh);
  } else {
    const float p = m * xh;
    float e = fmaf(m, xh, -p);  // exact: m xh = p + e
    e = fmaf(m, xl, e);
    if (MODE == 2) e = fmaf(ml, xh, e);
    float err;
    two_sum(sh, p, err);
    sl += err + e;
  }
}

template <int MODE, int TRI, int OUT>
__global__ void __launch_bounds__(256, MODE == 0 ? 2 : 1)
gemv16_kernel(int m, int ncol, const float* __restrict__ Mh, const float* __restrict__ Ml,
              int64_t ldm, int k, const float* __restrict__ xh, const float* __restrict__ xl,
              int64_t ldx, float* __restrict__ yh, float* __restrict__ yl,
              double* __restrict__ y64, const double* __restrict__ b64, int64_t ldy) {
  const int nblk = (m + kGvRows - 1) / kGvRows;
  // Lower triangles: the heaviest row blocks (last) start first.
  const int rb = (TRI == 1) ? (nblk - 1 - (int)blockIdx.x) : (int)blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int row0 = rb * kGvRows + (warp & 3) * 4;
  const int rhs0 = (int)blockIdx.y * kGvRhs + (warp >> 2) * 8;
  int c_lo = 0, c_hi = ncol;
  if (TRI == 1) c_hi = min(ncol, rb * kGvRows + kGvRows);
  if (TRI == 2) c_lo = rb * kGvRows;

  // Rows and right-hand sides past the ends are clamped to the last valid
  // one (in-bounds loads; their results are never written).
  const float* mr[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) mr[r] = Mh + (int64_t)min(row0 + r, m - 1) * ldm;
  const int64_t mlo = (MODE == 2) ? (Ml - Mh) : 0;  // lo matrix at the same offsets
  int xo[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) xo[q] = min(rhs0 + q, k - 1) * (int)ldx;
  const int64_t xlo = (MODE >= 1) ? (xl - xh) : 0;
  float ah[4][8], al[4][8];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int q = 0; q < 8; ++q) ah[r][q] = al[r][q] = 0.0f;

  // Double-float products are FP32-pipe bound with one CTA per SM: the next
  // column's operands are loaded while the current one is multiplied.
  float mv[4], mlv[4], xv[8], xlv[8];
  auto load = [&](int c, float (&m_)[4], float (&ml_)[4], float (&x_)[8], float (&xl_)[8]) {
    const bool ok = c < c_hi;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      m_[r] = ok ? __ldg(mr[r] + c) : 0.0f;
      ml_[r] = (MODE == 2 && ok) ? __ldg(mr[r] + mlo + c) : 0.0f;
    }
    const float* xc = xh + c;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      x_[q] = ok ? __ldg(xc + xo[q]) : 0.0f;
      xl_[q] = (MODE >= 1 && ok) ? __ldg(xc + xlo + xo[q]) : 0.0f;
    }
  };
  load(c_lo + lane, mv, mlv, xv, xlv);
  for (int c = c_lo + lane; c < c_hi; c += 32) {
    float nm[4], nml[4], nx[8], nxl[8];
    if (MODE != 0) load(c + 32, nm, nml, nx, nxl);
#pragma unroll
    for (int q = 0; q < 8; ++q)
#pragma unroll
      for (int r = 0; r < 4; ++r) acc_step<MODE>(ah[r][q], al[r][q], mv[r], mlv[r], xv[q], xlv[q]);
    if (MODE != 0) {
#pragma unroll
      for (int r = 0; r < 4; ++r) { mv[r] = nm[r]; mlv[r] = nml[r]; }
#pragma unroll
      for (int q = 0; q < 8; ++q) { xv[q] = nx[q]; xlv[q] = nxl[q]; }
    } else {
      load(c + 32, mv, mlv, xv, xlv);
    }
  }

  // Butterfly reduction across the lanes (every lane ends with every sum).
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const float oh = __shfl_xor_sync(0xffffffffu, ah[r][q], off);
        if (MODE == 0) {
          ah[r][q] += oh;
        } else {
          const float ol = __shfl_xor_sync(0xffffffffu, al[r][q], off);
          float err;
          two_sum(ah[r][q], oh, err);
          al[r][q] += ol + err;
        }
      }
  }
  // Lane r*8 + q writes (row0 + r, rhs0 + q).
  float oh = 0.0f, ol = 0.0f;
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int q = 0; q < 8; ++q)
      if (lane == r * 8 + q) {
        oh = ah[r][q];
        ol = al[r][q];
      }
  const int row = row0 + (lane >> 3), rhs = rhs0 + (lane & 7);
  if (row >= m || rhs >= k) return;
  const int64_t o = (int64_t)rhs * ldy + row;
  if (MODE >= 1) {
    float e;
    fast_two_sum(oh, ol, e);
    ol = e;
  }
  if (OUT == 0) {
    yh[o] = oh;
    if (MODE >= 1) yl[o] = ol;
  } else {
    const double v = (MODE >= 1) ? (double)oh + (double)ol : (double)oh;
    y64[o] = (OUT == 2) ? b64[o] - v : v;
  }
}

// Few right-hand sides (k <= 4): one warp per matrix row, lanes along the
// columns, k double-float accumulators per lane reduced across the warp.
// The matrix streams from HBM once; x (hi/lo, k × n) is shared through L1/L2.
template <int K, bool LO, int OUT>
__global__ void __launch_bounds__(256)
gemv_rows_df_kernel(int m, int ncol, const float* __restrict__ Mh, const float* __restrict__ Ml,
                    int64_t ldm, const float* __restrict__ xh, const float* __restrict__ xl,
                    int64_t ldx, double* __restrict__ y64, const double* __restrict__ b64,
                    int64_t ldy) {
  const int lane = threadIdx.x & 31;
  const int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (row >= m) return;  // whole warps
  const float* mr = Mh + (int64_t)row * ldm;
  const float* ml = LO ? Ml + (int64_t)row * ldm : mr;
  float sh[K], sl[K];
#pragma unroll
  for (int q = 0; q < K; ++q) sh[q] = sl[q] = 0.0f;
  for (int c = lane; c < ncol; c += 32) {
    const float a = __ldg(mr + c);
    const float al = LO ? __ldg(ml + c) : 0.0f;
#pragma unroll
    for (int q = 0; q < K; ++q) {
      const float x = __ldg(xh + (int64_t)q * ldx + c);
      const float xlv = __ldg(xl + (int64_t)q * ldx + c);
      const float p = a * x;
      float e = fmaf(a, x, -p);
      e = fmaf(a, xlv, e);
      if (LO) e = fmaf(al, x, e);
      float err;
      two_sum(sh[q], p, err);
      sl[q] += err + e;
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
#pragma unroll
    for (int q = 0; q < K; ++q) {
      const float oh = __shfl_xor_sync(0xffffffffu, sh[q], off);
      const float ol = __shfl_xor_sync(0xffffffffu, sl[q], off);
      float err;
      two_sum(sh[q], oh, err);
      sl[q] += ol + err;
    }
  if (lane < K) {
    float oh = sh[0], ol = sl[0];
#pragma unroll
    for (int q = 1; q < K; ++q)
      if (lane == q) { oh = sh[q]; ol = sl[q]; }
    const double v = (double)oh + (double)ol;
    const int64_t o = (int64_t)lane * ldy + row;
    y64[o] = (OUT == 2) ? b64[o] - v : v;
  }
}

template <int K, bool LO>
static void launch_rows_df(int m, int n, const float* ah, const float* al, int64_t lda,
                           const float* xh, const float* xl, int64_t ldx, double* y,
                           const double* b, int64_t ldy, cudaStream_t st) {
  const unsigned g = (unsigned)((m + 7) / 8);
  if (b)
    gemv_rows_df_kernel<K, LO, 2><<<g, 256, 0, st>>>(m, n, ah, al, lda, xh, xl, ldx, y, b, ldy);
  else
    gemv_rows_df_kernel<K, LO, 1><<<g, 256, 0, st>>>(m, n, ah, al, lda, xh, xl, ldx, y, b, ldy);
}

// zh/zl[q][i] = x[q][perm ? perm[i] : i] as a hi + lo pair (zl null: FP32 rounding).
__global__ void split_rows_kernel(int k, int n, const double* __restrict__ x, int64_t ldx,
                                  const int32_t* __restrict__ perm, float* __restrict__ zh,
                                  float* __restrict__ zl, int64_t ldz) {
  const int64_t total = (int64_t)k * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int q = (int)(e / n), i = (int)(e % n);
    const double v = x[(int64_t)q * ldx + (perm ? perm[i] : i)];
    if (zl) {
      float h, l;
      split_f64(v, h, l);
      zh[(int64_t)q * ldz + i] = h;
      zl[(int64_t)q * ldz + i] = l;
    } else {
      zh[(int64_t)q * ldz + i] = __double2float_rn(v);
    }
  }
}

__global__ void split_matrix_kernel(int64_t rows, int64_t cols, const double* __restrict__ a,
                                    int64_t lda, float* __restrict__ hi, float* __restrict__ lo,
                                    int64_t ld) {
  const int64_t total = rows * cols;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / cols, c = e % cols;
    float h, l;
    split_f64(a[r * lda + c], h, l);
    hi[r * ld + c] = h;
    if (lo) lo[r * ld + c] = l;
  }
}

template <int MODE, int TRI, int OUT>
int launch_gemv16(int m, int ncol, const float* Mh, const float* Ml, int64_t ldm, int k,
                  const float* xh, const float* xl, int64_t ldx, float* yh, float* yl,
                  double* y64, const double* b64, int64_t ldy, cudaStream_t st) {
  LXGB_REQUIRE((int64_t)k * ldx < ((int64_t)1 << 31), "gemv16: right-hand-side block above 2^31 entries");
  dim3 grid((unsigned)((m + kGvRows - 1) / kGvRows), (unsigned)((k + kGvRhs - 1) / kGvRhs));
  gemv16_kernel<MODE, TRI, OUT><<<grid, 256, 0, st>>>(m, ncol, Mh, Ml, ldm, k, xh, xl, ldx, yh,
                                                      yl, y64, b64, ldy);
  return check_launch("gemv16");
}

int launch_inv_diag_lower(int n, int j0, int nb, const float* lu, float* w, int c_begin,
                          int c_end, float* xt, cudaStream_t st) {
  if (c_end <= c_begin) return LXGB_SUCCESSFUL;
  inv_diag_kernel<true><<<(unsigned)((c_end - c_begin + kInvCols - 1) / kInvCols), kInvCols, 0,
                          st>>>(n, j0, nb, lu, w, c_begin, c_end, xt);
  return check_launch("inv_diag_lower");
}

static int64_t blk_bytes(int n) {
  return (((int64_t)(n > 0 ? n : 1) * kInvNB * (int64_t)sizeof(float)) + 255) & ~(int64_t)255;
}

static int64_t vec_bytes(int n, int nrhs) {
  return (((int64_t)(n > 0 ? n : 1) * (nrhs > 0 ? nrhs : 1) * (int64_t)sizeof(float)) + 255) &
         ~(int64_t)255;
}

}  // namespace lxgb

using namespace lxgb;

extern "C" int64_t lxgb_lu32_inverse_workspace_size(int32_t n, int32_t precision) {
  return 256 + (precision == 1 ? 5 : 1) * blk_bytes(n);
}

extern "C" int lxgb_lu32_inverse(int32_t n, const float* lu, const int32_t* piv, float* linv,
                                 float* uinv, int32_t* perm, int32_t precision, int32_t* err,
                                 void* work, int64_t work_bytes, void* stream) {
  LXGB_REQUIRE(precision == 0 || precision == 1, "lu32_inverse: precision must be 0 or 1");
  LXGB_REQUIRE(n >= 0, "lu32_inverse: negative size");
  if (n == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(n <= kPermMaxN, "lu32_inverse: n above 25600");
  LXGB_REQUIRE(lu && piv && (linv || uinv) && perm && err && work,
               "lu32_inverse: null pointer");
  LXGB_REQUIRE((n % 4) == 0, "lu32_inverse: n must be a multiple of 4 (16-byte TMA rows)");
  LXGB_REQUIRE((((uintptr_t)lu) & 15) == 0 && (((uintptr_t)work) & 255) == 0,
               "lu32_inverse: lu must be 16-byte and work 256-byte aligned");
  if (work_bytes < lxgb_lu32_inverse_workspace_size(n, precision)) {
    set_last_error("lu32_inverse: workspace too small");
    return LXGB_WORKSPACE_TOO_SMALL;
  }
  cudaStream_t st = as_stream(stream);
  const size_t psmem = (size_t)2 * n * sizeof(int32_t);
  LXGB_CUDA_TRY(ensure_dynamic_smem(reinterpret_cast<const void*>(perm_from_swaps_kernel), (int)psmem),
                "lu32_inverse: set smem");
  perm_from_swaps_kernel<<<1, 1024, psmem, st>>>(n, piv, perm);
  const unsigned idg = (unsigned)(n < 4096 ? n : 4096);
  if (linv) set_identity_f32_kernel<<<idg, 256, 0, st>>>(n, linv);
  if (uinv) set_identity_f32_kernel<<<idg, 256, 0, st>>>(n, uinv);
  const int64_t blk = blk_bytes(n);
  char* wb = reinterpret_cast<char*>(work) + 256;
  float* xt = reinterpret_cast<float*>(wb);
  float* ah = reinterpret_cast<float*>(wb + blk);
  float* al = reinterpret_cast<float*>(wb + 2 * blk);
  float* bh = reinterpret_cast<float*>(wb + 3 * blk);
  float* bl = reinterpret_cast<float*>(wb + 4 * blk);
  const bool split = precision == 1;
  // L^{-1}: top to bottom.  Row block j of W = L^{-1} has nonzeros in
  // columns < j0 + nb only.  (Skipped when linv is NULL: the square QR needs
  // only R^{-1}.)
  for (int j0 = 0; linv && j0 < n; j0 += kInvNB) {
    const int nb = min(kInvNB, n - j0);
    const int ncols = j0 + nb;
    inv_diag_kernel<true><<<(unsigned)((ncols + kInvCols - 1) / kInvCols), kInvCols, 0, st>>>(
        n, j0, nb, lu, linv, 0, ncols, xt);
    const int m2 = n - ncols;
    if (m2 > 0) {
      const float* a21 = lu + (int64_t)ncols * n + j0;
      float* c = linv + (int64_t)ncols * n;
      int rc;
      if (split) {
        rc = tf32_split(m2, nb, a21, n, ah, al, kInvNB, st);
        if (!rc) rc = tf32_split(ncols, kInvNB, xt, kInvNB, bh, bl, kInvNB, st);
        if (!rc)
          rc = gemm_tf32_nt_split(m2, ncols, nb, ah, al, kInvNB, bh, bl, kInvNB, c, n, -1.0f, 1.0f,
                                  err, st);
      } else {
        rc = gemm_tf32_nt(m2, ncols, nb, a21, n, xt, kInvNB, c, n, -1.0f, 1.0f, err, st);
      }
      if (rc) return rc;
    }
  }
  // U^{-1}: bottom to top.  Row block j of W = U^{-1} has nonzeros in
  // columns >= j0 only.  (Skipped when uinv is NULL: a Cholesky factor forms
  // it from L^{-1} with lxgb_chol32_uinv.)
  for (int j0 = ((n - 1) / kInvNB) * kInvNB; uinv && j0 >= 0; j0 -= kInvNB) {
    const int nb = min(kInvNB, n - j0);
    const int ncols = n - j0;
    inv_diag_kernel<false><<<(unsigned)((ncols + kInvCols - 1) / kInvCols), kInvCols, 0, st>>>(
        n, j0, nb, lu, uinv, j0, n, xt);
    if (j0 > 0) {
      const float* a01 = lu + j0;  // rows [0, j0), columns [j0, j0 + nb)
      float* c = uinv + j0;
      int rc;
      if (split) {
        rc = tf32_split(j0, nb, a01, n, ah, al, kInvNB, st);
        if (!rc) rc = tf32_split(ncols, kInvNB, xt, kInvNB, bh, bl, kInvNB, st);
        if (!rc)
          rc = gemm_tf32_nt_split(j0, ncols, nb, ah, al, kInvNB, bh, bl, kInvNB, c, n, -1.0f, 1.0f,
                                  err, st);
      } else {
        rc = gemm_tf32_nt(j0, ncols, nb, a01, n, xt, kInvNB, c, n, -1.0f, 1.0f, err, st);
      }
      if (rc) return rc;
    }
  }
  return check_launch("lu32_inverse");
}

extern "C" int64_t lxgb_lu32_apply_workspace_size(int32_t n, int32_t nrhs) {
  return 4 * vec_bytes(n, nrhs);
}

extern "C" int lxgb_lu32_apply(int32_t n, int32_t nrhs, const float* linv, const float* uinv,
                               const int32_t* perm, int32_t mode, const double* x, double* y,
                               void* work, int64_t work_bytes, void* stream) {
  LXGB_REQUIRE(mode == 0 || mode == 1, "lu32_apply: mode must be 0 (FP32) or 1 (double-float)");
  LXGB_REQUIRE(n >= 0 && nrhs >= 0, "lu32_apply: negative size");
  if (n == 0 || nrhs == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(linv && uinv && perm && x && y && work, "lu32_apply: null pointer");
  if (work_bytes < lxgb_lu32_apply_workspace_size(n, nrhs)) {
    set_last_error("lu32_apply: workspace too small");
    return LXGB_WORKSPACE_TOO_SMALL;
  }
  cudaStream_t st = as_stream(stream);
  const int64_t vb = vec_bytes(n, nrhs);
  char* wb = reinterpret_cast<char*>(work);
  float* zh = reinterpret_cast<float*>(wb);
  float* zl = reinterpret_cast<float*>(wb + vb);
  float* th = reinterpret_cast<float*>(wb + 2 * vb);
  float* tl = reinterpret_cast<float*>(wb + 3 * vb);
  const int64_t total = (int64_t)n * nrhs;
  const unsigned g = (unsigned)((total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096);
  split_rows_kernel<<<g, 256, 0, st>>>(nrhs, n, x, n, perm, zh, mode ? zl : nullptr, n);
  int rc;
  if (mode == 0) {
    rc = launch_gemv16<0, 1, 0>(n, n, linv, nullptr, n, nrhs, zh, nullptr, n, th, nullptr, nullptr,
                                nullptr, n, st);
    if (!rc)
      rc = launch_gemv16<0, 2, 1>(n, n, uinv, nullptr, n, nrhs, th, nullptr, n, nullptr, nullptr,
                                  y, nullptr, n, st);
  } else {
    rc = launch_gemv16<1, 1, 0>(n, n, linv, nullptr, n, nrhs, zh, zl, n, th, tl, nullptr, nullptr,
                                n, st);
    if (!rc)
      rc = launch_gemv16<1, 2, 1>(n, n, uinv, nullptr, n, nrhs, th, tl, n, nullptr, nullptr, y,
                                  nullptr, n, st);
  }
  return rc;
}

extern "C" int64_t lxgb_qr32_apply_workspace_size(int32_t n, int32_t nrhs) {
  return 4 * vec_bytes(n, nrhs);
}

extern "C" int lxgb_qr32_apply(int32_t n, int32_t nrhs, const float* qt, const float* rinv,
                               int32_t mode, const double* x, double* y, void* work,
                               int64_t work_bytes, void* stream) {
  LXGB_REQUIRE(mode == 0 || mode == 1, "qr32_apply: mode must be 0 (FP32) or 1 (double-float)");
  LXGB_REQUIRE(n >= 0 && nrhs >= 0, "qr32_apply: negative size");
  if (n == 0 || nrhs == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(qt && rinv && x && y && work, "qr32_apply: null pointer");
  if (work_bytes < lxgb_qr32_apply_workspace_size(n, nrhs)) {
    set_last_error("qr32_apply: workspace too small");
    return LXGB_WORKSPACE_TOO_SMALL;
  }
  cudaStream_t st = as_stream(stream);
  const int64_t vb = vec_bytes(n, nrhs);
  char* wb = reinterpret_cast<char*>(work);
  float* zh = reinterpret_cast<float*>(wb);
  float* zl = reinterpret_cast<float*>(wb + vb);
  float* th = reinterpret_cast<float*>(wb + 2 * vb);
  float* tl = reinterpret_cast<float*>(wb + 3 * vb);
  const int64_t total = (int64_t)n * nrhs;
  const unsigned g = (unsigned)((total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096);
  split_rows_kernel<<<g, 256, 0, st>>>(nrhs, n, x, n, nullptr, zh, mode ? zl : nullptr, n);
  int rc;
  if (mode == 0) {
    rc = launch_gemv16<0, 0, 0>(n, n, qt, nullptr, n, nrhs, zh, nullptr, n, th, nullptr, nullptr,
                                nullptr, n, st);
    if (!rc)
      rc = launch_gemv16<0, 2, 1>(n, n, rinv, nullptr, n, nrhs, th, nullptr, n, nullptr, nullptr,
                                  y, nullptr, n, st);
  } else {
    rc = launch_gemv16<1, 0, 0>(n, n, qt, nullptr, n, nrhs, zh, zl, n, th, tl, nullptr, nullptr,
                                n, st);
    if (!rc)
      rc = launch_gemv16<1, 2, 1>(n, n, rinv, nullptr, n, nrhs, th, tl, n, nullptr, nullptr, y,
                                  nullptr, n, st);
  }
  return rc;
}

extern "C" int lxgb_split_f64(int64_t rows, int64_t cols, const double* a, int64_t lda, float* hi,
                              float* lo, int64_t ld, void* stream) {
  LXGB_REQUIRE(rows >= 0 && cols >= 0, "split_f64: negative size");
  if (rows == 0 || cols == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(a && hi, "split_f64: null pointer");
  LXGB_REQUIRE(lda >= cols && ld >= cols, "split_f64: leading dimension too small");
  const int64_t total = rows * cols;
  const unsigned g = (unsigned)((total + 255) / 256 < 8192 ? (total + 255) / 256 : 8192);
  split_matrix_kernel<<<g, 256, 0, as_stream(stream)>>>(rows, cols, a, lda, hi, lo, ld);
  return check_launch("split_f64");
}

extern "C" int64_t lxgb_gemv_df_workspace_size(int32_t n, int32_t nrhs) {
  return 2 * vec_bytes(n, nrhs);
}

extern "C" int lxgb_gemv_df(int32_t m, int32_t n, const float* a_hi, const float* a_lo,
                            int64_t lda, int32_t nrhs, const double* x, int64_t ldx,
                            const double* b, double* y, int64_t ldy, int32_t mode, void* work,
                            int64_t work_bytes, void* stream) {
  LXGB_REQUIRE(mode == 0 || mode == 1, "gemv_df: mode must be 0 (FP32) or 1 (double-float)");
  LXGB_REQUIRE(m >= 0 && n >= 0 && nrhs >= 0, "gemv_df: negative size");
  if (m == 0 || nrhs == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(a_hi && y && (n == 0 || x) && work, "gemv_df: null pointer");
  LXGB_REQUIRE(lda >= n && ldx >= n && ldy >= m, "gemv_df: leading dimension too small");
  if (work_bytes < lxgb_gemv_df_workspace_size(n, nrhs)) {
    set_last_error("gemv_df: workspace too small");
    return LXGB_WORKSPACE_TOO_SMALL;
  }
  cudaStream_t st = as_stream(stream);
  const int64_t vb = vec_bytes(n, nrhs);
  float* xh = reinterpret_cast<float*>(work);
  float* xl = reinterpret_cast<float*>(reinterpret_cast<char*>(work) + vb);
  const int nn = n > 0 ? n : 1;
  if (n > 0) {
    const int64_t total = (int64_t)n * nrhs;
    const unsigned g = (unsigned)((total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096);
    split_rows_kernel<<<g, 256, 0, st>>>(nrhs, n, x, ldx, nullptr, xh, mode ? xl : nullptr, nn);
  }
  const bool res = b != nullptr;
  if (mode == 1 && nrhs <= 4 && n > 0) {
    // few right-hand sides: one warp per row (the 16 × 16 tiles would idle)
    switch (nrhs * 2 + (a_lo ? 1 : 0)) {
      case 2: launch_rows_df<1, false>(m, n, a_hi, a_lo, lda, xh, xl, nn, y, b, ldy, st); break;
      case 3: launch_rows_df<1, true>(m, n, a_hi, a_lo, lda, xh, xl, nn, y, b, ldy, st); break;
      case 4: launch_rows_df<2, false>(m, n, a_hi, a_lo, lda, xh, xl, nn, y, b, ldy, st); break;
      case 5: launch_rows_df<2, true>(m, n, a_hi, a_lo, lda, xh, xl, nn, y, b, ldy, st); break;
      case 6: launch_rows_df<3, false>(m, n, a_hi, a_lo, lda, xh, xl, nn, y, b, ldy, st); break;
      case 7: launch_rows_df<3, true>(m, n, a_hi, a_lo, lda, xh, xl, nn, y, b, ldy, st); break;
      case 8: launch_rows_df<4, false>(m, n, a_hi, a_lo, lda, xh, xl, nn, y, b, ldy, st); break;
      default: launch_rows_df<4, true>(m, n, a_hi, a_lo, lda, xh, xl, nn, y, b, ldy, st); break;
    }
    return check_launch("gemv_df");
  }
  if (mode == 0)
    return res ? launch_gemv16<0, 0, 2>(m, n, a_hi, nullptr, lda, nrhs, xh, nullptr, nn, nullptr,
                                        nullptr, y, b, ldy, st)
               : launch_gemv16<0, 0, 1>(m, n, a_hi, nullptr, lda, nrhs, xh, nullptr, nn, nullptr,
                                        nullptr, y, nullptr, ldy, st);
  if (a_lo)
    return res ? launch_gemv16<2, 0, 2>(m, n, a_hi, a_lo, lda, nrhs, xh, xl, nn, nullptr, nullptr,
                                        y, b, ldy, st)
               : launch_gemv16<2, 0, 1>(m, n, a_hi, a_lo, lda, nrhs, xh, xl, nn, nullptr, nullptr,
                                        y, nullptr, ldy, st);
  return res ? launch_gemv16<1, 0, 2>(m, n, a_hi, nullptr, lda, nrhs, xh, xl, nn, nullptr, nullptr,
                                      y, b, ldy, st)
             : launch_gemv16<1, 0, 1>(m, n, a_hi, nullptr, lda, nrhs, xh, xl, nn, nullptr, nullptr,
                                      y, nullptr, ldy, st);
}
