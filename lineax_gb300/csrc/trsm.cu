// General triangular solve op(T) X = B (lower/upper, trans, unit diagonal),
// FP64: one CTA per right-hand side with the vector staged in shared memory,
// or for large n a multi-CTA blocked solve (below).
#include "common.cuh"
#include "tri.cuh"

namespace lxgb {

constexpr int kTrsmThreads = 256;
// From this order on the multi-CTA blocked solve replaces the one-CTA one.
constexpr int kTrsmBlockedMin = 768;

__global__ void __launch_bounds__(kTrsmThreads)
trsm_kernel(int n, const double* __restrict__ t, int64_t ldt, int lower, int trans, int unit,
            double* __restrict__ b, int in_smem) {
  extern __shared__ double smem_v[];
  __shared__ TrsvSmem<double> tsm;
  double* g = b + (int64_t)blockIdx.x * n;
  double* x = in_smem ? smem_v : g;
  if (in_smem) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] = g[i];
    __syncthreads();
  }
  cta_trsv<double>(t, ldt, n, lower != 0, trans != 0, unit != 0, x, tsm);
  if (in_smem)
    for (int i = threadIdx.x; i < n; i += blockDim.x) g[i] = x[i];
}

// --- multi-CTA blocked solve for large n ------------------------------------
// One CTA per right-hand side runs the substitution of the whole vector; for
// large n that chain of dependent block steps is latency-bound.  The blocked
// form splits each 64-row block step into (1) the substitution inside the
// block, one CTA per right-hand side with the block in shared memory, and (2)
// the update of every row not yet solved by the block's solved unknowns,
// spread over many CTAs (right-looking).
constexpr int kTbNB = 64;

__device__ __forceinline__ double op_t(const double* __restrict__ t, int64_t ldt, bool trans,
                                       int64_t i, int64_t j) {
  return trans ? t[j * ldt + i] : t[i * ldt + j];
}

// Block [r0, r0+rn) of op(T) x = b for right-hand side blockIdx.x (vector c at
// b + c*n), in place: warp 0 with two unknowns per lane, the block staged.
__global__ void __launch_bounds__(256)
trsm_block_diag_kernel(int n, const double* __restrict__ t, int64_t ldt, int trans, int unit,
                       int fwd, int r0, int rn, double* __restrict__ b) {
  __shared__ double d[kTbNB][kTbNB + 1];
  for (int e = threadIdx.x; e < kTbNB * kTbNB; e += blockDim.x) {
    const int ii = e / kTbNB, jj = e % kTbNB;
    d[ii][jj] = (ii < rn && jj < rn) ? op_t(t, ldt, trans, r0 + ii, r0 + jj) : 0.0;
  }
  __syncthreads();
  if (threadIdx.x >= 32) return;
  const int lane = threadIdx.x;
  double* x = b + (int64_t)blockIdx.x * n + r0;
  double v0 = (lane < rn) ? x[lane] : 0.0;
  double v1 = (lane + 32 < rn) ? x[lane + 32] : 0.0;
  for (int step = 0; step < rn; ++step) {
    const int tt = fwd ? step : rn - 1 - step;
    const bool hi = tt >= 32;
    const int src = tt & 31;
    double mine = hi ? v1 : v0;
    if (lane == src && !unit) mine = mine / d[tt][tt];
    const double xt = __shfl_sync(0xffffffffu, mine, src);
    if (lane == src) { if (hi) v1 = xt; else v0 = xt; }
    // rows solved after tt take its contribution
    const int i0 = lane, i1 = lane + 32;
    if (fwd ? (i0 > tt) : (i0 < tt)) v0 = fma(-d[i0][tt], xt, v0);
    if (i1 < rn && (fwd ? (i1 > tt) : (i1 < tt))) v1 = fma(-d[i1][tt], xt, v1);
  }
  if (lane < rn) x[lane] = v0;
  if (lane + 32 < rn) x[lane + 32] = v1;
}

// Rows [lo, hi) of every right-hand side: x_i -= sum_{p in block} op(T)[i][p] x_p.
// op(T)[i][·] contiguous (no transpose): a warp per (row, vector), lanes over p;
// otherwise a thread per row, p in the loop (op(T)[·][p] contiguous in i).
__global__ void __launch_bounds__(256)
trsm_block_update_kernel(int n, const double* __restrict__ t, int64_t ldt, int trans, int r0,
                         int rn, int lo, int hi, int nrhs, double* __restrict__ b) {
  __shared__ double xb[kTbNB];
  const int c = blockIdx.y;
  double* x = b + (int64_t)c * n;
  for (int p = threadIdx.x; p < kTbNB; p += blockDim.x) xb[p] = (p < rn) ? x[r0 + p] : 0.0;
  __syncthreads();
  if (!trans) {
    const int lane = threadIdx.x & 31;
    const int warps = (int)(gridDim.x * (blockDim.x >> 5));
    for (int i = lo + (int)(blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)); i < hi;
         i += warps) {
      const double* row = t + (int64_t)i * ldt + r0;
      double acc = 0.0;
      if (lane < rn) acc = row[lane] * xb[lane];
      if (lane + 32 < rn) acc = fma(row[lane + 32], xb[lane + 32], acc);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if (lane == 0) x[i] -= acc;
    }
  } else {
    for (int i = lo + (int)(blockIdx.x * blockDim.x + threadIdx.x); i < hi;
         i += (int)(gridDim.x * blockDim.x)) {
      double acc = 0.0;
      for (int p = 0; p < rn; ++p) acc = fma(t[(int64_t)(r0 + p) * ldt + i], xb[p], acc);
      x[i] -= acc;
    }
  }
}

static int trsm_blocked(int n, int nrhs, const double* t, int64_t ldt, int lower, int trans,
                        int unit, double* b, cudaStream_t st) {
  const bool fwd = (lower != 0) != (trans != 0);
  const int nblk = (n + kTbNB - 1) / kTbNB;
  for (int bi = 0; bi < nblk; ++bi) {
    const int blk = fwd ? bi : nblk - 1 - bi;
    const int r0 = blk * kTbNB;
    const int rn = (n - r0 < kTbNB) ? n - r0 : kTbNB;
    trsm_block_diag_kernel<<<(unsigned)nrhs, 256, 0, st>>>(n, t, ldt, trans, unit, fwd, r0, rn, b);
    const int lo = fwd ? r0 + rn : 0, hi = fwd ? n : r0;
    if (hi > lo) {
      const int rows = hi - lo;
      const int per_cta = trans ? 256 : 8;
      int g = (rows + per_cta - 1) / per_cta;
      const int cap = 2 * sm_count();
      if (g > cap) g = cap;
      trsm_block_update_kernel<<<dim3((unsigned)g, (unsigned)nrhs), 256, 0, st>>>(
          n, t, ldt, trans, r0, rn, lo, hi, nrhs, b);
    }
  }
  return check_launch("trsm blocked");
}

}  // namespace lxgb

using namespace lxgb;

extern "C" int lxgb_trsm_f64(int32_t n, int32_t nrhs, const double* t, int64_t ldt, int32_t lower,
                             int32_t trans, int32_t unit_diag, double* b, void* stream) {
  LXGB_REQUIRE(n >= 0 && nrhs >= 0, "trsm: negative size");
  if (n == 0 || nrhs == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(t && b, "trsm: null pointer");
  LXGB_REQUIRE(ldt >= n, "trsm: ldt < n");
  if (n >= kTrsmBlockedMin && nrhs <= 65535)
    return trsm_blocked(n, nrhs, t, ldt, lower, trans, unit_diag, b, as_stream(stream));
  const size_t need = (size_t)n * sizeof(double);
  const int in_smem = need <= 160 * 1024;
  const size_t smem = in_smem ? need : 0;
  if (in_smem)
    LXGB_CUDA_TRY(ensure_dynamic_smem(reinterpret_cast<const void*>(trsm_kernel), (int)smem),
                  "trsm: set smem");
  trsm_kernel<<<(unsigned)nrhs, kTrsmThreads, smem, as_stream(stream)>>>(
      n, t, ldt, lower, trans, unit_diag, b, in_smem);
  return check_launch("trsm");
}
