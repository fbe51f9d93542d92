// Cholesky factorisation (upper, A = Uᵀ U) of ragged batches, the matching
// solve, and the mixed-precision solve (FP32 factor + FP64 refinement).
//
// One persistent launch covers a ragged batch: in the mixed path CTAs pull
// systems from an atomic work queue, largest order first (a counting sort by
// n ahead of the launch), in the plain FP64 path they take them round-robin.  Each system is factored by one CTA with
// a right-looking blocked algorithm; the matrix is staged in shared memory
// when it fits and otherwise factored where it lies (FP64 path: in place in
// the caller's buffer; FP32 path: in a per-CTA slice of the workspace), where
// it stays L2-resident while the CTA works on it.
#include <float.h>

#include <atomic>

#include "common.cuh"
#include "df.cuh"
#include "potrf.cuh"
#include "tcgen05.cuh"
#include "tri.cuh"

namespace lxgb {

constexpr int kCholThreads = 256;
// Largest order factored in shared memory: FP64 160*161*8 B = 206 KB,
// FP32 224*225*4 B = 202 KB (+ the correction vectors of the mixed path).
constexpr int kCholSmemMaxF64 = 160;
constexpr int kQueueHeader = 256;  // bytes reserved for the work-queue counter

__device__ __forceinline__ int next_system(int* queue, int* s_next) {
  __syncthreads();
  if (threadIdx.x == 0) *s_next = atomicAdd(queue, 1);
  __syncthreads();
  return *s_next;
}

// ---------------------------------------------------------------------------
// Plain FP64 ragged potrf.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kCholThreads)
potrf_ragged_f64_kernel(int64_t batch, int max_n, const int32_t* __restrict__ nvec,
                        const int64_t* __restrict__ a_off, double* __restrict__ a,
                        int32_t* __restrict__ info) {
  extern __shared__ double smem_chol[];
  // Static round-robin over systems: deterministic, and needs no scratch
  // counter (this entry point has no workspace argument).
  for (int64_t s = blockIdx.x; s < batch; s += gridDim.x) {
    __syncthreads();
    const int n = nvec[s];
    double* g = a + a_off[s];
    if (n > max_n || n < 0) {
      if (threadIdx.x == 0) info[s] = -2;
      continue;
    }
    int rc;
    if (n <= kCholSmemMaxF64) {
      const int ld = n | 1;
      for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int i = e / n, j = e - i * n;
        smem_chol[i * ld + j] = g[e];
      }
      __syncthreads();
      rc = cta_potrf_upper<double, 16>(smem_chol, ld, n);
      __syncthreads();
      for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int i = e / n, j = e - i * n;
        g[e] = (j >= i) ? smem_chol[i * ld + j] : 0.0;
      }
    } else {
      rc = cta_potrf_upper<double, 32>(g, n, n);
      __syncthreads();
      for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int i = e / n, j = e - i * n;
        if (j < i) g[e] = 0.0;
      }
    }
    if (threadIdx.x == 0) info[s] = rc;
  }
}

// ---------------------------------------------------------------------------
// FP64 ragged potrs: one CTA per (system, rhs) pair is wasteful for ragged
// batches with few vectors each, so one CTA handles a system and loops over
// its vectors.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kCholThreads)
potrs_ragged_f64_kernel(int64_t batch, int max_n, const int32_t* __restrict__ nvec,
                        const int32_t* __restrict__ nrhs, const int64_t* __restrict__ a_off,
                        const double* __restrict__ u, const int64_t* __restrict__ b_off,
                        double* __restrict__ b) {
  extern __shared__ double smem_x[];
  __shared__ TrsvSmem<double> tsm;
  for (int64_t s = blockIdx.x; s < batch; s += gridDim.x) {
    const int n = nvec[s];
    if (n > max_n || n <= 0) continue;
    const double* U = u + a_off[s];
    for (int r = 0; r < nrhs[s]; ++r) {
      double* g = b + b_off[s] + (int64_t)r * n;
      for (int i = threadIdx.x; i < n; i += blockDim.x) smem_x[i] = g[i];
      __syncthreads();
      cta_trsv<double>(U, n, n, /*lower=*/false, /*trans=*/true, /*unit=*/false, smem_x, tsm);
      cta_trsv<double>(U, n, n, /*lower=*/false, /*trans=*/false, /*unit=*/false, smem_x, tsm);
      for (int i = threadIdx.x; i < n; i += blockDim.x) g[i] = smem_x[i];
      __syncthreads();
    }
  }
}

// ---------------------------------------------------------------------------
// Mixed precision: FP32 factor, FP64-accurate refinement.
//
// One persistent launch, two 256-thread CTAs per SM, systems from an atomic
// queue.  Per system:
//  * factor in FP32 — n <= kMxSmallN: right-looking in shared memory with
//    16-column panels (diagonal block by one warp, column-parallel TRSM of the
//    block row, register-tiled SYRK of the trailing matrix: three barriers per
//    panel); larger n: right-looking by 32-row block rows of U kept in this
//    CTA's workspace slice (an FP32 n×n array, L2-resident while the CTA works
//    on it) — TRSM of the block row, then a register-tiled SYRK of the
//    trailing matrix, during which one warp updates and factors the next
//    diagonal block (lookahead);
//  * all right-hand sides of a chunk (<= 8) solved together with the FP32
//    factor (blocked forward/backward substitution, one warp per vector on the
//    32×32 diagonal blocks, all threads on the off-diagonal updates);
//  * refinement: r = b - A x to FP64 accuracy from the FP64 matrix with
//    error-free FP32 transformations — A and x are split bitwise into hi+lo
//    FP32 pairs (|a - hi - lo| <= 2^-46 |a|), hi*hi products are made exact
//    with an FMA (TwoProd) and summed with TwoSum, lower-order terms in a
//    second FP32 accumulator.  GB300 issues one FP64 FMA per ~68 FP32 lane
//    operations, so this costs ~6x less than native FP64 while keeping the
//    residual's error near 1e-14 of ||A|| ||x||;
//  * x accumulated in FP64; a right-hand side is frozen once its normwise
//    backward error is <= tol (its result is the same alone or in a batch).
// ---------------------------------------------------------------------------
constexpr int kMxThreads = 256;
constexpr int kMxSmallN = 144;   // 144*145*4 B = 82 KB factor in shared memory (the most)
constexpr int kMxKc = 8;         // right-hand sides per refinement chunk
constexpr int kMxNB = 32;        // block rows of the large path and of the solves
constexpr int kMxMaxN = 1024;

struct MxSmem {
  float rd[kMxMaxN];                     // 1 / diagonal of the FP32 factor
  float ublk[kMxNB][kMxNB + 1];          // the current diagonal block of U
  float linv[kMxNB][kMxNB + 1];          // its inverse transpose, U_JJ^{-T} (lower)
  float red[kMxThreads / 32][kMxKc];     // per-warp partial maxima
  float red2[kMxThreads / 32][kMxKc + 1];  // [0]: row-sum max, [1 + c]: max |x_c|
  float anorm;
  float bnorm[kMxKc];
  double berr[kMxKc];
  int done[kMxKc];
  int next;
  int flag;
  int tcstat;                     // status of the tensor-core update (0 or -3)
  unsigned tcphase;               // completed phases of tcbar
  unsigned tmem;                  // tensor-memory accumulator (128 columns) of the update
  alignas(8) unsigned long long tcbar;  // completion of the update's MMAs
};


// Split W FP64 values, given as their two 32-bit words (x = low, y = high),
// with one warp vote (see split_f64).  Only 32-bit integer operations run on
// the common path.
template <int W>
__device__ __forceinline__ void splitw(const uint2 (&a)[W], float (&hi)[W], float (&lo)[W]) {
  bool slow = false;
#pragma unroll
  for (int u = 0; u < W; ++u) {
    const unsigned wl = a[u].x, wh = a[u].y;
    const unsigned e = (wh >> 20) & 0x7FFu;
    const unsigned sign = wh & 0x80000000u;
    const unsigned mh = ((wh & 0xFFFFFu) << 3) | (wl >> 29);
    const unsigned rem = wl & 0x1FFFFFFFu;
    const int sh = __clz(rem | 1u) - 8;
    const unsigned m = (sh >= 0) ? (rem << sh) : (rem >> (-sh));
    const int ex = (int)e - 1052 - sh + 127;
    const bool zero = ((wh << 1) | wl) == 0u;
    hi[u] = zero ? __uint_as_float(sign) : __uint_as_float(sign | (((e - 1023u + 127u) & 0xFFu) << 23) | mh);
    lo[u] = (rem == 0u) ? 0.0f : __uint_as_float(sign | (((unsigned)ex & 0xFFu) << 23) | (m & 0x7FFFFFu));
    slow |= !zero && ((e < 949u) || (e > 1150u));
  }
  if (__any_sync(__activemask(), slow)) {
#pragma unroll
    for (int u = 0; u < W; ++u) {
      const unsigned wl = a[u].x, wh = a[u].y;
      const unsigned e = (wh >> 20) & 0x7FFu;
      if (((wh << 1) | wl) != 0u && ((e < 949u) || (e > 1150u))) {
        const double d = __hiloint2double((int)wh, (int)wl);
        hi[u] = __double2float_rz(d);
        lo[u] = __double2float_rn(d - (double)hi[u]);
      }
    }
  }
}

// FP32 copy (the hi part of split_f64) of the upper triangle of the row-major
// n×n FP64 matrix A into F (row stride ld).  A warp walks 256-column chunks of
// its rows (j >= i); the next chunk's eight loads per lane are issued before
// the current one is converted, so two chunks are in flight (the copy streams
// A from DRAM and was latency-bound one chunk at a time).
__device__ __forceinline__ void mx_copy_upper(const double* __restrict__ A, int n, float* F,
                                              int64_t ld) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  auto load = [&](int r, int j0, uint2 (&v)[8]) {
    const uint2* arow = reinterpret_cast<const uint2*>(A + (int64_t)r * n);
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int j = j0 + lane + 32 * u;
      v[u] = (r < n && j < n) ? arow[j] : make_uint2(0u, 0u);
    }
  };
  int i = warp, j0 = warp;
  uint2 v[8];
  load(i, j0, v);
  while (i < n) {
    int ni = i, nj = j0 + 256;
    if (nj >= n) { ni = i + nw; nj = ni; }
    uint2 vn[8];
    load(ni, nj, vn);
    float hi[8], lo[8];
    splitw<8>(v, hi, lo);
    float* frow = F + (int64_t)i * ld;
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int j = j0 + lane + 32 * u;
      if (j < n) frow[j] = hi[u];
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) v[u] = vn[u];
    i = ni;
    j0 = nj;
  }
}

// Factor the nb×nb diagonal block at F[j0.., j0..] (upper triangle, row
// stride ld) by one warp entirely in registers: lane j holds column j; row k
// of U is formed in place and rows i > k updated with u_ki fetched by shuffle.
// The block is padded to NBMAX with the identity, so every step runs
// unconditionally (shuffles outside data-dependent branches); a pivot that is
// not positive is recorded, not branched on.  Writes U_JJ back to F and to
// ublk (NBMAX×(NBMAX+1) shared array) and 1/diag into rd[0..nb).  Returns 0 or
// (j0+k+1) for the first pivot that is not positive.
template <int NBMAX>
__device__ __noinline__ int warp_potrf_block(float* F, int64_t ld, int j0, int nb, float* rd, float* ublk,
                                             float* linv) {
  const int lane = threadIdx.x & 31;
  const int ldi = (int)ld;
  float* base = F + (int64_t)j0 * ld + j0 + lane;  // row i of the block at base + i * ldi
  float col[NBMAX];
#pragma unroll
  for (int i = 0; i < NBMAX; ++i) {
    const bool in = (i < nb) && (i <= lane) && (lane < nb);
    col[i] = in ? base[i * ldi] : ((i == lane) ? 1.0f : 0.0f);
  }
  // Linv = U_JJ^{-T} in the same loop: lane j carries column j of Linv, z_k =
  // (e_k - sum_{q<k} U[q][k] z_q) / U[k][k], whose sums acc[k] grow by
  // U[k][i] z_k as each row k of U is broadcast for the rank-1 update — no
  // second pass of dependent substitutions.
  float acc[NBMAX];
#pragma unroll
  for (int i = 0; i < NBMAX; ++i) acc[i] = 0.0f;
  int bad = 0;
#pragma unroll
  for (int k = 0; k < NBMAX; ++k) {
    const float akk = __shfl_sync(0xffffffffu, col[k], k);
    if (!(akk > 0.0f) && bad == 0) bad = j0 + k + 1;
    const float d = sqrtf(akk);
    const float r = 1.0f / d;
    col[k] = (lane == k) ? d : ((lane > k) ? col[k] * r : col[k]);
    if (lane == 0 && k < nb) rd[k] = r;
    const float zk = (((lane == k) ? 1.0f : 0.0f) - acc[k]) * r;
    if (lane < NBMAX) linv[k * (NBMAX + 1) + lane] = zk;
#pragma unroll
    for (int i = k + 1; i < NBMAX; ++i) {
      const float uki = __shfl_sync(0xffffffffu, col[k], i);
      col[i] = (lane >= i) ? fmaf(-uki, col[k], col[i]) : col[i];
      acc[i] = fmaf(uki, zk, acc[i]);
    }
  }
#pragma unroll
  for (int i = 0; i < NBMAX; ++i)
    if (bad == 0 && i < nb && i <= lane && lane < nb) base[i * ldi] = col[i];
  __syncwarp();
  return bad;
}

// Rows [kb, kb+nb) of the block row: U[kb:kb+nb, j] = U_kk^{-T} A[kb:kb+nb, j]
// for columns j in [j_lo, n), one column per thread, as a triangular
// matrix-vector product with Linv = U_kk^{-T} (shared): each output row is
// formed and stored at once, keeping register pressure at one column.
template <int NBMAX>
__device__ __noinline__ void block_row_trsm(float* F, int64_t ld, int kb, int nb, int j_lo, int n,
                                            const float* linv) {
  const int ldi = (int)ld;  // 32-bit row offsets: one base address per column
  for (int j = j_lo + threadIdx.x; j < n; j += blockDim.x) {
    float* col = F + (int64_t)kb * ld + j;
    float a[NBMAX];
#pragma unroll
    for (int p = 0; p < NBMAX; ++p) a[p] = (p < nb) ? col[p * ldi] : 0.0f;
#pragma unroll
    for (int p = 0; p < NBMAX; ++p) {
      float y[4] = {0.0f, 0.0f, 0.0f, 0.0f};  // four chains instead of one
#pragma unroll
      for (int q = 0; q <= p; ++q) y[q & 3] = fmaf(linv[p * (NBMAX + 1) + q], a[q], y[q & 3]);
      if (p < nb) col[p * ldi] = (y[0] + y[1]) + (y[2] + y[3]);
    }
  }
}

// --- small path: right-looking in shared memory ---------------------------
// Returns 0 or k+1.  F row stride ld, upper triangle.
__device__ __noinline__ int mx_factor_small(float* F, int ld, int n, MxSmem& sm) {
  const int tid = threadIdx.x, warp = tid >> 5;
  const int tx = tid & 15, ty = tid >> 4;
  for (int kb = 0; kb < n; kb += 16) {
    const int ke = min(kb + 16, n);
    if (warp == 0) {
      const int bad = warp_potrf_block<16>(F, ld, kb, ke - kb, sm.rd + kb, &sm.ublk[0][0],
                                           &sm.linv[0][0]);
      if ((tid & 31) == 0) sm.flag = bad;
    }
    __syncthreads();
    if (sm.flag) return sm.flag;
    block_row_trsm<16>(F, ld, kb, ke - kb, ke, n, &sm.linv[0][0]);
    __syncthreads();
    // trailing update of [ke, n): F[i][j] -= sum_p F[p][i] F[p][j], j >= i
    const int m = n - ke;
    if (m > 0) {
      const int tiles = (m + 63) >> 6;
      for (int t = 0; t < tiles * tiles; ++t) {
        const int ti = t / tiles, tj = t % tiles;
        if (tj < ti) continue;
        const int i0 = ke + (ti << 6), j0 = ke + (tj << 6);
        float acc[4][4];
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            const int i = i0 + ty + 16 * r, j = j0 + tx + 16 * c;
            acc[r][c] = (i < n && j < n && j >= i) ? F[i * ld + j] : 0.0f;
          }
        for (int p = kb; p < ke; ++p) {
          float ui[4], uj[4];
#pragma unroll
          for (int r = 0; r < 4; ++r) {
            const int i = i0 + ty + 16 * r;
            ui[r] = (i < n) ? F[p * ld + i] : 0.0f;
          }
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            const int j = j0 + tx + 16 * c;
            uj[c] = (j < n) ? F[p * ld + j] : 0.0f;
          }
#pragma unroll
          for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int c = 0; c < 4; ++c) acc[r][c] = fmaf(-ui[r], uj[c], acc[r][c]);
        }
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            const int i = i0 + ty + 16 * r, j = j0 + tx + 16 * c;
            if (i < n && j < n && j >= i) F[i * ld + j] = acc[r][c];
          }
      }
      __syncthreads();
    }
  }
  return 0;
}

// --- large path: right-looking by 32-row block rows, U in global ----------
// U (row stride ldu = n rounded up to 32, so 8-float tiles stay inside the
// row) first receives the upper triangle of A in FP32.  Per block row J:
// the diagonal block by one warp in registers, the TRSM of the rest of the
// block row (U_JJ from shared memory), the block row staged in shared memory
// (up to kMxStageCols columns), then the trailing update of the upper
// triangle in 8×8 register tiles, U[i][j] -= sum_p U[p][i] U[p][j].
constexpr int kMxStageCols = 512;

struct MxStage {
  float brow[kMxNB][kMxStageCols];
};

// --- trailing update on the tensor cores ------------------------------------
// C -= Wᵀ W for the upper triangle of the trailing matrix, W = U[j0:j0+nb,
// t0:n] the block row just formed: 128×128 tiles of C, each the product of
// two 128-row bands of Wᵀ (K = 32) held in shared memory in the 128-byte
// swizzled K-major layout, accumulated in tensor memory by tcgen05.mma with
// split TF32 operands (W = Wh + Wl, both rounded to TF32; Wh Whᵀ + Wh Wlᵀ +
// Wl Whᵀ, three MMAs per K-step of 8), which keeps the update at FP32-level
// accuracy.  Thread 0 issues the MMAs; every warp then reads its 32 TMEM
// lanes (tile rows) × 64 columns back and subtracts them from C.
constexpr int kTcBand = 128;
constexpr int kTcBandFloats = kTcBand * kMxNB;  // 16 KB per band and part

struct TcBands {
  float ah[kTcBandFloats];  // band ti of Wᵀ, hi and lo parts
  float al[kTcBandFloats];
  float bh[kTcBandFloats];  // band tj
  float bl[kTcBandFloats];
};
static_assert(sizeof(TcBands) == 4 * kTcBandFloats * 4, "band layout");

// Rows [128 band, +128) of Wᵀ (Wᵀ[i][p] = U[j0+p][t0+i], zero for p >= nb or
// i >= m) into hi/lo: row r is 128 bytes, 16-byte granule g of row r at
// position g ^ (r & 7) — the layout smem_desc_sw128 describes.
// Stages band `band` with the threads [t_lo, t_lo + nthr) of the CTA.
__device__ __forceinline__ void tc_stage_band(const float* __restrict__ U, int ldu, int j0, int nb,
                                              int t0, int m, int band, float* hi, float* lo,
                                              int t_lo, int nthr) {
  const int me = threadIdx.x - t_lo;
  // all loads first, then the splits and the shared-memory stores, so the
  // loads of one thread are in flight together
  constexpr int kMaxPer = (kTcBand * 8 + 223) / 224;
  float v[kMaxPer][4];
#pragma unroll
  for (int it = 0; it < kMaxPer; ++it) {
    const int e = me + it * nthr;
    const int r = e & (kTcBand - 1), g = e >> 7;
    const int i = band * kTcBand + r;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int p = 4 * g + q;
      v[it][q] = (e < kTcBand * 8 && i < m && p < nb) ? __ldg(U + (int64_t)(j0 + p) * ldu + t0 + i)
                                                      : 0.0f;
    }
  }
#pragma unroll
  for (int it = 0; it < kMaxPer; ++it) {
    const int e = me + it * nthr;
    if (e >= kTcBand * 8) break;
    const int r = e & (kTcBand - 1), g = e >> 7;
    float4 h, l;
    h.x = round_tf32(v[it][0]); l.x = round_tf32(v[it][0] - h.x);
    h.y = round_tf32(v[it][1]); l.y = round_tf32(v[it][1] - h.y);
    h.z = round_tf32(v[it][2]); l.z = round_tf32(v[it][2] - h.z);
    h.w = round_tf32(v[it][3]); l.w = round_tf32(v[it][3] - h.w);
    const int off = r * kMxNB + ((g ^ (r & 7)) << 2);
    *reinterpret_cast<float4*>(hi + off) = h;
    *reinterpret_cast<float4*>(lo + off) = l;
  }
}

// Barrier over warps 1..7 (named barrier 1), with an OR of `flag`.
__device__ __forceinline__ int bar_w17_or(int flag) {
  int r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.s32 q, %1, 0;\n\t"
      "bar.red.or.pred p, 1, 224, q;\n\t"
      "selp.s32 %0, 1, 0, p;\n\t}"
      : "=r"(r)
      : "r"(flag)
      : "memory");
  return r;
}

__device__ __forceinline__ void bar_w17() { asm volatile("bar.sync 1, 224;" ::: "memory"); }

// The update of one trailing step on the tensor cores, and the factor of the
// next diagonal block (rows/columns [t0, t0+32)).  Tile (0,0), which holds
// that block, goes first with every warp; warp 0 then factors the block
// (writing sm.flag) while warps 1..7 run the other tiles behind a named
// barrier — warp 4 then reads TMEM lane quadrant 0 (rows 0..31 of a tile) for
// both column halves.  Returns 0, or -3 if an MMA completion wait timed out
// (after a last bounded wait that lets outstanding MMAs drain).
__device__ __noinline__ int mx_update_tc(float* U, int ldu, int j0, int nb, int t0, int m,
                                         MxSmem& sm, TcBands& tb, unsigned& phase) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nbands = (m + kTcBand - 1) / kTcBand;
  constexpr unsigned idesc = idesc_tf32(kTcBand, kTcBand);
  if (tid == 0) sm.tcstat = 0;
  int t = 0;
  bool out = false;  // warp 0 leaves the tile loop after tile (0,0)
  for (int ti = 0; ti < nbands && !out; ++ti) {
    for (int tj = ti; tj < nbands; ++tj, ++t) {
      const bool solo = t > 0;  // warps 1..7 only from the second tile on
      if (solo && warp == 0) {
        out = true;
        break;
      }
      const int t_lo = solo ? 32 : 0, nthr = solo ? 224 : 256;
      const bool same = tj == ti;
      if (t == 0 || tj == ti) tc_stage_band(U, ldu, j0, nb, t0, m, ti, tb.ah, tb.al, t_lo, nthr);
      if (!same) tc_stage_band(U, ldu, j0, nb, t0, m, tj, tb.bh, tb.bl, t_lo, nthr);
      // generic-proxy smem writes -> visible to the tensor core's async proxy
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      if (solo) bar_w17(); else __syncthreads();
      if (tid == t_lo) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const float* bh = same ? tb.ah : tb.bh;
        const float* bl = same ? tb.al : tb.bl;
#pragma unroll
        for (int k = 0; k < kMxNB / 8; ++k) {  // K = 8 TF32 (32 bytes) per instruction
          const unsigned long long adh = smem_desc_sw128(tb.ah) + ((k * 32) >> 4);
          const unsigned long long adl = smem_desc_sw128(tb.al) + ((k * 32) >> 4);
          const unsigned long long bdh = smem_desc_sw128(bh) + ((k * 32) >> 4);
          const unsigned long long bdl = smem_desc_sw128(bl) + ((k * 32) >> 4);
          mma_tf32(sm.tmem, adh, bdh, idesc, k > 0 ? 1 : 0);
          mma_tf32(sm.tmem, adh, bdl, idesc, 1);
          mma_tf32(sm.tmem, adl, bdh, idesc, 1);
        }
        mma_commit(&sm.tcbar);
      }
      __syncwarp();
      const bool ok = mbar_wait(&sm.tcbar, phase & 1);
      ++phase;
      // one decision for every participating thread
      const int timed_out = solo ? bar_w17_or(!ok) : __syncthreads_or(!ok);
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      if (timed_out) {
        if (!ok) mbar_wait(&sm.tcbar, (phase - 1) & 1);
        if (tid == t_lo) sm.tcstat = -3;
        out = true;
        break;
      }
      // epilogue: warp w reads TMEM lanes 32 (w % 4).. (tile rows); column
      // half w / 4, or both halves for warp 4 while warp 0 is away
      const int quad = warp & 3;
      const int r = 32 * quad + lane;
      const int i = ti * kTcBand + r;
      const int c_first = (solo && quad == 0) ? 0 : 64 * (warp >> 2);
      const int c_count = (solo && quad == 0) ? 4 : 2;
#pragma unroll 1
      for (int cc = 0; cc < c_count; ++cc) {
        const int c0 = c_first + 32 * cc;
        const int jb = tj * kTcBand + c0;
        float* dst = U + (int64_t)(t0 + min(i, m - 1)) * ldu + t0 + jb;
        // the row's eight granules of C are loaded before anything is stored
        float4 c[8];
#pragma unroll
        for (int g = 0; g < 8; ++g) {
          const int col = jb + 4 * g;
          c[g] = (i < m && col < m && col + 3 >= i) ? *reinterpret_cast<const float4*>(dst + 4 * g)
                                                    : make_float4(0.f, 0.f, 0.f, 0.f);
        }
        float v[32];
        tmem_ld32(sm.tmem + ((unsigned)(32 * quad) << 16) + (unsigned)c0, v);
#pragma unroll
        for (int g = 0; g < 8; ++g) {
          const int col = jb + 4 * g;
          if (i < m && col < m && col + 3 >= i) {
            c[g].x -= v[4 * g + 0];
            c[g].y -= v[4 * g + 1];
            c[g].z -= v[4 * g + 2];
            c[g].w -= v[4 * g + 3];
            *reinterpret_cast<float4*>(dst + 4 * g) = c[g];
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      if (solo) bar_w17(); else __syncthreads();  // TMEM and the bands are free again
    }
  }
  __syncwarp();
  if (warp == 0 && sm.tcstat == 0) {
    // the next diagonal block, updated by tile (0,0), while the other warps
    // finish the remaining tiles
    const int bad = warp_potrf_block<kMxNB>(U, ldu, t0, min(kMxNB, m), sm.rd + t0, &sm.ublk[0][0],
                                            &sm.linv[0][0]);
    if (lane == 0) sm.flag = bad;
  }
  // warp 1 waited on every tile's commit: its phase count is everyone's now
  if (tid == 32) sm.tcphase = phase;
  __syncthreads();
  phase = sm.tcphase;
  return sm.tcstat;
}

__device__ __noinline__ int mx_factor_large(const double* __restrict__ A, float* U, int n, int ldu, MxSmem& sm,
                               MxStage& st, bool use_tc, unsigned& phase) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  mx_copy_upper(A, n, U, ldu);
  __syncthreads();
  // Lookahead: warp 0 factors the first diagonal block here and every later
  // one inside the previous block's trailing update (it updates the next
  // diagonal block's tiles first, then factors them while warps 1.. update the
  // rest), so the single-warp factorisation no longer idles the CTA.
  if (warp == 0) {
    const int bad = warp_potrf_block<kMxNB>(U, ldu, 0, min(kMxNB, n), sm.rd, &sm.ublk[0][0],
                                            &sm.linv[0][0]);
    if (lane == 0) sm.flag = bad;
  }
  __syncthreads();
  if (sm.flag) return sm.flag;
  for (int j0 = 0; j0 < n; j0 += kMxNB) {
    const int nb = min(kMxNB, n - j0);
    const int t0 = j0 + nb;          // first trailing row/column
    const int m = n - t0;            // trailing order
    if (m <= 0) break;
    block_row_trsm<kMxNB>(U, ldu, j0, nb, t0, n, &sm.linv[0][0]);
    __syncthreads();
    if (use_tc && m <= kMxStageCols) {
      // tensor-core update, with the next diagonal block factored by warp 0
      TcBands& tb = *reinterpret_cast<TcBands*>(
          (reinterpret_cast<uintptr_t>(&st) + 1023) & ~static_cast<uintptr_t>(1023));
      const int rc = mx_update_tc(U, ldu, j0, nb, t0, m, sm, tb, phase);
      if (rc) return rc;
      if (sm.flag) return sm.flag;
      continue;
    }
    const bool staged = m <= kMxStageCols;
    if (staged) {
      const int m4 = (m + 3) >> 2;
      for (int e = tid; e < kMxNB * m4; e += blockDim.x) {
        const int p = e / m4, q = e % m4;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (p < nb) v = *reinterpret_cast<const float4*>(U + (int64_t)(j0 + p) * ldu + t0 + 4 * q);
        *reinterpret_cast<float4*>(&st.brow[p][4 * q]) = v;
      }
      __syncthreads();
    }
    // 8×8 tiles of the upper triangle of the trailing matrix; the tiles of
    // the next diagonal block (ti <= tj < dt) belong to warp 0.
    const int mt = (m + 7) >> 3;
    const int ntiles = mt * (mt + 1) / 2;
    const int nbn = min(kMxNB, m);
    const int dt = (nbn + 7) >> 3;
    auto tile = [&](int ti, int tj) {
      const int ri = ti << 3, cj = tj << 3;   // offsets inside the trailing matrix
      float acc[8][8];
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        const float* src = U + (int64_t)(t0 + ri + r) * ldu + t0 + cj;
        const float4 a0 = *reinterpret_cast<const float4*>(src);
        const float4 a1 = *reinterpret_cast<const float4*>(src + 4);
        acc[r][0] = a0.x; acc[r][1] = a0.y; acc[r][2] = a0.z; acc[r][3] = a0.w;
        acc[r][4] = a1.x; acc[r][5] = a1.y; acc[r][6] = a1.z; acc[r][7] = a1.w;
      }
      for (int p = 0; p < nb; ++p) {
        float ai[8], bj[8];
        if (staged) {
          const float4 x0 = *reinterpret_cast<const float4*>(&st.brow[p][ri]);
          const float4 x1 = *reinterpret_cast<const float4*>(&st.brow[p][ri + 4]);
          const float4 y0 = *reinterpret_cast<const float4*>(&st.brow[p][cj]);
          const float4 y1 = *reinterpret_cast<const float4*>(&st.brow[p][cj + 4]);
          ai[0] = x0.x; ai[1] = x0.y; ai[2] = x0.z; ai[3] = x0.w;
          ai[4] = x1.x; ai[5] = x1.y; ai[6] = x1.z; ai[7] = x1.w;
          bj[0] = y0.x; bj[1] = y0.y; bj[2] = y0.z; bj[3] = y0.w;
          bj[4] = y1.x; bj[5] = y1.y; bj[6] = y1.z; bj[7] = y1.w;
        } else {
          const float* rowp = U + (int64_t)(j0 + p) * ldu + t0;
#pragma unroll
          for (int q = 0; q < 8; ++q) { ai[q] = rowp[ri + q]; bj[q] = rowp[cj + q]; }
        }
#pragma unroll
        for (int r = 0; r < 8; ++r)
#pragma unroll
          for (int q = 0; q < 8; ++q) acc[r][q] = fmaf(-ai[r], bj[q], acc[r][q]);
      }
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        float* dst = U + (int64_t)(t0 + ri + r) * ldu + t0 + cj;
        *reinterpret_cast<float4*>(dst) = make_float4(acc[r][0], acc[r][1], acc[r][2], acc[r][3]);
        *reinterpret_cast<float4*>(dst + 4) = make_float4(acc[r][4], acc[r][5], acc[r][6], acc[r][7]);
      }
    };
    if (warp == 0) {
      // lane -> (ti, tj) over the dt×dt upper triangle (at most 10 tiles)
      int t = lane, ti = 0;
      while (ti < dt && t >= dt - ti) { t -= dt - ti; ++ti; }
      if (ti < dt) tile(ti, ti + t);
      __syncwarp();
      const int bad = warp_potrf_block<kMxNB>(U, ldu, t0, nbn, sm.rd + t0, &sm.ublk[0][0],
                                              &sm.linv[0][0]);
      if (lane == 0) sm.flag = bad;
    } else {
      for (int t = tid - 32; t < ntiles; t += blockDim.x - 32) {
        // (ti, tj) with tj >= ti from the linear index over the triangle
        int ti = (int)((2.0f * mt + 1.0f - sqrtf((2.0f * mt + 1.0f) * (2.0f * mt + 1.0f) - 8.0f * t)) * 0.5f);
        while (ti > 0 && ti * (2 * mt - ti + 1) / 2 > t) --ti;
        while ((ti + 1) * (2 * mt - ti) / 2 <= t) ++ti;
        const int tj = ti + (t - ti * (2 * mt - ti + 1) / 2);
        if (tj < dt) continue;  // the next diagonal block: warp 0's
        tile(ti, tj);
      }
    }
    __syncthreads();
    if (sm.flag) return sm.flag;
  }
  return 0;
}

// --- solves: (Uᵀ U) D = D for the live vectors of a chunk ------------------
// U row stride ld (shared or global memory); D[i*kMxKc + c] in shared memory;
// rd = 1/diag(U).  The warp solving a 32×32 diagonal block loads its column
// (forward) or row (backward) of the block into registers first, so the
// sequential steps only exchange values by shuffles; the off-diagonal
// updates take one matrix row or column per thread for all NC vectors.
// Off-diagonal updates of the blocked substitution for the first W vectors
// of D (the rest are padding): rows below block [r0, r0+rn) in the forward
// pass, rows above it in the backward pass; one matrix row per thread.  D is
// row-major with kMxKc vectors per row (16-byte aligned rows), so the solved
// values of step t reach every thread as W/4 broadcast 16-byte loads.
template <int W>
__device__ __forceinline__ void mx_rows_fma(float (&v)[W], float u, const float* drow) {
  const float4* d4 = reinterpret_cast<const float4*>(drow);
#pragma unroll
  for (int q = 0; q < W / 4; ++q) {
    const float4 d = d4[q];
    v[4 * q + 0] = fmaf(-u, d.x, v[4 * q + 0]);
    v[4 * q + 1] = fmaf(-u, d.y, v[4 * q + 1]);
    v[4 * q + 2] = fmaf(-u, d.z, v[4 * q + 2]);
    v[4 * q + 3] = fmaf(-u, d.w, v[4 * q + 3]);
  }
}

// Rows [i_lo, i_hi) of D updated with the solved block [r0, r0+rn): row i's
// coefficient of step t is u[i * si + t * st] (rows below the block in the
// forward pass: u = U + r0*ld, si = 1, st = ld; rows above it in the backward
// pass: u = U + r0, si = ld, st = 1).  One function, called (not inlined) at
// the full chunk width by both passes, keeps the substitution's code small:
// with two widths and a copy per pass the step took 1 % longer (instruction
// fetch stalls of two CTAs in different phases), though padding vectors now
// take their FMAs.
template <int W>
__device__ __noinline__ void mx_solve_rows(const float* u, int si, int st, int i_lo, int i_hi,
                                          int r0, int rn, float* D) {
  static_assert(W % 4 == 0, "vectors go in groups of four");
  for (int i = i_lo + threadIdx.x; i < i_hi; i += blockDim.x) {
    const float* up = u + (int64_t)i * si;
    float v[W];
#pragma unroll
    for (int c = 0; c < W; ++c) v[c] = D[i * kMxKc + c];
    if (rn == kMxNB) {
      // a full block: each half's 16 matrix values are loaded before they
      // are used, so their latency is paid twice per block, not per step
      // (a single 32-value batch measured slower: larger code)
#pragma unroll 1
      for (int t0 = 0; t0 < kMxNB; t0 += 16) {
        float uu[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) uu[k] = up[(t0 + k) * st];
#pragma unroll
        for (int k = 0; k < 16; ++k) mx_rows_fma<W>(v, uu[k], D + (r0 + t0 + k) * kMxKc);
      }
    } else {
      for (int t = 0; t < rn; ++t) mx_rows_fma<W>(v, up[t * st], D + (r0 + t) * kMxKc);
    }
#pragma unroll
    for (int c = 0; c < W; ++c) D[i * kMxKc + c] = v[c];
  }
}

template <int NC>
__device__ __noinline__ void mx_solve_t(const float* U, int ld, int n, int nc, float* D,
                                        const float* rd, const MxSmem& sm) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nw = blockDim.x >> 5;
  const int nblk = (n + 31) >> 5;
  for (int bi = 0; bi < nblk; ++bi) {  // forward: Uᵀ y = d
    const int r0 = bi << 5, rn = min(32, n - r0);
    for (int c = warp; c < NC; c += nw) {
      if (sm.done[c]) continue;
      float col[32];
#pragma unroll
      for (int t = 0; t < 32; ++t) col[t] = (t < lane && lane < rn) ? U[(r0 + t) * ld + r0 + lane] : 0.0f;
      const float rdl = (lane < rn) ? rd[r0 + lane] : 0.0f;
      float v = (lane < rn) ? D[(r0 + lane) * kMxKc + c] : 0.0f;
#pragma unroll
      for (int t = 0; t < 32; ++t) {  // lanes >= rn carry zeros, so all 32 steps run
        const float yt = __shfl_sync(0xffffffffu, v * rdl, t);
        v = (lane == t) ? yt : ((lane > t) ? fmaf(-col[t], yt, v) : v);
      }
      if (lane < rn) D[(r0 + lane) * kMxKc + c] = v;
    }
    __syncthreads();
    mx_solve_rows<NC>(U + (int64_t)r0 * ld, 1, ld, r0 + rn, n, r0, rn, D);
    __syncthreads();
  }
  for (int bi = nblk - 1; bi >= 0; --bi) {  // backward: U x = y
    const int r0 = bi << 5, rn = min(32, n - r0);
    for (int c = warp; c < NC; c += nw) {
      if (sm.done[c]) continue;
      float row[32];
#pragma unroll
      for (int t = 0; t < 32; ++t) row[t] = (t > lane && t < rn) ? U[(r0 + lane) * ld + r0 + t] : 0.0f;
      const float rdl = (lane < rn) ? rd[r0 + lane] : 0.0f;
      float v = (lane < rn) ? D[(r0 + lane) * kMxKc + c] : 0.0f;
#pragma unroll
      for (int tt = 31; tt >= 0; --tt) {
        const float xt = __shfl_sync(0xffffffffu, v * rdl, tt);
        v = (lane == tt) ? xt : ((lane < tt) ? fmaf(-row[tt], xt, v) : v);
      }
      if (lane < rn) D[(r0 + lane) * kMxKc + c] = v;
    }
    __syncthreads();
    mx_solve_rows<NC>(U + r0, ld, 1, 0, r0, r0, rn, D);
    __syncthreads();
  }
}

// --- residual: D = fl32(B - A X) with X = hi + lo (float2), FP64-accurate, no FP64 ops
// A is split bitwise into hi+lo, hi*xh products made exact by an FMA
// (TwoProd) and summed with TwoSum; ah*xl + al*xh, the product errors and the
// summation errors go to a second FP32 accumulator.  b - Ax is formed in the
// same double-float arithmetic from the split of b.  Lane c of each warp
// finishes vector c.  Per-warp maxima of |r| and the row sums of |A| (for
// ||A||_inf) land in sm.red / sm.red2.  Vectors nc..NC-1 are padding: b = 0
// and x = 0 there, so their residual is 0.
template <int NC>
__device__ __noinline__ void mx_residual_t(const double* __restrict__ A, int n, int nc,
                              const double* __restrict__ B, const float2* XV, float* D,
                              MxSmem& sm) {
  static_assert(NC == 8, "the transposing reduction below is written for 8 vectors");
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  const int cl = lane >> 2;            // the vector this lane finishes (lanes 4c..4c+3)
  const bool b4 = lane & 16, b3 = lane & 8, b2 = lane & 4;
  float rmax = 0.0f;                   // lane 4c: max |r| of vector c
  float rowmax = 0.0f;
  // The warp walks (row, 256-column chunk) pairs; the loads of the next pair
  // (and b of the next row) are issued before the current chunk is used, so
  // the DRAM latency of A overlaps the arithmetic.
  const int nch = (n + 255) >> 8;
  auto load_chunk = [&](int r, int ch, uint2 (&v)[8]) {
    const uint2* rowp = reinterpret_cast<const uint2*>(A + (int64_t)r * n);
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int j = (ch << 8) + lane + 32 * u;
      v[u] = (r < n && j < n) ? rowp[j] : make_uint2(0u, 0u);
    }
  };
  uint2 av[8];
  load_chunk(warp, 0, av);
  double bnext = (warp < n && cl < nc) ? B[(int64_t)cl * n + warp] : 0.0;
  for (int i = warp; i < n; i += nw) {
    float S[NC], C[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) { S[c] = 0.0f; C[c] = 0.0f; }
    float rs = 0.0f;
    const double bval = bnext;
    for (int ch = 0; ch < nch; ++ch) {
      const int j0 = ch << 8;
      uint2 an[8];
      if (ch + 1 < nch) {
        load_chunk(i, ch + 1, an);
      } else {
        load_chunk(i + nw, 0, an);
        bnext = (i + nw < n && cl < nc) ? B[(int64_t)cl * n + i + nw] : 0.0;
      }
      float ah[8], al[8];
      splitw<8>(av, ah, al);
#pragma unroll
      for (int u = 0; u < 8; ++u) rs += fabsf(ah[u]);   // ah = 0 past the row's end
      // vectors in pairs, a pair only when it holds a live one (the rest
      // are padding); per vector the terms go in j order.  x is read as one
      // 8-byte (hi, lo) pair per element.
#pragma unroll
      for (int h = 0; h < 4; ++h) {
        if (h > 0 && 2 * h >= nc) break;
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int j = j0 + lane + 32 * u;
          if (j < n) {
#pragma unroll
            for (int k = 0; k < 2; ++k) {
              const int c = 2 * h + k;
              const float2 xv = XV[c * n + j];
              const float xh = xv.x, xl = xv.y;
              const float p = ah[u] * xh;
              const float pe = fmaf(ah[u], xh, -p);
              float err;
              two_sum(S[c], p, err);
              C[c] += fmaf(ah[u], xl, fmaf(al[u], xh, pe + err));
            }
          }
        }
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) av[u] = an[u];
    }
    // Transposing butterfly: each exchange halves the vectors a lane keeps
    // (xor 16: 4 of 8, xor 8: 2, xor 4: 1), then two plain steps; lane L ends
    // with the row's sum for vector L >> 2.  Nine double-float additions per
    // lane instead of forty.
    float S4[4], C4[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const float ss = __shfl_xor_sync(0xffffffffu, b4 ? S[k] : S[4 + k], 16);
      const float cs = __shfl_xor_sync(0xffffffffu, b4 ? C[k] : C[4 + k], 16);
      S4[k] = b4 ? S[4 + k] : S[k];
      C4[k] = b4 ? C[4 + k] : C[k];
      float err;
      two_sum(S4[k], ss, err);
      C4[k] += cs + err;
    }
    float S2[2], C2[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const float ss = __shfl_xor_sync(0xffffffffu, b3 ? S4[k] : S4[2 + k], 8);
      const float cs = __shfl_xor_sync(0xffffffffu, b3 ? C4[k] : C4[2 + k], 8);
      S2[k] = b3 ? S4[2 + k] : S4[k];
      C2[k] = b3 ? C4[2 + k] : C4[k];
      float err;
      two_sum(S2[k], ss, err);
      C2[k] += cs + err;
    }
    float S1, C1;
    {
      const float ss = __shfl_xor_sync(0xffffffffu, b2 ? S2[0] : S2[1], 4);
      const float cs = __shfl_xor_sync(0xffffffffu, b2 ? C2[0] : C2[1], 4);
      S1 = b2 ? S2[1] : S2[0];
      C1 = b2 ? C2[1] : C2[0];
      float err;
      two_sum(S1, ss, err);
      C1 += cs + err;
    }
#pragma unroll
    for (int o = 2; o > 0; o >>= 1) {
      const float ss = __shfl_xor_sync(0xffffffffu, S1, o);
      const float cs = __shfl_xor_sync(0xffffffffu, C1, o);
      float err;
      two_sum(S1, ss, err);
      C1 += cs + err;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) rs += __shfl_xor_sync(0xffffffffu, rs, o);
    rowmax = fmaxf(rowmax, rs);
    if ((lane & 3) == 0) {
      float bh, bl;
      split_f64(bval, bh, bl);
      float rh = bh, re;
      two_sum(rh, -S1, re);
      const float r = rh + ((bl - C1) + re);
      D[i * kMxKc + cl] = r;
      rmax = fmaxf(rmax, fabsf(r));
    }
  }
  if ((lane & 3) == 0) sm.red[warp][cl] = rmax;
  if (lane == 0) sm.red2[warp][0] = rowmax;
}

// x += d in double-float (TwoSum then Fast2Sum renormalisation) for live
// vectors; per-warp max |x| into sm.red2[warp][1 + c].
template <int NC>
__device__ __noinline__ void mx_update_x(int n, const float* D, float2* XV, MxSmem& sm) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  float xm[NC];
#pragma unroll
  for (int c = 0; c < NC; ++c) xm[c] = 0.0f;
  for (int i = tid; i < n; i += blockDim.x) {
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      if (!sm.done[c]) {
        const float2 xv = XV[c * n + i];
        float s = xv.x, e;
        two_sum(s, D[i * kMxKc + c], e);
        const float t = xv.y + e;
        const float h = s + t;
        XV[c * n + i] = make_float2(h, t - (h - s));
      }
      xm[c] = fmaxf(xm[c], fabsf(XV[c * n + i].x));
    }
  }
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    float v = xm[c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (lane == 0) sm.red2[warp][1 + c] = v;
  }
}

// One refinement chunk of nc <= NC vectors: solves, x updates and residuals
// until every vector's backward error is <= tol or max_iter solves were
// applied.  Vectors nc..NC-1 are zero padding, marked done from the start;
// a vector's arithmetic does not depend on NC or on the other vectors, so its
// result is the same whichever chunk width solves it.  The kernel instantiates
// one width (kMxKc) for every count: one copy per count overflowed the
// instruction cache when the CTAs of an SM ran systems with different
// right-hand-side counts (ragged 4096-system batch: 11.0 ms with eight
// widths, 8.6 ms with two, 7.7 ms with one).
template <int NC>
__device__ void mx_refine(const float* F, int ld, int n, int nc, const double* __restrict__ A,
                          const double* __restrict__ B, double* __restrict__ X, float* D,
                          float2* XV, double tol, int max_iter, bool& first_residual,
                          int& iters_out, bool& converged, MxSmem& sm) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  if (tid < kMxKc) { sm.done[tid] = tid >= nc; sm.berr[tid] = 0.0; }
  // d = fl32(b), x = 0, ||b||_inf
  float bm[NC];
#pragma unroll
  for (int c = 0; c < NC; ++c) bm[c] = 0.0f;
  for (int i = tid; i < n; i += blockDim.x) {
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      const float v = (c < nc) ? to_f32(B[(int64_t)c * n + i]) : 0.0f;
      D[i * kMxKc + c] = v;
      XV[c * n + i] = make_float2(0.0f, 0.0f);
      bm[c] = fmaxf(bm[c], fabsf(v));
    }
  }
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    float v = bm[c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (lane == 0) sm.red[warp][c] = v;
  }
  __syncthreads();
  if (tid < NC) {
    float m = 0.0f;
    for (int w = 0; w < nw; ++w) m = fmaxf(m, sm.red[w][tid]);
    sm.bnorm[tid] = m;
  }
  __syncthreads();
  int it = 0;
  bool all_done = false;
  for (;;) {
    mx_solve_t<NC>(F, ld, n, nc, D, sm.rd, sm);
    mx_update_x<NC>(n, D, XV, sm);
    ++it;
    __syncthreads();
    mx_residual_t<NC>(A, n, nc, B, XV, D, sm);
    __syncthreads();
    if (tid == 0) {
      if (first_residual) {
        float m = 0.0f;
        for (int w = 0; w < nw; ++w) m = fmaxf(m, sm.red2[w][0]);
        sm.anorm = m;
      }
      int all = 1;
      for (int c = 0; c < NC; ++c) {
        if (!sm.done[c]) {
          float rm = 0.0f, xm = 0.0f;
          for (int w = 0; w < nw; ++w) {
            rm = fmaxf(rm, sm.red[w][c]);
            xm = fmaxf(xm, sm.red2[w][1 + c]);
          }
          const double den = (double)sm.anorm * (double)xm + (double)sm.bnorm[c];
          const double be = (den > 0.0) ? (double)rm / den : (rm > 0.0f ? INFINITY : 0.0);
          sm.berr[c] = be;
          if (be <= tol) sm.done[c] = 1;
        }
        if (!sm.done[c]) all = 0;
      }
      sm.flag = all;
    }
    first_residual = false;
    __syncthreads();
    all_done = sm.flag != 0;
    if (all_done || it >= max_iter) break;
  }
  // x out in FP64
  for (int i = tid; i < n; i += blockDim.x) {
#pragma unroll
    for (int c = 0; c < NC; ++c)
      if (c < nc) {
        const float2 xv = XV[c * n + i];
        X[(int64_t)c * n + i] = (double)xv.x + (double)xv.y;
      }
  }
  iters_out = it;
  converged = all_done;
  __syncthreads();
}

__device__ __forceinline__ int mx_next(int* queue, int* s_next) {
  __syncthreads();
  if (threadIdx.x == 0) *s_next = atomicAdd(queue, 1);
  __syncthreads();
  return *s_next;
}

// Longest-first order for the work queue: a counting sort of the systems by
// n, descending (one CTA; ties in no particular order — a system's result does
// not depend on which CTA solves it).  Systems with n outside [0, kMxMaxN]
// are rejected by the solve and go last.  Also clears the queue counter.
constexpr int kOrderThreads = 1024;
constexpr int kOrderBins = kMxMaxN + 2;

__global__ void __launch_bounds__(kOrderThreads)
order_systems_kernel(int64_t batch, const int32_t* __restrict__ nvec, int32_t* __restrict__ order,
                     int* queue) {
  __shared__ int bins[kOrderBins];
  __shared__ int chunk_sum[32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  auto bin_of = [](int n) { return (n < 0 || n > kMxMaxN) ? kOrderBins - 1 : kMxMaxN - n; };
  for (int i = tid; i < kOrderBins; i += kOrderThreads) bins[i] = 0;
  __syncthreads();
  for (int64_t s = tid; s < batch; s += kOrderThreads) atomicAdd(&bins[bin_of(nvec[s])], 1);
  __syncthreads();
  // exclusive scan of the bins: warp 0, each lane a contiguous chunk
  constexpr int kChunk = (kOrderBins + 31) / 32;
  if (warp == 0) {
    const int lo = lane * kChunk, hi = min(lo + kChunk, kOrderBins);
    int sum = 0;
    for (int i = lo; i < hi; ++i) sum += bins[i];
    int incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    chunk_sum[lane] = incl - sum;
    __syncwarp();
    int run = chunk_sum[lane];
    for (int i = lo; i < hi; ++i) { const int c = bins[i]; bins[i] = run; run += c; }
  }
  __syncthreads();
  for (int64_t s = tid; s < batch; s += kOrderThreads)
    order[atomicAdd(&bins[bin_of(nvec[s])], 1)] = (int32_t)s;
  if (tid == 0) *queue = 0;
}

// Per-system factor handling of the mixed solve (fmode[s]).
constexpr int kFactorCompute = 0;  // factor A, keep nothing
constexpr int kFactorStore = 1;    // factor A and store the FP32 factor at fptr[s]
constexpr int kFactorLoad = 2;     // use the factor stored at fptr[s]; A is not factored

__global__ void __launch_bounds__(kMxThreads, 2)
posv_mixed_kernel(int64_t batch, int max_n, int max_nrhs, const int32_t* __restrict__ nvec,
                  const int32_t* __restrict__ nrhs_vec, const int64_t* __restrict__ a_off,
                  const double* __restrict__ a, const int64_t* __restrict__ b_off,
                  const double* __restrict__ b, double* __restrict__ x, double tol, int max_iter,
                  int32_t* __restrict__ info, int32_t* __restrict__ iters,
                  double* __restrict__ berr_out, int* queue, const int32_t* __restrict__ order,
                  float* __restrict__ factor_ws, int small_max, const int32_t* __restrict__ fmode,
                  float* const* __restrict__ fptr, int use_tc) {
  extern __shared__ float smem_mx[];
  __shared__ MxSmem sm;
  const int tid = threadIdx.x;
  unsigned tc_phase = 0;
  if (use_tc) {
    // 128 TMEM columns for the trailing-update accumulator (two CTAs per SM
    // hold 256 of the 512)
    if (tid == 0) {
      mbar_init(&sm.tcbar, 1);
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if ((tid >> 5) == 0) {
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 128;" ::"r"(
                       smem_u32(&sm.tmem))
                   : "memory");
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  } else if ((tid >> 5) == 0) {
    // A CTA of a kernel that can allocate tensor memory holds the SM's
    // allocation permit until it gives it up; keeping it would hold the SM to
    // one CTA of this kernel (measured: 7.5 -> 11.8 ms on the 4096-system
    // batch), so a CTA that will not allocate gives it up at once.
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  for (;;) {
    const int k = mx_next(queue, &sm.next);
    if (k >= batch) break;
    const int s = order ? order[k] : k;
    const int n = nvec[s];
    const int nrhs = nrhs_vec[s];
    if (n > max_n || n < 0 || nrhs > max_nrhs || nrhs < 0) {
      if (tid == 0) { info[s] = -2; iters[s] = 0; berr_out[s] = NAN; }
      continue;
    }
    if (n == 0) {
      if (tid == 0) { info[s] = 0; iters[s] = 0; berr_out[s] = 0.0; }
      continue;
    }
    const double* A = a + a_off[s];
    const bool small = n <= small_max;
    const int ld = small ? (n | 1) : ((n + 31) & ~31);
    const int ldmax = (max_n + 31) & ~31;
    float* F = small ? smem_mx : factor_ws + (int64_t)blockIdx.x * ldmax * ldmax;
    // D (n rows of kMxKc floats) | x as (hi, lo) pairs (kMxKc*n float2),
    // 16-byte aligned
    float* vec = small ? smem_mx + ((n * ld + 3) & ~3) : smem_mx;
    float* D = vec;
    float2* XV = reinterpret_cast<float2*>(vec + kMxKc * n);
    if (tid == 0) sm.flag = 0;
    const int fm = fmode ? fmode[s] : kFactorCompute;
    int rc;
    if (fm == kFactorLoad) {
      // A factor kept from an earlier call: the upper triangle as stored, and
      // 1/diag formed exactly as the factorisation forms it (1.0f / d).
      const float* src = fptr[s];
      __syncthreads();
      for (int e = tid; e < n * n; e += blockDim.x) {
        const int i = e / n, j = e - i * n;
        if (j >= i) F[(int64_t)i * ld + j] = src[e];
      }
      __syncthreads();
      for (int i = tid; i < n; i += blockDim.x) sm.rd[i] = 1.0f / F[(int64_t)i * ld + i];
      rc = 0;
    } else if (small) {
      mx_copy_upper(A, n, F, ld);
      __syncthreads();
      rc = mx_factor_small(F, ld, n, sm);
    } else {
      __syncthreads();
      rc = mx_factor_large(A, F, n, ld, sm, *reinterpret_cast<MxStage*>(smem_mx), use_tc != 0,
                           tc_phase);
    }
    __syncthreads();
    if (rc == 0 && fm == kFactorStore) {
      // keep the factor for later calls (upper triangle, lower zeroed)
      float* dst = fptr[s];
      for (int e = tid; e < n * n; e += blockDim.x) {
        const int i = e / n, j = e - i * n;
        dst[e] = (j >= i) ? F[(int64_t)i * ld + j] : 0.0f;
      }
    }
    if (rc != 0) {
      for (int e = tid; e < n * nrhs; e += blockDim.x) x[b_off[s] + e] = NAN;
      if (tid == 0) { info[s] = rc; iters[s] = 0; berr_out[s] = NAN; }
      continue;
    }
    double sys_berr = 0.0;
    int sys_iters = 0, sys_info = 0;
    bool first = true;
    for (int c0 = 0; c0 < nrhs; c0 += kMxKc) {
      const int nc = min(kMxKc, nrhs - c0);
      const double* B = b + b_off[s] + (int64_t)c0 * n;
      double* X = x + b_off[s] + (int64_t)c0 * n;
      int it = 0;
      bool conv = true;
      mx_refine<kMxKc>(F, ld, n, nc, A, B, X, D, XV, tol, max_iter, first, it, conv, sm);
      if (!conv) sys_info = -1;
      for (int c = 0; c < nc; ++c) sys_berr = fmax(sys_berr, sm.berr[c]);
      sys_iters = max(sys_iters, it);
      __syncthreads();
      if (tid == 0) sm.flag = 0;
    }
    if (tid == 0) { info[s] = sys_info; iters[s] = sys_iters; berr_out[s] = sys_berr; }
  }
  if (use_tc) {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if ((tid >> 5) == 0)
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 128;" ::"r"(sm.tmem)
                   : "memory");
  }
}

__global__ void reset_queue_kernel(int* queue) { *queue = 0; }

// Tuning table of the mixed solve: the largest order factored in shared
// memory (larger systems take the L2-slice path).  Set from the host's
// autotune table at initialisation (lxgb_posv_mixed_set_small_max); each call
// reads it once, and workspace sizes follow it.
static std::atomic<int> g_mx_small_max{kMxSmallN};
// Trailing updates of the large-system factor on the tensor cores (1) or on
// the CUDA cores (0); a tuning switch like small_max, fixed at start-up.
static std::atomic<int> g_mx_tc{0};

static size_t mixed_smem_bytes(int max_n, int max_nrhs, int small_max) {
  (void)max_nrhs;
  const int ns = max_n < small_max ? max_n : small_max;
  // + three floats: the vectors start on a 16-byte boundary after the factor
  const size_t small =
      (size_t)(ns * (ns | 1) + 3) * sizeof(float) + (size_t)3 * kMxKc * ns * sizeof(float);
  size_t large = (size_t)3 * kMxKc * max_n * sizeof(float);
  // the staged block row (or the tensor-core bands, aligned to 1024 bytes)
  if (max_n > small_max && large < sizeof(MxStage) + 1024) large = sizeof(MxStage) + 1024;
  return small > large ? small : large;
}

// Workspace: queue header, the longest-first order (batch int32, rounded up
// to 256 bytes), then one FP32 max_n² factor slice per CTA when some system
// can exceed the shared-memory size.
static int64_t mixed_order_bytes(int64_t batch) { return (batch * 4 + 255) & ~(int64_t)255; }

static int64_t mixed_slice_bytes(int max_n, int small_max) {
  const int64_t ld = (max_n + 31) & ~31;
  return (max_n > small_max) ? ld * ld * (int64_t)sizeof(float) : 0;
}

static int mixed_grid(int64_t batch) {
  const int64_t g = 2LL * sm_count();
  return (int)((batch < g) ? batch : g);
}

// Launch over `grid` CTAs with the given scratch (queue [+ order] + factor
// slices).  Without the order (ordered == false) systems go in index order.
static int mixed_launch(int grid, int64_t batch, int32_t max_n, int32_t max_nrhs, const int32_t* n,
                        const int32_t* nrhs, const int64_t* a_off, const double* a,
                        const int64_t* b_off, const double* b, double* x, double tol,
                        int32_t max_iter, int32_t* info, int32_t* iters, double* berr,
                        void* scratch, bool ordered, int small_max, cudaStream_t st,
                        const int32_t* fmode = nullptr, float* const* fptr = nullptr) {
  char* base = reinterpret_cast<char*>(scratch);
  int* queue = reinterpret_cast<int*>(base);
  int32_t* order = ordered ? reinterpret_cast<int32_t*>(base + kQueueHeader) : nullptr;
  float* factor_ws = reinterpret_cast<float*>(
      base + kQueueHeader + (ordered ? mixed_order_bytes(batch) : 0));
  if (ordered)
    order_systems_kernel<<<1, kOrderThreads, 0, st>>>(batch, n, order, queue);
  else
    reset_queue_kernel<<<1, 1, 0, st>>>(queue);
  const size_t smem = mixed_smem_bytes(max_n, max_nrhs, small_max);
  LXGB_CUDA_TRY(ensure_dynamic_smem(reinterpret_cast<const void*>(posv_mixed_kernel), (int)smem),
                "posv_mixed: set smem");
  posv_mixed_kernel<<<(unsigned)grid, kMxThreads, smem, st>>>(
      batch, max_n, max_nrhs, n, nrhs, a_off, a, b_off, b, x, tol, max_iter, info, iters, berr,
      queue, order, factor_ws, small_max, fmode, fptr,
      (g_mx_tc.load() && max_n > small_max) ? 1 : 0);
  return check_launch("posv_mixed");
}

}  // namespace lxgb

using namespace lxgb;

extern "C" int lxgb_potrf_ragged_f64(int64_t batch, int32_t max_n, const int32_t* n,
                                     const int64_t* a_off, double* a, int32_t* info,
                                     void* stream) {
  LXGB_REQUIRE(batch >= 0 && max_n >= 0, "potrf: negative size");
  if (batch == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(n && a_off && a && info, "potrf: null pointer");
  LXGB_REQUIRE(batch < (1LL << 31), "potrf: batch too large");
  cudaStream_t st = as_stream(stream);
  const int ns = max_n < kCholSmemMaxF64 ? max_n : kCholSmemMaxF64;
  const size_t smem = (size_t)ns * (ns | 1) * sizeof(double);
  LXGB_CUDA_TRY(ensure_dynamic_smem(reinterpret_cast<const void*>(potrf_ragged_f64_kernel), (int)smem),
                "potrf: set smem");
  const int64_t g = sm_count();
  potrf_ragged_f64_kernel<<<(unsigned)(batch < g ? batch : g), kCholThreads, smem, st>>>(
      batch, max_n, n, a_off, a, info);
  return check_launch("potrf ragged");
}

extern "C" int lxgb_potrs_ragged_f64(int64_t batch, int32_t max_n, const int32_t* n,
                                     const int32_t* nrhs, const int64_t* a_off, const double* u,
                                     const int64_t* b_off, double* b, void* stream) {
  LXGB_REQUIRE(batch >= 0 && max_n >= 0, "potrs: negative size");
  if (batch == 0 || max_n == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(n && nrhs && a_off && u && b_off && b, "potrs: null pointer");
  const size_t smem = (size_t)max_n * sizeof(double);
  LXGB_REQUIRE(smem <= 160 * 1024, "potrs: max_n too large for the shared-memory vector");
  LXGB_CUDA_TRY(ensure_dynamic_smem(reinterpret_cast<const void*>(potrs_ragged_f64_kernel), (int)smem),
                "potrs: set smem");
  const int64_t g = 4 * (int64_t)sm_count();
  potrs_ragged_f64_kernel<<<(unsigned)(batch < g ? batch : g), kCholThreads, smem,
                            as_stream(stream)>>>(batch, max_n, n, nrhs, a_off, u, b_off, b);
  return check_launch("potrs ragged");
}

static int64_t mixed_workspace_bytes(int64_t batch, int32_t max_n, int small_max) {
  if (batch <= 0 || max_n <= 0) return kQueueHeader;
  return kQueueHeader + mixed_order_bytes(batch) +
         (int64_t)mixed_grid(batch) * mixed_slice_bytes(max_n, small_max);
}

extern "C" int64_t lxgb_posv_ragged_mixed_workspace_size(int64_t batch, int32_t max_n,
                                                         int32_t max_nrhs) {
  (void)max_nrhs;
  return mixed_workspace_bytes(batch, max_n, g_mx_small_max.load());
}

extern "C" int lxgb_posv_mixed_set_small_max(int32_t small_max) {
  LXGB_REQUIRE(small_max >= 0 && small_max <= kMxSmallN,
               "posv_mixed: small_max must be in [0, 144]");
  g_mx_small_max.store(small_max);
  return LXGB_SUCCESSFUL;
}

extern "C" int32_t lxgb_posv_mixed_small_max(void) { return g_mx_small_max.load(); }

extern "C" int lxgb_posv_mixed_set_tensor_cores(int32_t on) {
  LXGB_REQUIRE(on == 0 || on == 1, "posv_mixed: tensor-core switch must be 0 or 1");
  g_mx_tc.store(on);
  return LXGB_SUCCESSFUL;
}

extern "C" int lxgb_posv_ragged_mixed(int64_t batch, int32_t max_n, int32_t max_nrhs,
                                      const int32_t* n, const int32_t* nrhs, const int64_t* a_off,
                                      const double* a, const int64_t* b_off, const double* b,
                                      double* x, double tol, int32_t max_iter, int32_t* info,
                                      int32_t* iters, double* berr, void* work,
                                      int64_t work_bytes, void* stream) {
  LXGB_REQUIRE(batch >= 0 && max_n >= 0 && max_nrhs >= 0, "posv_mixed: negative size");
  if (batch == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(batch < (1LL << 31), "posv_mixed: batch too large");
  LXGB_REQUIRE(n && nrhs && a_off && a && b_off && b && x && info && iters && berr && work,
               "posv_mixed: null pointer");
  LXGB_REQUIRE(max_iter >= 1, "posv_mixed: max_iter must be >= 1");
  LXGB_REQUIRE(max_n <= kMxMaxN, "posv_mixed: max_n above 1024");
  LXGB_REQUIRE(((uintptr_t)work & 255) == 0, "posv_mixed: workspace must be 256-byte aligned");
  const int small_max = g_mx_small_max.load();
  if (work_bytes < mixed_workspace_bytes(batch, max_n, small_max)) {
    set_last_error("posv_mixed: workspace too small");
    return LXGB_WORKSPACE_TOO_SMALL;
  }
  return mixed_launch(mixed_grid(batch), batch, max_n, max_nrhs, n, nrhs, a_off, a, b_off, b, x,
                      tol, max_iter, info, iters, berr, work, true, small_max,
                      as_stream(stream));
}

extern "C" int lxgb_posv_ragged_mixed_factors(
    int64_t batch, int32_t max_n, int32_t max_nrhs, const int32_t* n, const int32_t* nrhs,
    const int64_t* a_off, const double* a, const int64_t* b_off, const double* b, double* x,
    double tol, int32_t max_iter, int32_t* info, int32_t* iters, double* berr,
    const int32_t* fmode, float* const* factors, void* work, int64_t work_bytes, void* stream) {
  LXGB_REQUIRE(batch >= 0 && max_n >= 0 && max_nrhs >= 0, "posv_mixed_factors: negative size");
  if (batch == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(batch < (1LL << 31), "posv_mixed_factors: batch too large");
  LXGB_REQUIRE(n && nrhs && a_off && a && b_off && b && x && info && iters && berr && work &&
                   fmode && factors,
               "posv_mixed_factors: null pointer");
  LXGB_REQUIRE(max_iter >= 1, "posv_mixed_factors: max_iter must be >= 1");
  LXGB_REQUIRE(max_n <= kMxMaxN, "posv_mixed_factors: max_n above 1024");
  LXGB_REQUIRE(((uintptr_t)work & 255) == 0,
               "posv_mixed_factors: workspace must be 256-byte aligned");
  const int small_max = g_mx_small_max.load();
  if (work_bytes < mixed_workspace_bytes(batch, max_n, small_max)) {
    set_last_error("posv_mixed_factors: workspace too small");
    return LXGB_WORKSPACE_TOO_SMALL;
  }
  return mixed_launch(mixed_grid(batch), batch, max_n, max_nrhs, n, nrhs, a_off, a, b_off, b, x,
                      tol, max_iter, info, iters, berr, work, true, small_max,
                      as_stream(stream), fmode, factors);
}

// ---------------------------------------------------------------------------
// Allocation-free variant of lxgb_posv_ragged_mixed.
//
// Some callers cannot allocate device memory at the moment they need a solve:
// an XLA/JAX FFI handler owns no allocator of its own (device memory belongs to
// XLA, and a cudaMalloc inside the handler can synchronise the device or break
// a CUDA-graph capture XLA is recording), and a serving loop or real-time
// controller may forbid allocation once it has started.  For them the scratch
// of the mixed solve (work-queue counter + FP32 factors of systems too large for
// shared memory) lives in the fixed array below, which every GPU that loads this
// library holds until the process exits.
// ---------------------------------------------------------------------------
#include <mutex>

namespace lxgb {

static __device__ __align__(256) unsigned char g_posv_noalloc_scratch[LXGB_POSV_NOALLOC_SCRATCH_BYTES];

constexpr int kNoallocMaxDevices = 64;
static void* g_noalloc_addr[kNoallocMaxDevices] = {nullptr};
static std::mutex g_noalloc_mu;

// Device address of the scratch array on the current device, looked up once
// per device (the host-side symbol is not a device address).
static int noalloc_scratch_address(void** out) {
  int dev = -1;
  LXGB_CUDA_TRY(cudaGetDevice(&dev), "posv_mixed_noalloc: cudaGetDevice");
  if (dev < 0 || dev >= kNoallocMaxDevices) {
    set_last_error("posv_mixed_noalloc: device ordinal %d out of range", dev);
    return LXGB_INVALID_ARG;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (g_noalloc_addr[dev] == nullptr) {
    void* p = nullptr;
    LXGB_CUDA_TRY(cudaGetSymbolAddress(&p, g_posv_noalloc_scratch),
                  "posv_mixed_noalloc: cudaGetSymbolAddress");
    g_noalloc_addr[dev] = p;
  }
  *out = g_noalloc_addr[dev];
  return LXGB_SUCCESSFUL;
}

}  // namespace lxgb

extern "C" int lxgb_posv_ragged_mixed_noalloc(int64_t batch, int32_t max_n, int32_t max_nrhs,
                                              const int32_t* n, const int32_t* nrhs,
                                              const int64_t* a_off, const double* a,
                                              const int64_t* b_off, const double* b, double* x,
                                              double tol, int32_t max_iter, int32_t* info,
                                              int32_t* iters, double* berr, void* stream) {
  LXGB_REQUIRE(batch >= 0 && max_n >= 0 && max_nrhs >= 0, "posv_mixed_noalloc: negative size");
  if (batch == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(batch < (1LL << 31), "posv_mixed_noalloc: batch too large");
  LXGB_REQUIRE(n && nrhs && a_off && a && b_off && b && x && info && iters && berr,
               "posv_mixed_noalloc: null pointer");
  LXGB_REQUIRE(max_iter >= 1, "posv_mixed_noalloc: max_iter must be >= 1");
  LXGB_REQUIRE(max_n <= kMxMaxN,
               "posv_mixed_noalloc: max_n above 1024");
  // Grid: one FP32 factor slice per CTA for systems above the shared-memory
  // size, as many slices as the fixed scratch holds.  The longest-first order
  // goes in what the slices leave over; without room for it systems go in
  // index order.
  int64_t grid = mixed_grid(batch);
  const int small_max = g_mx_small_max.load();
  const int64_t slice = mixed_slice_bytes(max_n, small_max);
  const int64_t room = (int64_t)LXGB_POSV_NOALLOC_SCRATCH_BYTES - kQueueHeader;
  if (slice > 0) {
    const int64_t slices = room / slice;
    if (slices < 1) {
      set_last_error("posv_mixed_noalloc: max_n=%d needs %lld bytes of scratch, limit %lld", max_n,
                     (long long)(slice + kQueueHeader),
                     (long long)LXGB_POSV_NOALLOC_SCRATCH_BYTES);
      return LXGB_INVALID_ARG;
    }
    if (slices < grid) grid = slices;
  }
  const bool ordered = mixed_order_bytes(batch) + grid * slice <= room;
  void* scratch = nullptr;
  int rc = noalloc_scratch_address(&scratch);
  if (rc) return rc;
  // mixed_launch clears the work-queue counter, which the array keeps from the
  // previous call.
  return mixed_launch((int)grid, batch, max_n, max_nrhs, n, nrhs, a_off, a, b_off, b, x, tol,
                      max_iter, info, iters, berr, scratch, ordered, small_max,
                      as_stream(stream));
}
