// Householder QR (geqrf) and application of Q / Qᵀ (ormqr), FP64.
//
// Storage: the factor is kept in the "raw" layout JAX's jnp.linalg.qr(mode=
// "raw") returns, h = Mᵀ (nn rows of length mm) for a tall mm×nn matrix M, so
// every column of M — every Householder vector — is a contiguous row of h.
// On return h[k][k..] holds R's k-th column on and above the diagonal (R[i][k] =
// h[k][i], i <= k) and the k-th reflector below it (v_k[i] = h[k][i], i > k,
// v_k[k] = 1), tau[k] its scalar: H_k = I - tau_k v_k v_kᵀ, Q = H_0 H_1 ...
//
// Blocked right-looking with compact-WY panels of kQrNB reflectors
// (H_j0 ... H_{j0+nb-1} = I - V T Vᵀ, T upper triangular):
//   qr_panel_cluster_kernel — the reflectors of one panel and its T, rows
//                       split over a thread-block cluster (up to 16 CTAs)
//                       whose reductions meet in distributed shared memory;
//   qr_panel_kernel / qr_larft_kernel — the same on one CTA (fallback when a
//                       cluster cannot be scheduled)
//   qr_w_kernel       — W = Vᵀ C for the trailing columns C (split over rows)
//   qr_wt_kernel      — W' = Tᵀ W (summing the splits in fixed order)
//   qr_update_kernel  — C -= V W'  (64×64 tiles, K = nb)
// T of every panel is kept so that ormqr applies whole panels at once.
#include <cooperative_groups.h>
#include <math.h>

#include <map>
#include <type_traits>
#include <mutex>
#include <utility>

#include "common.cuh"
#include "tc_gemm.cuh"

namespace lxgb {

constexpr int kQrNB = 32;
constexpr int kQrPanelThreads = 512;

// v_p[i] for panel row p (global row r = j0 + p) read from h.
template <typename T>
__device__ __forceinline__ T refl(const T* h, int64_t mm, int r, int64_t i) {
  return (i < r) ? T(0) : (i == r ? T(1) : h[(int64_t)r * mm + i]);
}

__device__ double block_sum(double v, double* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double t = 0.0;
  for (int w = 0; w < nw; ++w) t += red[w];
  return t;
}

// Reflectors of panel rows [j0, pe) of h (mm columns).
__global__ void __launch_bounds__(kQrPanelThreads)
qr_panel_kernel(int64_t mm, int nn, int j0, int pe, double* __restrict__ h,
                double* __restrict__ tau) {
  __shared__ double red[32];
  __shared__ double wred[kQrPanelThreads / 32][kQrNB];
  __shared__ double s_tau, s_scal;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nw = blockDim.x >> 5;
  for (int k = j0; k < pe; ++k) {
    double* hk = h + (int64_t)k * mm;
    double ss = 0.0;
    for (int64_t i = k + 1 + tid; i < mm; i += blockDim.x) ss = fma(hk[i], hk[i], ss);
    const double xnorm2 = block_sum(ss, red);
    if (tid == 0) {
      const double alpha = hk[k];
      const double xnorm = sqrt(xnorm2);
      if (xnorm == 0.0) {
        s_tau = 0.0;
        s_scal = 1.0;
      } else {
        const double beta = -copysign(hypot(alpha, xnorm), alpha);
        s_tau = (beta - alpha) / beta;
        s_scal = 1.0 / (alpha - beta);
        hk[k] = beta;
      }
      tau[k] = s_tau;
    }
    __syncthreads();
    const double tk = s_tau;
    if (tk != 0.0) {
      const double sc = s_scal;
      for (int64_t i = k + 1 + tid; i < mm; i += blockDim.x) hk[i] *= sc;
    }
    __syncthreads();
    const int nrem = pe - k - 1;
    if (tk != 0.0 && nrem > 0) {
      double acc[kQrNB];
#pragma unroll
      for (int q = 0; q < kQrNB; ++q) acc[q] = 0.0;
      for (int64_t i = k + 1 + tid; i < mm; i += blockDim.x) {
        const double vi = hk[i];
#pragma unroll
        for (int q = 0; q < kQrNB; ++q)
          if (q < nrem) acc[q] = fma(vi, h[(int64_t)(k + 1 + q) * mm + i], acc[q]);
      }
#pragma unroll
      for (int q = 0; q < kQrNB; ++q) {
        if (q < nrem) {
          const double s = warp_sum(acc[q]);
          if (lane == 0) wred[warp][q] = s;
        }
      }
      __syncthreads();
      // w_j = h[j][k] + sum_{i>k} v_i h[j][i]; then h[j][i] -= tau w_j v_i, i >= k.
      for (int q = warp; q < nrem; q += nw) {
        double w = 0.0;
        for (int ww = 0; ww < nw; ++ww) w += wred[ww][q];
        double* hj = h + (int64_t)(k + 1 + q) * mm;
        w += hj[k];
        const double tw = tk * w;
        if (lane == 0) hj[k] -= tw;
        for (int64_t i = k + 1 + lane; i < mm; i += 32) hj[i] = fma(-tw, hk[i], hj[i]);
      }
    }
    __syncthreads();
  }
}

namespace cg = cooperative_groups;
constexpr int kQrCluThreads = 512;
constexpr int kQrCluMax = 16;

// Block-wide sums of NV values per thread, written to out[0..NV) (thread 0's
// view is complete after the trailing barrier).  red: [warps][NV].
template <int NV, typename T>
__device__ void block_sums(T (&v)[NV], T (*red)[kQrNB], T* out) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    const T s = warp_sum(v[q]);
    if (lane == 0) red[warp][q] = s;
  }
  __syncthreads();
  for (int q = threadIdx.x; q < NV; q += blockDim.x) {
    T t = T(0);
    for (int w = 0; w < nw; ++w) t += red[w][q];
    out[q] = t;
  }
  __syncthreads();
}

// Reflectors of panel rows [j0, pe) of h and the panel's T, with the
// reflector rows i in [j0, mm) split over the cluster's CTAs (rows_per_cta
// each).  Per column k: partial sums of squares -> barrier -> every CTA forms
// the same beta/tau/scale from the partials summed in rank order (alpha comes
// from the owner of row k's shared memory, since the owner overwrites it) ->
// scale the CTA's part of v_k and form partial dots v_kᵀ a_q, the owner of row
// k adding a_q[k] (v_k[k] = 1) -> barrier -> update a_q -= tau w_q v_k.
// Partials are double-buffered by column parity: two barriers per column.
// Then G = VᵀV from per-CTA partials and T by larft's recurrence in CTA 0.
// Same rules as qr_panel_kernel + qr_larft_kernel (LAPACK geqr2/larfg/larft).
// SM: the CTA's rows of the panel are staged in dynamic shared memory for the
// whole panel (32 × rows_per_cta values; the FP32 factor's slices fit) instead
// of being streamed from L2 column by column.
template <typename T, bool SM>
__global__ void __launch_bounds__(kQrCluThreads, 1)
qr_panel_cluster_kernel(int64_t mm, int j0, int pe, int64_t rows_per_cta,
                        T* __restrict__ h, T* __restrict__ tau, T* __restrict__ t_out) {
  extern __shared__ __align__(16) unsigned char qr_dyn[];
  __shared__ T red[kQrCluThreads / 32][kQrNB];
  __shared__ T p_ss[2], p_alpha[2];
  __shared__ T p_w[2][kQrNB];
  __shared__ T G[kQrNB][kQrNB + 1];
  __shared__ T Tm[kQrNB][kQrNB + 1];
  __shared__ T s_tau, s_scal;
  cg::cluster_group cluster = cg::this_cluster();
  const int ncta = (int)cluster.num_blocks();
  const int rank = (int)cluster.block_rank();
  const int tid = threadIdx.x;
  const int nb = pe - j0;
  const int64_t r_lo = j0 + (int64_t)rank * rows_per_cta;
  const int64_t r_hi = min(mm, r_lo + rows_per_cta);
  T* S = reinterpret_cast<T*>(qr_dyn);
  // element i (a global row, r_lo <= i < r_hi) of panel column q
  auto at = [&](int q, int64_t i) -> T& {
    return SM ? S[(int64_t)q * rows_per_cta + (i - r_lo)] : h[(int64_t)(j0 + q) * mm + i];
  };
  if (SM) {
    for (int q = 0; q < nb; ++q)
      for (int64_t i = r_lo + tid; i < r_hi; i += blockDim.x) at(q, i) = h[(int64_t)(j0 + q) * mm + i];
    __syncthreads();
  }
  for (int k = j0; k < pe; ++k) {
    const int par = (k - j0) & 1;
    const int kk = k - j0;
    const bool own_k = (k >= r_lo && k < r_hi);
    T ss[1] = {T(0)};
    for (int64_t i = max((int64_t)k + 1, r_lo) + tid; i < r_hi; i += blockDim.x)
      ss[0] = fma(at(kk, i), at(kk, i), ss[0]);
    block_sums<1>(ss, red, &p_ss[par]);
    if (tid == 0 && own_k) p_alpha[par] = at(kk, k);
    cluster.sync();
    if (tid < 32) {
      // lane c reads CTA c's partial (parallel remote loads), fixed-order tree
      T xnorm2 = (tid < ncta) ? *cluster.map_shared_rank(&p_ss[par], tid) : T(0);
      xnorm2 = warp_sum(xnorm2);
      const int own = (int)((k - j0) / rows_per_cta);
      const T alpha = *cluster.map_shared_rank(&p_alpha[par], own);
      if (tid == 0) {
        const T xnorm = sqrt(xnorm2);
        if (xnorm == T(0)) {
          s_tau = T(0);
          s_scal = T(1);
        } else {
          const T beta = -copysign(hypot(alpha, xnorm), alpha);
          s_tau = (beta - alpha) / beta;
          s_scal = T(1) / (alpha - beta);
          if (own_k) at(kk, k) = beta;
        }
        if (rank == 0) tau[k] = s_tau;
      }
    }
    __syncthreads();
    const T tk = s_tau;
    const int nrem = pe - k - 1;
    const int lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
    const int64_t i_lo = max((int64_t)k + 1, r_lo);
    if (tk != T(0)) {
      const T sc = s_scal;
      for (int64_t i = i_lo + tid; i < r_hi; i += blockDim.x) at(kk, i) *= sc;
    }
    __syncthreads();
    // one warp per trailing column: w_q partial = v_kᵀ a_q over this CTA's
    // rows (+ a_q[k] from the owner of row k, as v_k[k] = 1)
    for (int q = warp; q < nrem; q += nwarps) {
      T acc = T(0);
      const int qq = kk + 1 + q;
      if (tk != T(0)) {
        // eight independent loads in flight per lane when the rows sit in L2
        int64_t i = i_lo + lane;
        T a8[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) a8[u] = T(0);
        for (; i + 7 * 32 < r_hi; i += 8 * 32) {
          T vv[8], qv[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) { vv[u] = at(kk, i + 32 * u); qv[u] = at(qq, i + 32 * u); }
#pragma unroll
          for (int u = 0; u < 8; ++u) a8[u] = fma(vv[u], qv[u], a8[u]);
        }
        for (; i < r_hi; i += 32) a8[0] = fma(at(kk, i), at(qq, i), a8[0]);
#pragma unroll
        for (int u = 0; u < 8; ++u) acc += a8[u];
        acc = warp_sum(acc);
        if (own_k && lane == 0) acc += at(qq, k);
      }
      if (lane == 0) p_w[par][q] = acc;
    }
    cluster.sync();
    if (tk != T(0) && nrem > 0) {
      for (int q = warp; q < nrem; q += nwarps) {
        T w = (lane < ncta) ? cluster.map_shared_rank(&p_w[par][0], lane)[q] : T(0);
        w = warp_sum(w);
        const T tw = tk * w;
        const int qq = kk + 1 + q;
        if (own_k && lane == 0) at(qq, k) -= tw;
        int64_t i = i_lo + lane;
        for (; i + 7 * 32 < r_hi; i += 8 * 32) {
          T vv[8], qv[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) { vv[u] = at(kk, i + 32 * u); qv[u] = at(qq, i + 32 * u); }
#pragma unroll
          for (int u = 0; u < 8; ++u) at(qq, i + 32 * u) = fma(-tw, vv[u], qv[u]);
        }
        for (; i < r_hi; i += 32) at(qq, i) = fma(-tw, at(kk, i), at(qq, i));
      }
    }
    __syncthreads();
  }
  // G[q][p] = v_qᵀ v_p (q < p) over this CTA's rows, then summed in CTA 0.
  // Rows are staged through shared memory 64 at a time (coalesced loads);
  // thread t accumulates pair t of the strictly upper triangle.
  {
    __shared__ T Vc[64][kQrNB + 1];
    int pq = -1, pp = -1;
    for (int p2 = 1, t = 0; p2 < nb && pq < 0; ++p2) {
      if (tid < t + p2) { pq = tid - t; pp = p2; }
      t += p2;
    }
    T acc = T(0);
    for (int64_t i0 = r_lo; i0 < r_hi; i0 += 64) {
      for (int e = tid; e < 64 * kQrNB; e += blockDim.x) {
        const int q = e / 64, ii = e % 64;
        const int64_t i = i0 + ii;
        Vc[ii][q] = (q < nb && i < r_hi)
                        ? ((i < j0 + q) ? T(0) : (i == j0 + q ? T(1) : at(q, i)))
                        : T(0);
      }
      __syncthreads();
      if (pq >= 0) {
#pragma unroll 8
        for (int ii = 0; ii < 64; ++ii) acc = fma(Vc[ii][pq], Vc[ii][pp], acc);
      }
      __syncthreads();
    }
    if (pq >= 0) G[pq][pp] = acc;
  }
  cluster.sync();
  if (rank == 0) {
    __shared__ T Gs[kQrNB][kQrNB + 1];
    for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
      const int q = e / nb, pp = e % nb;
      T g = T(0);
      if (q < pp)
        for (int c = 0; c < ncta; ++c) g += cluster.map_shared_rank(&G[0][0], c)[q * (kQrNB + 1) + pp];
      Gs[q][pp] = g;
    }
    for (int e = threadIdx.x; e < kQrNB * kQrNB; e += blockDim.x) Tm[e / kQrNB][e % kQrNB] = T(0);
    __syncthreads();
    if ((threadIdx.x >> 5) == 0) {
      const int lane = threadIdx.x & 31;
      for (int k = 0; k < nb; ++k) {
        const T tk = tau[j0 + k];
        T v = T(0);
        if (lane < k) {
          for (int q = lane; q < k; ++q) v = fma(Tm[lane][q], Gs[q][k], v);
          v = -tk * v;
        }
        __syncwarp();
        if (lane < k) Tm[lane][k] = v;
        if (lane == k) Tm[k][k] = tk;
        __syncwarp();
      }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < kQrNB * kQrNB; e += blockDim.x)
      t_out[e] = Tm[e / kQrNB][e % kQrNB];
  }
  if (SM) {
    for (int q = 0; q < nb; ++q)
      for (int64_t i = r_lo + tid; i < r_hi; i += blockDim.x) h[(int64_t)(j0 + q) * mm + i] = at(q, i);
  }
  cluster.sync();  // CTA 0 has finished reading the others' shared memory
}

// FP32 panel with one cluster barrier per column (the panel of the
// mixed-precision QR).  The norm of column k below the diagonal and the dots
// d_q = a_kᵀ a_q of every trailing column q come out of one pass and one
// cluster-wide reduction; with scal = 1 / (alpha - beta), the reflector's
// dots are w_q = a_q[k] + scal d_q and the update is a_q[i] -= tau w_q scal a_k[i]
// (i > k), a_q[k] -= tau w_q — the same reflectors as larfg/larf, with one
// reduction per column instead of two.  Rows stay in shared memory for the
// whole panel.  Partials are double-buffered by column parity: a CTA can only
// overwrite a buffer after every CTA has passed the barrier of the column
// that read it.
__global__ void __launch_bounds__(kQrCluThreads, 1)
qr_panel_cluster_f32_kernel(int64_t mm, int j0, int pe, int64_t rows_per_cta,
                            float* __restrict__ h, float* __restrict__ tau,
                            float* __restrict__ t_out) {
  extern __shared__ __align__(16) unsigned char qr_dyn[];
  __shared__ float p_d[2][kQrNB + 1];   // [0]: |a_k below k|^2, [1 + q]: a_kᵀ a_q
  __shared__ float p_row[2][kQrNB + 1]; // the owner's row k: [0] alpha, [1 + q] a_q[k]
  __shared__ float g_row[kQrNB + 1];
  __shared__ float g_sum[kQrNB + 1];
  __shared__ float G[kQrNB][kQrNB + 1];
  __shared__ float Tm[kQrNB][kQrNB + 1];
  cg::cluster_group cluster = cg::this_cluster();
  const int ncta = (int)cluster.num_blocks();
  const int rank = (int)cluster.block_rank();
  const int tid = threadIdx.x, warp = tid >> 5, nwarps = blockDim.x >> 5;
  const int lane = tid & 31;
  const int nb = pe - j0;
  const int64_t r_lo = j0 + (int64_t)rank * rows_per_cta;
  const int64_t r_hi = min(mm, r_lo + rows_per_cta);
  float* S = reinterpret_cast<float*>(qr_dyn);
  auto at = [&](int q, int64_t i) -> float& { return S[(int64_t)q * rows_per_cta + (i - r_lo)]; };
  for (int q = 0; q < nb; ++q)
    for (int64_t i = r_lo + tid; i < r_hi; i += blockDim.x) at(q, i) = h[(int64_t)(j0 + q) * mm + i];
  __syncthreads();
  for (int k = j0; k < pe; ++k) {
    const int par = (k - j0) & 1;
    const int kk = k - j0;
    const bool own_k = (k >= r_lo && k < r_hi);
    const int nrem = pe - k - 1;
    const int64_t i_lo = max((int64_t)k + 1, r_lo);
    // pass 1: the norm (c = 0) and the trailing dots (c = 1 + q), one warp each
    for (int c = warp; c <= nrem; c += nwarps) {
      const int qq = c == 0 ? kk : kk + c;
      int64_t i = i_lo + lane;
      float a8[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) a8[u] = 0.0f;
      for (; i + 7 * 32 < r_hi; i += 8 * 32) {
        float vv[8], qv[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) { vv[u] = at(kk, i + 32 * u); qv[u] = at(qq, i + 32 * u); }
#pragma unroll
        for (int u = 0; u < 8; ++u) a8[u] = fmaf(vv[u], qv[u], a8[u]);
      }
      for (; i < r_hi; i += 32) a8[0] = fmaf(at(kk, i), at(qq, i), a8[0]);
      float acc = ((a8[0] + a8[1]) + (a8[2] + a8[3])) + ((a8[4] + a8[5]) + (a8[6] + a8[7]));
      acc = warp_sum(acc);
      if (lane == 0) p_d[par][c] = acc;
    }
    if (own_k && tid <= nrem) p_row[par][tid] = at(kk + tid, k);
    cluster.sync();
    // thread c sums partial c over the cluster's CTAs (independent
    // distributed-shared-memory loads, the same order in every CTA, so every
    // CTA forms the same reflector) and fetches the owner's a_c[k]
    const int own = (int)(kk / rows_per_cta);
    if (tid <= nrem) {
      float acc = 0.0f;
      for (int r = 0; r < ncta; ++r) acc += cluster.map_shared_rank(&p_d[par][0], r)[tid];
      g_sum[tid] = acc;
      g_row[tid] = cluster.map_shared_rank(&p_row[par][0], own)[tid];
    }
    __syncthreads();
    const float xn2 = g_sum[0];
    const float alpha = g_row[0];
    const float xnorm = sqrtf(xn2);
    float tk = 0.0f, scal = 1.0f, beta = alpha;
    if (xnorm != 0.0f) {
      beta = -copysignf(hypotf(alpha, xnorm), alpha);
      tk = (beta - alpha) / beta;
      scal = 1.0f / (alpha - beta);
    }
    if (tk != 0.0f) {
      for (int q = warp; q < nrem; q += nwarps) {
        const float d = g_sum[1 + q];
        const float aqk = g_row[1 + q];
        const float w = fmaf(scal, d, aqk);
        const float tw = tk * w;
        const float tws = tw * scal;
        const int qq = kk + 1 + q;
        if (own_k && lane == 0) at(qq, k) = aqk - tw;
        int64_t i = i_lo + lane;
        for (; i + 7 * 32 < r_hi; i += 8 * 32) {
          float vv[8], qv[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) { vv[u] = at(kk, i + 32 * u); qv[u] = at(qq, i + 32 * u); }
#pragma unroll
          for (int u = 0; u < 8; ++u) at(qq, i + 32 * u) = fmaf(-tws, vv[u], qv[u]);
        }
        for (; i < r_hi; i += 32) at(qq, i) = fmaf(-tws, at(kk, i), at(qq, i));
      }
    }
    __syncthreads();  // every trailing column has read the unscaled a_k
    // column kk is scaled into v while the next column's pass starts: that
    // pass reads columns kk+1.. only, and g_sum / g_row are rewritten only
    // after the next cluster barrier
    if (tk != 0.0f) {
      for (int64_t i = i_lo + tid; i < r_hi; i += blockDim.x) at(kk, i) *= scal;
      if (own_k && tid == 0) at(kk, k) = beta;
    }
    if (rank == 0 && tid == 0) tau[k] = tk;
  }
  __syncthreads();  // every column's scaling is done before V is read below
  // G[q][p] = v_qᵀ v_p (q < p) over this CTA's rows, summed in CTA 0; T by
  // larft's recurrence (as in qr_panel_cluster_kernel)
  {
    __shared__ float Vc[64][kQrNB + 1];
    int pq = -1, pp = -1;
    for (int p2 = 1, t = 0; p2 < nb && pq < 0; ++p2) {
      if (tid < t + p2) { pq = tid - t; pp = p2; }
      t += p2;
    }
    float acc = 0.0f;
    for (int64_t i0 = r_lo; i0 < r_hi; i0 += 64) {
      for (int e = tid; e < 64 * kQrNB; e += blockDim.x) {
        const int q = e / 64, ii = e % 64;
        const int64_t i = i0 + ii;
        Vc[ii][q] = (q < nb && i < r_hi)
                        ? ((i < j0 + q) ? 0.0f : (i == j0 + q ? 1.0f : at(q, i)))
                        : 0.0f;
      }
      __syncthreads();
      if (pq >= 0) {
#pragma unroll 8
        for (int ii = 0; ii < 64; ++ii) acc = fmaf(Vc[ii][pq], Vc[ii][pp], acc);
      }
      __syncthreads();
    }
    if (pq >= 0) G[pq][pp] = acc;
  }
  cluster.sync();
  if (rank == 0) {
    __shared__ float Gs[kQrNB][kQrNB + 1];
    for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
      const int q = e / nb, pp2 = e % nb;
      float g = 0.0f;
      if (q < pp2)
        for (int c = 0; c < ncta; ++c) g += cluster.map_shared_rank(&G[0][0], c)[q * (kQrNB + 1) + pp2];
      Gs[q][pp2] = g;
    }
    for (int e = threadIdx.x; e < kQrNB * kQrNB; e += blockDim.x) Tm[e / kQrNB][e % kQrNB] = 0.0f;
    __syncthreads();
    if (warp == 0) {
      for (int k = 0; k < nb; ++k) {
        const float tkk = tau[j0 + k];
        float v = 0.0f;
        if (lane < k) {
          for (int q = lane; q < k; ++q) v = fmaf(Tm[lane][q], Gs[q][k], v);
          v = -tkk * v;
        }
        __syncwarp();
        if (lane < k) Tm[lane][k] = v;
        if (lane == k) Tm[k][k] = tkk;
        __syncwarp();
      }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < kQrNB * kQrNB; e += blockDim.x)
      t_out[e] = Tm[e / kQrNB][e % kQrNB];
  }
  for (int q = 0; q < nb; ++q)
    for (int64_t i = r_lo + tid; i < r_hi; i += blockDim.x) h[(int64_t)(j0 + q) * mm + i] = at(q, i);
  cluster.sync();  // CTA 0 has finished reading the others' shared memory
}

// The panel kernel a launch uses: the FP32 single-barrier variant (FUSED,
// rows in shared memory), or qr_panel_cluster_kernel<T, SM>.
template <typename T, bool SM, bool FUSED>
static const void* qr_panel_fn() {
  if constexpr (FUSED) return reinterpret_cast<const void*>(qr_panel_cluster_f32_kernel);
  return reinterpret_cast<const void*>(qr_panel_cluster_kernel<T, SM>);
}

template <typename T, bool SM, bool FUSED>
static bool qr_cluster_fits(int c, size_t smem) {
  static std::mutex mu;
  static std::map<std::pair<int, int>, bool> known;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
  std::lock_guard<std::mutex> lock(mu);
  const auto key = std::make_pair(dev, c * 1000000 + (int)(smem >> 8));
  auto it = known.find(key);
  if (it != known.end()) return it->second;
  const void* fn = qr_panel_fn<T, SM, FUSED>();
  bool ok = cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) ==
            cudaSuccess;
  if (ok && smem > 0) ok = ensure_dynamic_smem(fn, (int)smem) == cudaSuccess;
  if (ok) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)c);
    cfg.blockDim = dim3(kQrCluThreads);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)c;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int nclusters = 0;
    ok = cudaOccupancyMaxActiveClusters(&nclusters, fn, &cfg) == cudaSuccess && nclusters >= 1;
  }
  if (!ok) cudaGetLastError();
  known[key] = ok;
  return ok;
}

template <typename T, bool SM, bool FUSED>
static int launch_qr_panel_variant(int c, int64_t r, size_t smem, int64_t mm, int j0, int pe,
                                   T* h, T* tau, T* t_out, cudaStream_t st) {
  if (!qr_cluster_fits<T, SM, FUSED>(c, smem)) return -1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)c);
  cfg.blockDim = dim3(kQrCluThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)c;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaError_t e;
  if constexpr (FUSED)
    e = cudaLaunchKernelEx(&cfg, qr_panel_cluster_f32_kernel, mm, j0, pe, r, h, tau, t_out);
  else
    e = cudaLaunchKernelEx(&cfg, qr_panel_cluster_kernel<T, SM>, mm, j0, pe, r, h, tau, t_out);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
  return 0;
}

// 0 when the cluster kernel was launched, -1 when the caller must fall back.
// The panel's rows stay in shared memory when a CTA's slice fits; the FP32
// factor then takes the single-barrier panel.
template <typename T>
static int launch_qr_panel_cluster(int64_t mm, int j0, int pe, T* h, T* tau, T* t_out,
                                   cudaStream_t st) {
  // 128 rows per CTA (up to 16 CTAs): the panel's passes are bound by each
  // SM's shared-memory bandwidth (two loads and a store per FMA), so more
  // CTAs per panel finish each column sooner (m = 2048, plain factorisation:
  // 11.8 ms at 1024 rows per CTA, 9.9 at 256, 9.0 at 128)
  const int64_t rows = mm - j0;
  int c = (int)((rows + 127) / 128);
  c = c < 1 ? 1 : (c > kQrCluMax ? kQrCluMax : c);
  const int64_t r = (rows + c - 1) / c;
  const size_t slice = (size_t)kQrNB * r * sizeof(T);
  if (slice <= 160 * 1024) {
    if constexpr (std::is_same<T, float>::value) {
      if (launch_qr_panel_variant<T, true, true>(c, r, slice, mm, j0, pe, h, tau, t_out, st) == 0)
        return 0;
    }
    if (launch_qr_panel_variant<T, true, false>(c, r, slice, mm, j0, pe, h, tau, t_out, st) == 0)
      return 0;
  }
  return launch_qr_panel_variant<T, false, false>(c, r, 0, mm, j0, pe, h, tau, t_out, st);
}

// T (nb×nb, upper) of panel rows [j0, j0+nb): T[k][k] = tau_k and
// T[0:k, k] = -tau_k T[0:k, 0:k] (V[:, 0:k]ᵀ v_k).
__global__ void __launch_bounds__(512)
qr_larft_kernel(int64_t mm, int j0, int nb, const double* __restrict__ h,
                const double* __restrict__ tau, double* __restrict__ t_out) {
  __shared__ double G[kQrNB][kQrNB + 1];
  __shared__ double T[kQrNB][kQrNB + 1];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  // G[q][k] = v_qᵀ v_k for q < k (rows i >= j0 + k contribute).
  for (int pair = warp; pair < nb * nb; pair += nw) {
    const int q = pair / nb, k = pair % nb;
    if (q >= k) continue;
    const int rk = j0 + k, rq = j0 + q;
    double acc = 0.0;
    for (int64_t i = rk + lane; i < mm; i += 32)
      acc = fma(refl(h, mm, rq, i), refl(h, mm, rk, i), acc);
    acc = warp_sum(acc);
    if (lane == 0) G[q][k] = acc;
  }
  for (int e = threadIdx.x; e < kQrNB * kQrNB; e += blockDim.x) T[e / kQrNB][e % kQrNB] = 0.0;
  __syncthreads();
  if (warp == 0) {
    for (int k = 0; k < nb; ++k) {
      const double tk = tau[j0 + k];
      // lane i < k: T[i][k] = -tk * sum_{q=i}^{k-1} T[i][q] G[q][k]
      double v = 0.0;
      if (lane < k) {
        for (int q = lane; q < k; ++q) v = fma(T[lane][q], G[q][k], v);
        v = -tk * v;
      }
      __syncwarp();
      if (lane < k) T[lane][k] = v;
      if (lane == k) T[k][k] = tk;
      __syncwarp();
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < kQrNB * kQrNB; e += blockDim.x)
    t_out[e] = T[e / kQrNB][e % kQrNB];
}

// W_part[s][p][j] = sum_{i in split s} v_p[i] h[j][i] for trailing rows j.
constexpr int kWRows = 32, kWChunk = 64;
__global__ void __launch_bounds__(256)
qr_w_kernel(int64_t mm, int nn, int j0, int nb, const double* __restrict__ h,
            double* __restrict__ wpart, int64_t split_len) {
  __shared__ double Vs[kQrNB][kWChunk + 1];
  __shared__ double Hs[kWRows][kWChunk + 1];
  const int s = blockIdx.y;
  const int jbase = j0 + nb + blockIdx.x * kWRows;
  const int n2 = nn - (j0 + nb);
  const int64_t i_lo = j0 + (int64_t)s * split_len;
  const int64_t i_hi = min((int64_t)mm, i_lo + split_len);
  const int p = threadIdx.x & 31;        // reflector
  const int jg = threadIdx.x >> 5;       // 8 groups of 4 rows
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int64_t c0 = i_lo; c0 < i_hi; c0 += kWChunk) {
    for (int e = threadIdx.x; e < kQrNB * kWChunk; e += blockDim.x) {
      const int pp = e / kWChunk, cc = e % kWChunk;
      const int64_t i = c0 + cc;
      Vs[pp][cc] = (pp < nb && i < i_hi) ? refl(h, mm, j0 + pp, i) : 0.0;
    }
    for (int e = threadIdx.x; e < kWRows * kWChunk; e += blockDim.x) {
      const int jj = e / kWChunk, cc = e % kWChunk;
      const int64_t i = c0 + cc;
      const int j = jbase + jj;
      Hs[jj][cc] = (j < nn && i < i_hi) ? h[(int64_t)j * mm + i] : 0.0;
    }
    __syncthreads();
#pragma unroll 4
    for (int cc = 0; cc < kWChunk; ++cc) {
      const double v = Vs[p][cc];
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[r] = fma(v, Hs[jg * 4 + r][cc], acc[r]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int jj = blockIdx.x * kWRows + jg * 4 + r;
    if (p < nb && jj < n2) wpart[((int64_t)s * kQrNB + p) * n2 + jj] = acc[r];
  }
}

// W2[p][j] = sum_q T[q][p] * (sum_s W_part[s][q][j])   (Tᵀ W)
__global__ void qr_wt_kernel(int n2, int nb, int splits, const double* __restrict__ wpart,
                             const double* __restrict__ T, double* __restrict__ w2) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n2) return;
  double w[kQrNB];
#pragma unroll
  for (int q = 0; q < kQrNB; ++q) {
    double acc = 0.0;
    if (q < nb)
      for (int s = 0; s < splits; ++s) acc += wpart[((int64_t)s * kQrNB + q) * n2 + j];
    w[q] = acc;
  }
#pragma unroll
  for (int p = 0; p < kQrNB; ++p) {
    if (p >= nb) break;
    double acc = 0.0;
    for (int q = 0; q <= p; ++q) acc = fma(T[q * kQrNB + p], w[q], acc);
    w2[(int64_t)p * n2 + j] = acc;
  }
}

// h[j][i] -= sum_p W2[p][j] v_p[i] for trailing rows j, columns i >= j0.
constexpr int kUT = 64;
__global__ void __launch_bounds__(256)
qr_update_kernel(int64_t mm, int nn, int j0, int nb, double* __restrict__ h,
                 const double* __restrict__ w2) {
  __shared__ double Ws[kQrNB][kUT + 1];
  __shared__ double Vs[kQrNB][kUT + 1];
  const int n2 = nn - (j0 + nb);
  const int jt = blockIdx.y * kUT;            // trailing row tile
  const int64_t it = j0 + (int64_t)blockIdx.x * kUT;
  for (int e = threadIdx.x; e < kQrNB * kUT; e += blockDim.x) {
    const int p = e / kUT, c = e % kUT;
    const int jj = jt + c;
    Ws[p][c] = (p < nb && jj < n2) ? w2[(int64_t)p * n2 + jj] : 0.0;
    const int64_t i = it + c;
    Vs[p][c] = (p < nb && i < mm) ? refl(h, mm, j0 + p, i) : 0.0;
  }
  __syncthreads();
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double acc[4][4];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int jj = jt + ty + 16 * r;
      const int64_t i = it + tx + 16 * c;
      acc[r][c] = (jj < n2 && i < mm) ? h[(int64_t)(j0 + nb + jj) * mm + i] : 0.0;
    }
  for (int p = 0; p < nb; ++p) {
    double wv[4], vv[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) wv[r] = Ws[p][ty + 16 * r];
#pragma unroll
    for (int c = 0; c < 4; ++c) vv[c] = Vs[p][tx + 16 * c];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[r][c] = fma(-wv[r], vv[c], acc[r][c]);
  }
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int jj = jt + ty + 16 * r;
      const int64_t i = it + tx + 16 * c;
      if (jj < n2 && i < mm) h[(int64_t)(j0 + nb + jj) * mm + i] = acc[r][c];
    }
}

// h = Mᵀ from M (mm×nn row-major) through 32×32 shared-memory tiles.
__global__ void transpose_kernel(int64_t rows, int64_t cols, const double* __restrict__ src,
                                 double* __restrict__ dst) {
  __shared__ double tile[32][33];
  const int64_t c0 = blockIdx.x * 32LL, r0 = blockIdx.y * 32LL;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int64_t r = r0 + k, c = c0 + threadIdx.x;
    if (r < rows && c < cols) tile[k][threadIdx.x] = src[r * cols + c];
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int64_t c = c0 + k, r = r0 + threadIdx.x;
    if (r < rows && c < cols) dst[c * rows + r] = tile[threadIdx.x][k];
  }
}

__global__ void copy_kernel(int64_t n, const double* __restrict__ src, double* __restrict__ dst) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

// ormqr: partial dots part[r][chunk][p] = sum_{i in chunk} v_p[i] c_r[i].
constexpr int kOrmChunk = 2048;
__global__ void __launch_bounds__(256)
ormqr_dots_kernel(int64_t mm, int j0, int nb, const double* __restrict__ h,
                  const double* __restrict__ c, int nchunks, double* __restrict__ part) {
  __shared__ double red[8][kQrNB];
  const int r = blockIdx.y, ch = blockIdx.x;
  const double* cr = c + (int64_t)r * mm;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t lo = j0 + (int64_t)ch * kOrmChunk;
  const int64_t hi = min(mm, lo + kOrmChunk);
  double acc[kQrNB];
#pragma unroll
  for (int p = 0; p < kQrNB; ++p) acc[p] = 0.0;
  for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    const double ci = cr[i];
#pragma unroll
    for (int p = 0; p < kQrNB; ++p)
      if (p < nb) acc[p] = fma(refl(h, mm, j0 + p, i), ci, acc[p]);
  }
#pragma unroll
  for (int p = 0; p < kQrNB; ++p) {
    const double s = warp_sum(acc[p]);
    if (lane == 0) red[warp][p] = s;
  }
  __syncthreads();
  if (threadIdx.x < kQrNB) {
    double s = 0.0;
    for (int w = 0; w < 8; ++w) s += red[w][threadIdx.x];
    part[((int64_t)r * nchunks + ch) * kQrNB + threadIdx.x] = s;
  }
}

// c_r[i] -= sum_p v_p[i] w'[p], w' = op(T) (sum over chunks of part).
__global__ void __launch_bounds__(256)
ormqr_apply_kernel(int64_t mm, int j0, int nb, const double* __restrict__ h,
                   const double* __restrict__ T, int trans, double* __restrict__ c, int nchunks,
                   const double* __restrict__ part) {
  __shared__ double w[kQrNB], w2[kQrNB];
  const int r = blockIdx.y, ch = blockIdx.x;
  double* cr = c + (int64_t)r * mm;
  if (threadIdx.x < kQrNB) {
    double s = 0.0;
    for (int k = 0; k < nchunks; ++k) s += part[((int64_t)r * nchunks + k) * kQrNB + threadIdx.x];
    w[threadIdx.x] = s;
  }
  __syncthreads();
  if (threadIdx.x < kQrNB) {
    const int p = threadIdx.x;
    double s = 0.0;
    if (p < nb) {
      if (trans) {  // Qᵀ c: w' = Tᵀ w
        for (int q = 0; q <= p; ++q) s = fma(T[q * kQrNB + p], w[q], s);
      } else {      // Q c: w' = T w
        for (int q = p; q < nb; ++q) s = fma(T[p * kQrNB + q], w[q], s);
      }
    }
    w2[p] = s;
  }
  __syncthreads();
  const int64_t lo = j0 + (int64_t)ch * kOrmChunk;
  const int64_t hi = min(mm, lo + kOrmChunk);
  for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    double acc = cr[i];
    for (int p = 0; p < nb; ++p) acc = fma(-refl(h, mm, j0 + p, i), w2[p], acc);
    cr[i] = acc;
  }
}

static int64_t qr_splits(int64_t mm, int n2) {
  const int64_t jt = (n2 + kWRows - 1) / kWRows;
  int64_t s = (2LL * sm_count() + jt - 1) / (jt > 0 ? jt : 1);
  const int64_t cap = (mm + 255) / 256;
  if (s > cap) s = cap;
  if (s < 1) s = 1;
  return s;
}

}  // namespace lxgb

using namespace lxgb;

extern "C" int64_t lxgb_geqrf_t_elems(int64_t n) {
  return ((n + kQrNB - 1) / kQrNB) * (int64_t)kQrNB * kQrNB;
}

// Split geometry of the W = Vᵀ C pass of panel j0 (shared by the size query
// and the launch so both agree exactly).
static void qr_w_geometry(int64_t m, int nn, int j0, int nb, int64_t* split_len, int64_t* used) {
  const int n2 = nn - (j0 + nb);
  const int64_t span = m - j0;
  const int64_t splits = qr_splits(span, n2);
  *split_len = ((span + splits - 1) / splits + kWChunk - 1) / kWChunk * kWChunk;
  *used = (span + *split_len - 1) / *split_len;
}

extern "C" int64_t lxgb_geqrf_workspace_size(int64_t m, int64_t n) {
  if (m <= 0 || n <= 0 || n > m) return 256;
  int64_t worst = 0;
  for (int j0 = 0; j0 < n; j0 += kQrNB) {
    const int nb = (int)(n - j0 < kQrNB ? n - j0 : kQrNB);
    const int n2 = (int)n - (j0 + nb);
    if (n2 <= 0) continue;
    int64_t split_len, used;
    qr_w_geometry(m, (int)n, j0, nb, &split_len, &used);
    const int64_t need = (used + 1) * kQrNB * (int64_t)n2;
    if (need > worst) worst = need;
  }
  return 256 + worst * (int64_t)sizeof(double);
}

extern "C" int lxgb_geqrf_f64(int64_t m, int64_t n, const double* a, int32_t a_layout, double* h,
                              double* tau, double* t, void* work, int64_t work_bytes,
                              void* stream) {
  LXGB_REQUIRE(m >= 0 && n >= 0, "geqrf: negative size");
  LXGB_REQUIRE(n <= m, "geqrf: needs a tall matrix (n <= m); transpose wide ones");
  LXGB_REQUIRE(a_layout == 0 || a_layout == 1, "geqrf: a_layout must be 0 or 1");
  LXGB_REQUIRE(n < (1LL << 31), "geqrf: n too large");
  if (m == 0 || n == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(a && h && tau && t && work, "geqrf: null pointer");
  if (work_bytes < lxgb_geqrf_workspace_size(m, n)) {
    set_last_error("geqrf: workspace too small");
    return LXGB_WORKSPACE_TOO_SMALL;
  }
  cudaStream_t st = as_stream(stream);
  if (a_layout == 0) {
    dim3 grid((unsigned)((n + 31) / 32), (unsigned)((m + 31) / 32));
    transpose_kernel<<<grid, dim3(32, 8), 0, st>>>(m, n, a, h);
  } else if (a != h) {
    const int64_t cnt = m * n;
    const int64_t blocks = (cnt + 255) / 256 < 4096 ? (cnt + 255) / 256 : 4096;
    copy_kernel<<<(unsigned)blocks, 256, 0, st>>>(cnt, a, h);
  }
  const int nn = (int)n;
  double* wbase = reinterpret_cast<double*>(reinterpret_cast<char*>(work) + 256);
  for (int j0 = 0; j0 < nn; j0 += kQrNB) {
    const int nb = min(kQrNB, nn - j0);
    double* Tp = t + (int64_t)(j0 / kQrNB) * kQrNB * kQrNB;
    if (launch_qr_panel_cluster(m, j0, j0 + nb, h, tau, Tp, st) != 0) {
      qr_panel_kernel<<<1, kQrPanelThreads, 0, st>>>(m, nn, j0, j0 + nb, h, tau);
      qr_larft_kernel<<<1, 512, 0, st>>>(m, j0, nb, h, tau, Tp);
    }
    const int n2 = nn - (j0 + nb);
    if (n2 > 0) {
      int64_t split_len, used;
      qr_w_geometry(m, nn, j0, nb, &split_len, &used);
      double* wpart = wbase;
      double* w2 = wbase + used * kQrNB * (int64_t)n2;
      dim3 gw((unsigned)((n2 + kWRows - 1) / kWRows), (unsigned)used);
      qr_w_kernel<<<gw, 256, 0, st>>>(m, nn, j0, nb, h, wpart, split_len);
      qr_wt_kernel<<<(n2 + 127) / 128, 128, 0, st>>>(n2, nb, (int)used, wpart, Tp, w2);
      dim3 gu((unsigned)((m - j0 + kUT - 1) / kUT), (unsigned)((n2 + kUT - 1) / kUT));
      qr_update_kernel<<<gu, 256, 0, st>>>(m, nn, j0, nb, h, w2);
    }
  }
  return check_launch("geqrf");
}

extern "C" int64_t lxgb_ormqr_workspace_size(int64_t m, int32_t nrhs) {
  const int64_t chunks = (m + kOrmChunk - 1) / kOrmChunk;
  return 256 + (int64_t)(nrhs > 0 ? nrhs : 0) * chunks * kQrNB * (int64_t)sizeof(double);
}

extern "C" int lxgb_ormqr_f64(int64_t m, int64_t n, const double* h, const double* tau,
                              const double* t, int32_t nrhs, double* c, int32_t trans, void* work,
                              int64_t work_bytes, void* stream) {
  (void)tau;  // the panel T matrices carry the tau values
  LXGB_REQUIRE(m >= 0 && n >= 0 && n <= m && nrhs >= 0, "ormqr: bad sizes");
  LXGB_REQUIRE(trans == 0 || trans == 1, "ormqr: trans must be 0 or 1");
  if (m == 0 || n == 0 || nrhs == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(h && t && c && work, "ormqr: null pointer");
  LXGB_REQUIRE(nrhs <= 65535, "ormqr: too many vectors");
  if (work_bytes < lxgb_ormqr_workspace_size(m, nrhs)) {
    set_last_error("ormqr: workspace too small");
    return LXGB_WORKSPACE_TOO_SMALL;
  }
  cudaStream_t st = as_stream(stream);
  double* part = reinterpret_cast<double*>(reinterpret_cast<char*>(work) + 256);
  const int npan = (int)((n + kQrNB - 1) / kQrNB);
  for (int q = 0; q < npan; ++q) {
    const int pidx = trans ? q : npan - 1 - q;  // Qᵀ: H_0 first; Q: last panel first
    const int j0 = pidx * kQrNB;
    const int nb = (int)(n - j0 < kQrNB ? n - j0 : kQrNB);
    const int64_t span = m - j0;
    const int nchunks = (int)((span + kOrmChunk - 1) / kOrmChunk);
    dim3 g((unsigned)nchunks, (unsigned)nrhs);
    const double* Tp = t + (int64_t)pidx * kQrNB * kQrNB;
    ormqr_dots_kernel<<<g, 256, 0, st>>>(m, j0, nb, h, c, nchunks, part);
    ormqr_apply_kernel<<<g, 256, 0, st>>>(m, j0, nb, h, Tp, trans, c, nchunks, part);
  }
  return check_launch("ormqr");
}

namespace lxgb {

// ---------------------------------------------------------------------------
// FP32 Householder QR with the trailing updates on the tcgen05 tensor cores
// (TF32 products): the factor of the mixed-precision least-squares solver.
// Same raw layout as lxgb_geqrf_f64 (h = Mᵀ, n rows of length m, FP32), same
// 32-column panels (the cluster panel kernel in FP32, with its T), then per
// panel, with V the panel's reflectors (zeros above the diagonal, ones on it)
// and C the trailing rows of h:
//   W  = C Vᵀ        (n2 × 32; tcgen05, the K = m range split in chunks)
//   W' = W T         (fold the chunks and multiply by T on the CUDA cores)
//   C -= W' V        (tcgen05, a rank-32 update of the trailing rows)
// ---------------------------------------------------------------------------
constexpr int kQr32Split = 8;

// vrows[p][i] = v_p[i] (32 × m, row stride m) and vcols[i][p] (m × 32).
__global__ void qr32_make_v_kernel(int64_t mm, int j0, int nb, const float* __restrict__ h,
                                   float* __restrict__ vrows, float* __restrict__ vcols) {
  const int64_t total = (int64_t)kQrNB * mm;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int p = (int)(e / mm);
    const int64_t i = e % mm;
    const float v = (p < nb) ? refl(h, mm, j0 + p, i) : 0.0f;
    vrows[(int64_t)p * mm + i] = v;
    vcols[i * kQrNB + p] = v;
  }
}

// w2[j][p] = sum_q (sum_s wpart[s][j][q]) T[q][p], j < n2: one warp per row
// j, lane q sums the K-split partials of W[j][q] (coalesced), then lane p
// forms its output from W[j][·] broadcast by shuffles.
__global__ void __launch_bounds__(256)
qr32_wt_kernel(int n2, int nb, int splits, const float* __restrict__ wpart,
               const float* __restrict__ T, float* __restrict__ w2) {
  __shared__ float Ts[kQrNB][kQrNB + 1];
  for (int e = threadIdx.x; e < kQrNB * kQrNB; e += blockDim.x)
    Ts[e / kQrNB][e % kQrNB] = T[e];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int j = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (j >= n2) return;
  float w = 0.0f;
  if (lane < nb)
    for (int sp = 0; sp < splits; ++sp) w += wpart[((int64_t)sp * n2 + j) * kQrNB + lane];
  float a = 0.0f;
#pragma unroll
  for (int q = 0; q < kQrNB; ++q) a = fmaf(__shfl_sync(0xffffffffu, w, q), Ts[q][lane], a);
  w2[(int64_t)j * kQrNB + lane] = (lane < nb) ? a : 0.0f;
}

__global__ void qr32_transpose_cvt_kernel(int64_t rows, int64_t cols, const double* __restrict__ a,
                                          float* __restrict__ h) {
  __shared__ float tile[32][33];
  const int64_t r0 = (int64_t)blockIdx.y * 32, c0 = (int64_t)blockIdx.x * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int64_t r = r0 + k, c = c0 + threadIdx.x;
    tile[k][threadIdx.x] = (r < rows && c < cols) ? (float)a[r * cols + c] : 0.0f;
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const int64_t c = c0 + k, r = r0 + threadIdx.x;
    if (c < cols && r < rows) h[c * rows + r] = tile[threadIdx.x][k];
  }
}

static int64_t qr32_align(int64_t b) { return (b + 255) & ~(int64_t)255; }

// q = the m×m identity (row-major FP32), one CTA per row stride.
__global__ void set_identity_rows_kernel(int64_t m, float* __restrict__ q) {
  for (int64_t r = blockIdx.x; r < m; r += gridDim.x)
    for (int64_t c = threadIdx.x; c < m; c += blockDim.x) q[r * m + c] = (r == c) ? 1.0f : 0.0f;
}

}  // namespace lxgb

extern "C" int64_t lxgb_geqrf_f32_tc_workspace_size(int64_t m, int64_t n) {
  using namespace lxgb;
  const int64_t v = qr32_align((int64_t)kQrNB * m * 4);
  const int64_t wp = qr32_align((int64_t)kQr32Split * (n > 0 ? n : 1) * kQrNB * 4);
  const int64_t w2 = qr32_align((int64_t)(n > 0 ? n : 1) * kQrNB * 4);
  return 256 + 2 * v + wp + w2;
}

namespace lxgb {

// FP32 Householder QR with tcgen05 TF32 trailing updates.  With q != nullptr
// the reflectors are also applied to the columns of the m×m identity held as
// the rows of q (the same two GEMMs per panel, on m rows instead of the
// trailing n2), so q ends as Q in row-major order (row j = Qᵀ e_j).
static int geqrf_f32_tc_driver(int64_t m, int64_t n, const double* a, float* h, float* tau,
                               float* t, float* q, int32_t* err, void* work, int64_t work_bytes,
                               const char* who, cudaStream_t st) {
  LXGB_REQUIRE(m >= 0 && n >= 0, "geqrf_f32_tc: negative size");
  LXGB_REQUIRE(n <= m, "geqrf_f32_tc: needs a tall matrix (n <= m)");
  if (m == 0 || n == 0) return LXGB_SUCCESSFUL;
  LXGB_REQUIRE(a && h && tau && t && err && work, "geqrf_f32_tc: null pointer");
  LXGB_REQUIRE((m % 4) == 0, "geqrf_f32_tc: m must be a multiple of 4 (16-byte TMA rows)");
  LXGB_REQUIRE(m < (1LL << 31) && n < (1LL << 31), "geqrf_f32_tc: too large");
  LXGB_REQUIRE((((uintptr_t)h) & 15) == 0 && (((uintptr_t)work) & 255) == 0,
               "geqrf_f32_tc: h must be 16-byte and work 256-byte aligned");
  LXGB_REQUIRE(q == nullptr || (((uintptr_t)q) & 15) == 0, "geqrf_f32_tc: q must be 16-byte aligned");
  const int64_t rows_w = q ? m : n;  // rows a trailing update may cover
  if (work_bytes < lxgb_geqrf_f32_tc_workspace_size(m, rows_w)) {
    set_last_error("%s: workspace too small", who);
    return LXGB_WORKSPACE_TOO_SMALL;
  }
  {
    dim3 grid((unsigned)((n + 31) / 32), (unsigned)((m + 31) / 32));
    qr32_transpose_cvt_kernel<<<grid, dim3(32, 8), 0, st>>>(m, n, a, h);
  }
  if (q) {
    const unsigned g = (unsigned)(m < 65535 ? m : 65535);
    set_identity_rows_kernel<<<g, 256, 0, st>>>(m, q);
  }
  const int64_t vb = qr32_align((int64_t)kQrNB * m * 4);
  const int64_t wpb = qr32_align((int64_t)kQr32Split * rows_w * kQrNB * 4);
  char* wb = reinterpret_cast<char*>(work) + 256;
  float* vrows = reinterpret_cast<float*>(wb);
  float* vcols = reinterpret_cast<float*>(wb + vb);
  float* wpart = reinterpret_cast<float*>(wb + 2 * vb);
  float* w2 = reinterpret_cast<float*>(wb + 2 * vb + wpb);
  const int nn = (int)n;
  // C -= (C Vᵀ) T' V on the rows c[0..rows) (each a column being transformed)
  auto apply = [&](float* c, int rows, int j0, int nb, const float* Tp) -> int {
    const int64_t klen = m - j0;
    const int64_t chunk = ((klen + kQr32Split - 1) / kQr32Split + 31) / 32 * 32;
    const int used = (int)((klen + chunk - 1) / chunk);
    // W partials over `used` K ranges in one split-K launch
    int rc0 = gemm_tf32_nt_splitk(rows, nb, (int)klen, c + j0, m, vrows + j0, m, wpart, kQrNB,
                                  (int)chunk, used, err, st);
    if (rc0) return rc0;
    qr32_wt_kernel<<<(unsigned)((rows + 7) / 8), 256, 0, st>>>(rows, nb, used, wpart, Tp, w2);
    return gemm_tf32_nt(rows, (int)klen, nb, w2, kQrNB, vcols + (int64_t)j0 * kQrNB, kQrNB,
                        c + j0, m, -1.0f, 1.0f, err, st);
  };
  for (int j0 = 0; j0 < nn; j0 += kQrNB) {
    const int nb = min(kQrNB, nn - j0);
    float* Tp = t + (int64_t)(j0 / kQrNB) * kQrNB * kQrNB;
    if (launch_qr_panel_cluster<float>(m, j0, j0 + nb, h, tau, Tp, st) != 0) {
      set_last_error("%s: the panel's thread-block cluster cannot be scheduled", who);
      return LXGB_NOT_SUPPORTED;
    }
    const int n2 = nn - (j0 + nb);
    if (n2 <= 0 && !q) continue;
    const int64_t tot = (int64_t)kQrNB * m;
    qr32_make_v_kernel<<<(unsigned)((tot + 255) / 256 < 4096 ? (tot + 255) / 256 : 4096), 256, 0,
                         st>>>(m, j0, nb, h, vrows, vcols);
    if (n2 > 0) {
      int rc = apply(h + (int64_t)(j0 + nb) * m, n2, j0, nb, Tp);  // trailing rows of h
      if (rc) return rc;
    }
    if (q) {
      int rc = apply(q, (int)m, j0, nb, Tp);
      if (rc) return rc;
    }
  }
  return check_launch(who);
}

}  // namespace lxgb

extern "C" int lxgb_geqrf_f32_tc(int64_t m, int64_t n, const double* a, float* h, float* tau,
                                 float* t, int32_t* err, void* work, int64_t work_bytes,
                                 void* stream) {
  return lxgb::geqrf_f32_tc_driver(m, n, a, h, tau, t, nullptr, err, work, work_bytes,
                                   "geqrf_f32_tc", lxgb::as_stream(stream));
}

extern "C" int64_t lxgb_geqrf_f32_tc_q_workspace_size(int64_t m, int64_t n) {
  (void)n;
  return lxgb_geqrf_f32_tc_workspace_size(m, m);
}

extern "C" int lxgb_geqrf_f32_tc_q(int64_t m, int64_t n, const double* a, float* h, float* tau,
                                   float* t, float* q, int32_t* err, void* work,
                                   int64_t work_bytes, void* stream) {
  LXGB_REQUIRE(q != nullptr, "geqrf_f32_tc_q: null q");
  return lxgb::geqrf_f32_tc_driver(m, n, a, h, tau, t, q, err, work, work_bytes,
                                   "geqrf_f32_tc_q", lxgb::as_stream(stream));
}
