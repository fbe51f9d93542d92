// Blocked triangular solve of one vector by one CTA (the building block of
// getrs, potrs and trsm).  Solves op(T) x = x in place, where T is row-major
// with leading dimension ldt and op(T) = T or Tᵀ.
//
// The vector is swept in blocks of 32 rows.  For each block the CTA first
// forms the contribution of the already-solved unknowns (a GEMV over the
// solved part, coalesced along T's rows whichever op applies), then warp 0
// solves the 32×32 diagonal block by substitution with one unknown per lane.
#pragma once

#include "common.cuh"

namespace lxgb {

template <typename T>
struct TrsvSmem {
  T part[32][33];  // per-warp partial sums (trans) / row sums (no trans)
  T diag[32][33];  // the diagonal block of op(T)
};

// `x` may point to shared or global memory.  All threads of the CTA must call.
// blockDim.x must be a multiple of 32 and at most 1024.
template <typename T>
__device__ void cta_trsv(const T* __restrict__ t, int64_t ldt, int n, bool lower,
                         bool trans, bool unit, T* x, TrsvSmem<T>& sm) {
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
  const bool fwd = (lower != trans);  // op(T) is lower triangular
  const int nblk = (n + 31) >> 5;
  for (int bi = 0; bi < nblk; ++bi) {
    const int blk = fwd ? bi : nblk - 1 - bi;
    const int r0 = blk << 5;
    const int rn = min(32, n - r0);
    const int js = fwd ? 0 : r0 + rn;  // solved range [js, je)
    const int je = fwd ? r0 : n;
    // 1. contribution of solved unknowns to the rows of this block.
    if (!trans) {
      for (int ii = warp; ii < 32; ii += nw) {
        T acc = T(0);
        if (ii < rn) {
          const T* row = t + (int64_t)(r0 + ii) * ldt;
          for (int j = js + lane; j < je; j += 32) acc = fma(row[j], x[j], acc);
        }
        acc = warp_sum(acc);
        if (lane == 0) sm.part[0][ii] = acc;
      }
    } else {
      T acc = T(0);
      if (lane < rn)
        for (int j = js + warp; j < je; j += nw) acc = fma(t[(int64_t)j * ldt + r0 + lane], x[j], acc);
      sm.part[warp][lane] = acc;
    }
    // 2. the diagonal block of op(T).
    for (int e = threadIdx.x; e < 32 * 32; e += blockDim.x) {
      const int ii = e >> 5, jj = e & 31;
      T v = T(0);
      if (ii < rn && jj < rn) {
        v = trans ? t[(int64_t)(r0 + jj) * ldt + r0 + ii] : t[(int64_t)(r0 + ii) * ldt + r0 + jj];
      }
      sm.diag[ii][jj] = v;
    }
    __syncthreads();
    // 3. substitution inside the block by warp 0.
    if (warp == 0) {
      T s = T(0);
      if (!trans) {
        s = sm.part[0][lane];
      } else {
        for (int w = 0; w < nw; ++w) s += sm.part[w][lane];
      }
      T rhs = (lane < rn) ? x[r0 + lane] - s : T(0);
      for (int step = 0; step < rn; ++step) {
        const int tt = fwd ? step : rn - 1 - step;
        T xt = T(0);
        if (lane == tt) xt = unit ? rhs : rhs / sm.diag[tt][tt];
        xt = __shfl_sync(0xffffffffu, xt, tt);
        if (lane == tt) rhs = xt;
        const bool later = fwd ? (lane > tt) : (lane < tt);
        if (later && lane < rn) rhs = fma(-sm.diag[lane][tt], xt, rhs);
      }
      if (lane < rn) x[r0 + lane] = rhs;
    }
    __syncthreads();
  }
}

}  // namespace lxgb
