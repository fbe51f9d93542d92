// In-CTA upper Cholesky shared by the ragged batched kernels (chol.cu) and
// the diagonal blocks of the multi-CTA factorisation (syrk.cu).
#pragma once

#include "common.cuh"

namespace lxgb {

// Right-looking blocked upper Cholesky by the whole CTA.  a has row stride ld;
// only j >= i is read or written.  Each element receives its updates as an FMA
// chain over k ascending.  Returns 0 or k+1 for the first pivot that is not
// positive (NaN included).  Must be entered and left by all threads together.
template <typename T, int NB>
__device__ int cta_potrf_upper(T* a, int ld, int n) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nw = blockDim.x >> 5;
  for (int kb = 0; kb < n; kb += NB) {
    const int ke = min(kb + NB, n);
    for (int k = kb; k < ke; ++k) {
      const T akk = a[k * ld + k];
      if (!(akk > T(0))) return k + 1;  // uniform: every thread read the same value
      const T d = sqrt(akk);
      const T r = T(1) / d;
      for (int j = k + 1 + tid; j < n; j += blockDim.x) a[k * ld + j] *= r;
      __syncthreads();
      if (tid == 0) a[k * ld + k] = d;
      for (int i = k + 1 + warp; i < ke; i += nw) {
        const T uki = a[k * ld + i];
        for (int j = i + lane; j < n; j += 32) a[i * ld + j] = fma(-uki, a[k * ld + j], a[i * ld + j]);
      }
      __syncthreads();
    }
    // Trailing update of rows/cols [ke, n), upper triangle, 64×64 tiles.
    const int m = n - ke;
    if (m > 0) {
      const int tiles = (m + 63) >> 6;
      const int tx = tid & 15, ty = tid >> 4;
      for (int t = 0; t < tiles * tiles; ++t) {
        const int ti = t / tiles, tj = t % tiles;
        if (tj < ti) continue;
        const int i0 = ke + (ti << 6), j0 = ke + (tj << 6);
        T acc[4][4];
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            const int i = i0 + ty + 16 * r, j = j0 + tx + 16 * c;
            acc[r][c] = (i < n && j < n && j >= i) ? a[i * ld + j] : T(0);
          }
        for (int k = kb; k < ke; ++k) {
          T ui[4], uj[4];
#pragma unroll
          for (int r = 0; r < 4; ++r) {
            const int i = i0 + ty + 16 * r;
            ui[r] = (i < n) ? a[k * ld + i] : T(0);
          }
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            const int j = j0 + tx + 16 * c;
            uj[c] = (j < n) ? a[k * ld + j] : T(0);
          }
#pragma unroll
          for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int c = 0; c < 4; ++c) acc[r][c] = fma(-ui[r], uj[c], acc[r][c]);
        }
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            const int i = i0 + ty + 16 * r, j = j0 + tx + 16 * c;
            if (i < n && j < n && j >= i) a[i * ld + j] = acc[r][c];
          }
      }
      __syncthreads();
    }
  }
  return 0;
}

}  // namespace lxgb
