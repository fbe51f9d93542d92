// Device helpers shared by the Krylov solvers (CG and GMRES in krylov.cu,
// BiCGStab in bicgstab.cu): two-stage deterministic reductions over k
// right-hand sides and lineax's max-norm stopping test without division.
#pragma once

#include <math.h>

#include "common.cuh"

namespace lxgb {

constexpr int kKThreads = 256;
constexpr int kKMaxParts = 512;  // partials per vector

__device__ __forceinline__ double nanmax2(double a, double b) {
  return (a != a || b != b) ? NAN : fmax(a, b);
}

// |v| / s compared with 1 without dividing (GB300's FP64 pipe makes a
// division per element the most expensive part of a Krylov iteration):
// code 0 when the quotient is <= 1, 1 when it is > 1, 2 when it is NaN
// (v or s NaN, 0/0, inf/inf).  For finite positive s, |v| > s exactly when
// fl(|v| / s) > 1, and non-negative doubles order like their bit patterns.
// The max code over the elements, as the class 0.0 / 2.0 / NaN compared with
// 1, is the lineax test  max_norm(v / s) > 1.
__device__ __forceinline__ int ratio_code(double v, double s) {
  const long long kInf = 0x7FF0000000000000LL;
  const long long av = __double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFLL;
  const long long sb = __double_as_longlong(s);
  const long long as = sb & 0x7FFFFFFFFFFFFFFFLL;
  if (av > kInf || as > kInf) return 2;
  if (as == 0) return av == 0 ? 2 : 1;
  if (as == kInf) return av == kInf ? 2 : 0;
  if (sb < 0) return 0;  // negative finite s: the quotient is <= 0
  return av > sb ? 1 : 0;
}

// Codes 0/1/2 (integer max over elements, on the integer pipe) back to the
// classes 0.0 / 2.0 / NaN that the FP64 max-norm combination expects.
__device__ __forceinline__ double code_class(int code) {
  return code == 0 ? 0.0 : (code == 1 ? 2.0 : NAN);
}

inline int kparts(int64_t n) {
  int64_t p = (n + kKThreads * 4 - 1) / (kKThreads * 4);
  if (p < 1) p = 1;
  if (p > kKMaxParts) p = kKMaxParts;
  return (int)p;
}

// Block reduction (sum or NaN-propagating max) to thread 0.
template <bool MAX>
__device__ __forceinline__ double block_reduce(double v, double* sm) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double u = __shfl_xor_sync(0xffffffffu, v, o);
    v = MAX ? nanmax2(v, u) : v + u;
  }
  if (lane == 0) sm[warp] = v;
  __syncthreads();
  double t = sm[0];
  if (threadIdx.x == 0)
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) t = MAX ? nanmax2(t, sm[w]) : t + sm[w];
  __syncthreads();
  return t;
}

// Combine the partials of vector c in index order (one warp per vector).
__device__ __forceinline__ double combine(const double* part, int P, bool is_max) {
  const int lane = threadIdx.x & 31;
  double v = is_max ? 0.0 : 0.0;
  // lanes take a fixed interleaved subset, then a fixed shuffle tree.
  for (int i = lane; i < P; i += 32) v = is_max ? nanmax2(v, part[i]) : v + part[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double u = __shfl_xor_sync(0xffffffffu, v, o);
    v = is_max ? nanmax2(v, u) : v + u;
  }
  return v;
}

}  // namespace lxgb
